// Collocation-matrix assembly and field evaluation kernels (FP64 arithmetic).
//
// updes_assemble replaces assemble_op_Phi_P / assemble_bd_Phi_P / the P^T
// block of assemble_A (updes/assembly.py:93-362, 62-85); updes_eval_values
// evaluates vals = [Phi P] c (updes/assembly.py:404-410 read backwards).
#include "common.cuh"
#include "df.cuh"
#include "entries.cuh"
#include "rbf.cuh"
#include "stats.cuh"

namespace {

constexpr int kAsmRowsPerWarp = 8;
constexpr int kAsmWarps = 8;
constexpr int kAsmRows = kAsmRowsPerWarp * kAsmWarps;  // 64 rows per CTA
constexpr int kAsmCols = 128;                          // 32 lanes x 4 columns

template <int KIND>
__global__ void __launch_bounds__(256) assemble_kernel(updes_problem p, int n, double* __restrict__ K64,
                                                       int64_t ld64, float* __restrict__ K32, int64_t ld32,
                                                       int64_t ncols) {
  const int lane = threadIdx.x, warp = threadIdx.y;
  const int64_t c0 = int64_t(blockIdx.x) * kAsmCols + 4 * lane;
  if (c0 >= ncols) return;
  const int ip = (KIND == UPDES_RBF_POLYHARMONIC) ? 2 * int(p.rbf_param) + 1 : int(p.rbf_param);
  const double param = p.rbf_param;
  double xc[4], yc[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int64_t c = c0 + u;
    if (c < p.N) {
      xc[u] = p.nodes[2 * c];
      yc[u] = p.nodes[2 * c + 1];
    } else {
      xc[u] = yc[u] = 0.0;
    }
  }
  const int rbase = blockIdx.y * kAsmRows + warp * kAsmRowsPerWarp;
  const bool local = p.supports != nullptr;  // local supports: assemble_local_kernel writes the Phi columns
  for (int i = 0; i < kAsmRowsPerWarp; ++i) {
    const int r = rbase + i;
    if (r >= n) break;
    const RowInfo ri = load_row(p, r);
    double v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t c = c0 + u;
      if (c < p.N) v[u] = (local && ri.kind != -2) ? 0.0 : entry_rbf<KIND>(ri, int(c), xc[u], yc[u], param, ip, p.self_term);
      else if (c < n) v[u] = entry_mono(ri, int(c - p.N));
      else v[u] = 0.0;
    }
    if (K64) {
      double* dst = K64 + int64_t(r) * ld64 + c0;
      if (c0 + 3 < ncols) {
        reinterpret_cast<double2*>(dst)[0] = make_double2(v[0], v[1]);
        reinterpret_cast<double2*>(dst)[1] = make_double2(v[2], v[3]);
      } else {
        for (int u = 0; u < 4 && c0 + u < ncols; ++u) dst[u] = v[u];
      }
    }
    if (K32) {
      float* dst = K32 + int64_t(r) * ld32 + c0;
      if (c0 + 3 < ncols) {
        *reinterpret_cast<float4*>(dst) = make_float4(float(v[0]), float(v[1]), float(v[2]), float(v[3]));
      } else {
        for (int u = 0; u < 4 && c0 + u < ncols; ++u) dst[u] = float(v[u]);
      }
    }
  }
}

// Local supports (p.supports, p.support_width = S): the Phi columns of row r < N are the support of its node
// (updes/assembly.py:20-32, 125-128, 169-212), of both its nodes on a periodic row (assembly.py:215-258).
// assemble_kernel has written zeros there; one warp per row writes the support's entries.  A column in both
// supports of a periodic row is written twice with the same value.
template <int KIND>
__global__ void __launch_bounds__(256) assemble_local_kernel(updes_problem p, double* __restrict__ K64, int64_t ld64,
                                                             float* __restrict__ K32, int64_t ld32) {
  const int r = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (r >= p.N) return;
  const int ip = (KIND == UPDES_RBF_POLYHARMONIC) ? 2 * int(p.rbf_param) + 1 : int(p.rbf_param);
  const RowInfo ri = load_row(p, r);
  const int S = p.support_width;
  const bool two = ri.kind == UPDES_ROW_PERIODIC_VALUE || ri.kind == UPDES_ROW_PERIODIC_FLUX;
  for (int t = lane; t < (two ? 2 * S : S); t += 32) {
    const int node = t < S ? ri.a : ri.b;
    const int c = p.supports[int64_t(node) * S + (t < S ? t : t - S)];
    const double v = entry_rbf<KIND>(ri, c, p.nodes[2ll * c], p.nodes[2ll * c + 1], p.rbf_param, ip, p.self_term);
    if (K64) K64[int64_t(r) * ld64 + c] = v;
    if (K32) K32[int64_t(r) * ld32 + c] = float(v);
  }
}

// vals[i] = sum_{j in S(i)} phi(x_i - x_j) c_j + sum_k m_k(x_i) c_{N+k} with local supports (one warp per row).
template <int KIND>
__global__ void __launch_bounds__(256) eval_values_local_kernel(updes_problem p, const double* __restrict__ coeffs,
                                                                double* __restrict__ vals) {
  const int r = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (r >= p.N) return;
  const int ip = (KIND == UPDES_RBF_POLYHARMONIC) ? 2 * int(p.rbf_param) + 1 : int(p.rbf_param);
  const int S = p.support_width;
  const double xi = p.nodes[2ll * r], yi = p.nodes[2ll * r + 1];
  double acc = 0.0;
  for (int t = lane; t < S; t += 32) {
    const int c = p.supports[int64_t(r) * S + t];
    acc += rbf_value<KIND>(xi - p.nodes[2ll * c], yi - p.nodes[2ll * c + 1], p.rbf_param, ip) * coeffs[c];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) {
    for (int k = 0; k < p.M; ++k) acc += monomial_terms(k, xi, yi).m * coeffs[p.N + k];
    vals[r] = acc;
  }
}

// out[j] += sum over rows i whose support holds j of phi(x_i - x_j) g_i (the Phi^T g part of [Phi P]^T g with
// local supports, where Phi is not symmetric): one warp per row, FP64 atomic adds into a zeroed out[0, N),
// so the summation order, and the last bits, can differ between calls.
template <int KIND>
__global__ void __launch_bounds__(256) eval_values_local_t_kernel(updes_problem p, const double* __restrict__ g,
                                                                  double* __restrict__ out) {
  const int r = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (r >= p.N) return;
  const int ip = (KIND == UPDES_RBF_POLYHARMONIC) ? 2 * int(p.rbf_param) + 1 : int(p.rbf_param);
  const int S = p.support_width;
  const double xi = p.nodes[2ll * r], yi = p.nodes[2ll * r + 1], gi = g[r];
  for (int t = lane; t < S; t += 32) {
    const int c = p.supports[int64_t(r) * S + t];
    atomicAdd(out + c, rbf_value<KIND>(xi - p.nodes[2ll * c], yi - p.nodes[2ll * c + 1], p.rbf_param, ip) * gi);
  }
}

// coeff_grad_kernel with local supports: dW[i][k] = -lambda_i (sum_{j in S(i)} D_k(x_i, x_j) c_j + monomials).
template <int KIND>
__global__ void __launch_bounds__(256) coeff_grad_local_kernel(updes_problem p, const double* __restrict__ coeffs,
                                                               const double* __restrict__ lambda,
                                                               double* __restrict__ dW) {
  const int r = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (r >= p.Ni) return;
  const int ip = (KIND == UPDES_RBF_POLYHARMONIC) ? 2 * int(p.rbf_param) + 1 : int(p.rbf_param);
  const int S = p.support_width;
  const double xi = p.nodes[2ll * r], yi = p.nodes[2ll * r + 1];
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int t = lane; t < S; t += 32) {
    const int c = p.supports[int64_t(r) * S + t];
    const double dx = xi - p.nodes[2ll * c], dy = yi - p.nodes[2ll * c + 1];
    const double r2 = dx * dx + dy * dy, cj = coeffs[c];
    if (r2 == 0.0) { acc[0] += rbf_phi0<KIND>() * cj; continue; }
    const RbfG gg = rbf_g<KIND>(r2, p.rbf_param, ip);
    acc[0] += gg.phi * cj;
    acc[1] += gg.g1 * dx * cj;
    acc[2] += gg.g1 * dy * cj;
    acc[3] += (gg.g1 + gg.g2 * dx * dx) * cj;
    acc[4] += (gg.g1 + gg.g2 * dy * dy) * cj;
  }
  for (int k = 0; k < 5; ++k)
    for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
  if (lane == 0) {
    for (int m = 0; m < p.M; ++m) {
      const MonoT mt = monomial_terms(m, xi, yi);
      const double gm = coeffs[p.N + m];
      acc[0] += mt.m * gm; acc[1] += mt.mx * gm; acc[2] += mt.my * gm; acc[3] += mt.mxx * gm; acc[4] += mt.myy * gm;
    }
    const double l = lambda[r];
    for (int k = 0; k < 5; ++k) dW[5ll * r + k] = -l * acc[k];
  }
}

// Launch KERNEL<KIND> for the problem's kernel kind with the given grid and arguments.
#define UPDES_DISPATCH_KIND(KERNEL, GRID, BLOCK, STREAM, ...)                                                        \
  switch (p->rbf) {                                                                                               \
    case UPDES_RBF_POLYHARMONIC: KERNEL<UPDES_RBF_POLYHARMONIC><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break;   \
    case UPDES_RBF_GAUSSIAN: KERNEL<UPDES_RBF_GAUSSIAN><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break;           \
    case UPDES_RBF_MULTIQUADRIC: KERNEL<UPDES_RBF_MULTIQUADRIC><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break;   \
    case UPDES_RBF_INVERSE_MULTIQUADRIC:                                                                          \
      KERNEL<UPDES_RBF_INVERSE_MULTIQUADRIC><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break;                     \
    default: KERNEL<UPDES_RBF_THIN_PLATE><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break;                          \
  }

// vals[i] = sum_{j != i} phi(x_i - x_j) c_j + sum_k m_k(x_i) c_{N+k}
constexpr int kEvalRows = 16;     // rows per CTA (2 per warp)
constexpr int kEvalChunk = 512;   // columns staged per pass

template <int KIND, bool POLY = true>
__global__ void __launch_bounds__(256) eval_values_kernel(updes_problem p, const double* __restrict__ coeffs,
                                                          double* __restrict__ vals) {
  __shared__ double sx[kEvalChunk], sy[kEvalChunk], sc[kEvalChunk];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ip = (KIND == UPDES_RBF_POLYHARMONIC) ? 2 * int(p.rbf_param) + 1 : int(p.rbf_param);
  const int r0 = blockIdx.x * kEvalRows + warp * 2;
  double xi[2], yi[2], acc[2] = {0.0, 0.0};
  for (int u = 0; u < 2; ++u) {
    const int r = min(r0 + u, p.N - 1);
    xi[u] = p.nodes[2 * r];
    yi[u] = p.nodes[2 * r + 1];
  }
  for (int base = 0; base < p.N; base += kEvalChunk) {
    __syncthreads();
    for (int t = tid; t < kEvalChunk; t += blockDim.x) {
      const int c = base + t;
      if (c < p.N) {
        sx[t] = p.nodes[2 * c];
        sy[t] = p.nodes[2 * c + 1];
        sc[t] = coeffs[c];
      } else {
        sx[t] = sy[t] = sc[t] = 0.0;
      }
    }
    __syncthreads();
    const int lim = min(kEvalChunk, p.N - base);
    for (int t = lane; t < lim; t += 32) {
      const int c = base + t;
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        if (c == r0 + u && !p.self_term) continue;
        acc[u] += rbf_value<KIND>(xi[u] - sx[t], yi[u] - sy[t], p.rbf_param, ip) * sc[t];
      }
    }
  }
  for (int u = 0; u < 2; ++u) {
    double a = acc[u];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    acc[u] = a;
  }
  if (lane < 2) {
    const int r = r0 + lane;
    if (r < p.N) {
      double s = acc[lane];
      if (POLY)
        for (int k = 0; k < p.M; ++k) s += monomial_terms(k, xi[lane], yi[lane]).m * coeffs[p.N + k];
      vals[r] = s;
    }
  }
}

// vals = [Phi P] c with the symmetry of Phi (phi(x_i - x_j) = phi(x_j - x_i)): every kernel value of a
// 64 x 64 tile pair (I, J), I < J, serves row i of block I (phi_ij c_j) and row j of block J (phi_ij c_i),
// so half the FP64 evaluations of eval_values_kernel.  part[b * N + i] receives the sum over block b's
// columns for row i, written exactly once (by tile (I, b) when b >= I, as the column sum of tile (b, I)
// otherwise); eval_values_sym_reduce adds the blocks in order, so the result is deterministic.
constexpr int kSymT = 64;

template <int KIND>
__global__ void __launch_bounds__(256) eval_values_sym_kernel(updes_problem p, const double* __restrict__ coeffs,
                                                              double* __restrict__ part) {
  const int J = blockIdx.x, I = blockIdx.y;
  if (I > J) return;
  __shared__ double scol[16][kSymT + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int N = p.N;
  const int ip = (KIND == UPDES_RBF_POLYHARMONIC) ? 2 * int(p.rbf_param) + 1 : int(p.rbf_param);
  const int i0 = I * kSymT + ty * 4, j0 = J * kSymT + tx * 4;
  double xi[4], yi[4], ci[4], xj[4], yj[4], cj[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int i = min(i0 + u, N - 1), j = min(j0 + u, N - 1);
    xi[u] = p.nodes[2 * i];
    yi[u] = p.nodes[2 * i + 1];
    ci[u] = i0 + u < N ? coeffs[i] : 0.0;
    xj[u] = p.nodes[2 * j];
    yj[u] = p.nodes[2 * j + 1];
    cj[u] = j0 + u < N ? coeffs[j] : 0.0;
  }
  double racc[4] = {0.0, 0.0, 0.0, 0.0}, cacc[4] = {0.0, 0.0, 0.0, 0.0};
  const bool diag = (I == J);
#pragma unroll
  for (int u = 0; u < 4; ++u) {
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      if (diag && i0 + u == j0 + v && !p.self_term) continue;
      const double phi = rbf_value<KIND>(xi[u] - xj[v], yi[u] - yj[v], p.rbf_param, ip);
      racc[u] = fma(phi, cj[v], racc[u]);   // padding columns carry c = 0
      cacc[v] = fma(phi, ci[u], cacc[v]);   // padding rows carry c = 0
    }
  }
  // row sums over the tile's 64 columns: the 16 lanes of a row group (xor 1..8 stay inside the group)
#pragma unroll
  for (int u = 0; u < 4; ++u)
    for (int o = 8; o > 0; o >>= 1) racc[u] += __shfl_xor_sync(0xffffffffu, racc[u], o);
  if (tx == 0)
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (i0 + u < N) part[int64_t(J) * N + i0 + u] = racc[u];
  if (!diag) {
    // column sums over the tile's 64 rows, through shared memory (the 16 row groups span warps)
#pragma unroll
    for (int v = 0; v < 4; ++v) scol[ty][tx * 4 + v] = cacc[v];
    __syncthreads();
    if (tid < kSymT) {
      double sum = 0.0;
#pragma unroll
      for (int q = 0; q < 16; ++q) sum += scol[q][tid];
      const int j = J * kSymT + tid;
      if (j < N) part[int64_t(I) * N + j] = sum;
    }
  }
}

__global__ void eval_values_sym_reduce(updes_problem p, const double* __restrict__ part, int nblk,
                                       const double* __restrict__ coeffs, double* __restrict__ vals) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.N) return;
  double s = 0.0;
  for (int b = 0; b < nblk; ++b) s += part[int64_t(b) * p.N + i];
  const double x = p.nodes[2 * i], y = p.nodes[2 * i + 1];
  for (int k = 0; k < p.M; ++k) s += monomial_terms(k, x, y).m * coeffs[p.N + k];
  vals[i] = s;
}

// Field at arbitrary points from coefficients, summing over every center
// (updes/operators.py:118-184 value / gradient, :319-348 laplacian).
// what: 0 value (out m), 1 gradient (out m x 2), 2 laplacian (out m).
template <int KIND>
__global__ void __launch_bounds__(256) eval_field_kernel(int m, const double* __restrict__ pts, int N,
                                                         const double* __restrict__ ctr, int M, double param,
                                                         const double* __restrict__ coeffs, int what,
                                                         double* __restrict__ out) {
  __shared__ double sx[kEvalChunk], sy[kEvalChunk], sc[kEvalChunk];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ip = (KIND == UPDES_RBF_POLYHARMONIC) ? 2 * int(param) + 1 : int(param);
  const int r0 = blockIdx.x * kEvalRows + warp * 2;
  double xi[2], yi[2], a0[2] = {0.0, 0.0}, a1[2] = {0.0, 0.0};
  for (int u = 0; u < 2; ++u) {
    const int r = min(r0 + u, m - 1);
    xi[u] = pts[2 * r];
    yi[u] = pts[2 * r + 1];
  }
  for (int base = 0; base < N; base += kEvalChunk) {
    __syncthreads();
    for (int t = tid; t < kEvalChunk; t += blockDim.x) {
      const int c = base + t;
      if (c < N) { sx[t] = ctr[2 * c]; sy[t] = ctr[2 * c + 1]; sc[t] = coeffs[c]; }
      else { sx[t] = sy[t] = sc[t] = 0.0; }
    }
    __syncthreads();
    const int lim = min(kEvalChunk, N - base);
    for (int t = lane; t < lim; t += 32) {
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const double dx = xi[u] - sx[t], dy = yi[u] - sy[t];
        if (what == 0) {
          a0[u] += rbf_value<KIND>(dx, dy, param, ip) * sc[t];
        } else {
          const double r2 = dx * dx + dy * dy;
          if (r2 == 0.0) continue;
          const RbfG g = rbf_g<KIND>(r2, param, ip);
          if (what == 1) { a0[u] += g.g1 * dx * sc[t]; a1[u] += g.g1 * dy * sc[t]; }
          else a0[u] += (2.0 * g.g1 + g.g2 * r2) * sc[t];
        }
      }
    }
  }
  for (int u = 0; u < 2; ++u)
    for (int o = 16; o > 0; o >>= 1) {
      a0[u] += __shfl_xor_sync(0xffffffffu, a0[u], o);
      a1[u] += __shfl_xor_sync(0xffffffffu, a1[u], o);
    }
  if (lane < 2) {
    const int r = r0 + lane;
    if (r < m) {
      double v0 = a0[lane], v1 = a1[lane];
      for (int k = 0; k < M; ++k) {
        const MonoT mt = monomial_terms(k, xi[lane], yi[lane]);
        const double gk = coeffs[N + k];
        if (what == 0) v0 += gk * mt.m;
        else if (what == 1) { v0 += gk * mt.mx; v1 += gk * mt.my; }
        else v0 += gk * (mt.mxx + mt.myy);
      }
      if (what == 1) { out[2 * r] = v0; out[2 * r + 1] = v1; }
      else out[r] = v0;
    }
  }
}

// dW[i][k] = -lambda_i * sum_j D_k(x_i, x_j) c_j (+ monomial columns) for interior rows i, where D_k is the
// k-th operator primitive (value, d/dx, d/dy, d2/dx2, d2/dy2) and j != i unless self_term: the derivative
// of lambda^T K c with respect to the operator weights of row i, the entries regenerated on the fly.
template <int KIND>
__global__ void __launch_bounds__(256) coeff_grad_kernel(updes_problem p, const double* __restrict__ coeffs,
                                                         const double* __restrict__ lambda,
                                                         double* __restrict__ dW) {
  __shared__ double sx[kEvalChunk], sy[kEvalChunk], sc[kEvalChunk];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ip = (KIND == UPDES_RBF_POLYHARMONIC) ? 2 * int(p.rbf_param) + 1 : int(p.rbf_param);
  const int r0 = blockIdx.x * kEvalRows + warp * 2;
  double xi[2], yi[2], acc[2][5] = {};
  for (int u = 0; u < 2; ++u) {
    const int r = min(r0 + u, max(p.Ni - 1, 0));
    xi[u] = p.nodes[2 * r];
    yi[u] = p.nodes[2 * r + 1];
  }
  for (int base = 0; base < p.N; base += kEvalChunk) {
    __syncthreads();
    for (int t = tid; t < kEvalChunk; t += blockDim.x) {
      const int c = base + t;
      if (c < p.N) { sx[t] = p.nodes[2 * c]; sy[t] = p.nodes[2 * c + 1]; sc[t] = coeffs[c]; }
      else { sx[t] = sy[t] = sc[t] = 0.0; }
    }
    __syncthreads();
    const int lim = min(kEvalChunk, p.N - base);
    for (int t = lane; t < lim; t += 32) {
      const int c = base + t;
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        if (c == r0 + u && !p.self_term) continue;
        const double dx = xi[u] - sx[t], dy = yi[u] - sy[t];
        const double r2 = dx * dx + dy * dy;
        const double cj = sc[t];
        if (r2 == 0.0) { acc[u][0] += rbf_phi0<KIND>() * cj; continue; }
        const RbfG g = rbf_g<KIND>(r2, p.rbf_param, ip);
        acc[u][0] += g.phi * cj;
        acc[u][1] += g.g1 * dx * cj;
        acc[u][2] += g.g1 * dy * cj;
        acc[u][3] += (g.g1 + g.g2 * dx * dx) * cj;
        acc[u][4] += (g.g1 + g.g2 * dy * dy) * cj;
      }
    }
  }
  for (int u = 0; u < 2; ++u)
    for (int k = 0; k < 5; ++k)
      for (int o = 16; o > 0; o >>= 1) acc[u][k] += __shfl_xor_sync(0xffffffffu, acc[u][k], o);
  if (lane < 2) {
    const int r = r0 + lane;
    if (r < p.Ni) {
      double v[5];
      for (int k = 0; k < 5; ++k) v[k] = acc[lane][k];
      for (int m = 0; m < p.M; ++m) {
        const MonoT mt = monomial_terms(m, xi[lane], yi[lane]);
        const double gm = coeffs[p.N + m];
        v[0] += mt.m * gm; v[1] += mt.mx * gm; v[2] += mt.my * gm; v[3] += mt.mxx * gm; v[4] += mt.myy * gm;
      }
      const double l = lambda[r];
      for (int k = 0; k < 5; ++k) dW[5 * r + k] = -l * v[k];
    }
  }
}

// out[N + k] = sum_i m_k(x_i) g_i  (the P^T part of A^T g)
__global__ void pt_matvec_kernel(updes_problem p, const double* __restrict__ g, double* __restrict__ out) {
  __shared__ double red[15][32];
  double acc[15] = {};
  for (int i = threadIdx.x; i < p.N; i += blockDim.x) {
    const double gi = g[i];
    for (int k = 0; k < p.M; ++k) acc[k] += monomial_terms(k, p.nodes[2 * i], p.nodes[2 * i + 1]).m * gi;
  }
  for (int k = 0; k < p.M; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < p.M) {
    double v = 0.0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) v += red[threadIdx.x][w];
    out[p.N + threadIdx.x] = v;
  }
}

// vals[i][c] = sum_{j != i} phi(x_i - x_j) C[j][c] + sum_k m_k(x_i) C[N+k][c] for R <= 64 columns: phi is
// evaluated once per pair in FP64 and applied to every column in double-float (FP32 ALU).
constexpr int kEvBRows = 16;
template <int KIND>
__global__ void __launch_bounds__(256) eval_values_batch_kernel(updes_problem p, int R, const double* __restrict__ C,
                                                                int64_t ldc, double* __restrict__ vals, int64_t ldv) {
  __shared__ double sx[64], sy[64];
  __shared__ float sch[64][65], scl[64][65];
  __shared__ float sph[kEvBRows][65], spl[kEvBRows][65];
  const int tid = threadIdx.x;
  const int ip = (KIND == UPDES_RBF_POLYHARMONIC) ? 2 * int(p.rbf_param) + 1 : int(p.rbf_param);
  const int r0 = blockIdx.x * kEvBRows;
  // thread owns row tid / 16 and columns (tid % 16) * 4 + {0..3}
  const int ty = tid >> 4, tx = tid & 15;
  float ah[1][4] = {}, al[1][4] = {};
  for (int j0 = 0; j0 < p.N; j0 += 64) {
    __syncthreads();
    for (int e = tid; e < 64; e += blockDim.x) {
      const int j = j0 + e;
      sx[e] = j < p.N ? p.nodes[2 * j] : 0.0;
      sy[e] = j < p.N ? p.nodes[2 * j + 1] : 0.0;
    }
    for (int e = tid; e < 64 * 64; e += blockDim.x) {
      const int jj = e >> 6, c = e & 63;
      const double v = (j0 + jj < p.N && c < R) ? C[int64_t(j0 + jj) * ldc + c] : 0.0;
      const float h = float(v);
      sch[jj][c] = h;
      scl[jj][c] = float(v - double(h));
    }
    __syncthreads();
    for (int e = tid; e < kEvBRows * 64; e += blockDim.x) {
      const int ii = e >> 6, jj = e & 63;
      const int i = r0 + ii, j = j0 + jj;
      double v = 0.0;
      if (i < p.N && j < p.N && (j != i || p.self_term)) {
        const double xi = p.nodes[2 * i], yi = p.nodes[2 * i + 1];
        v = rbf_value<KIND>(xi - sx[jj], yi - sy[jj], p.rbf_param, ip);
      }
      const float h = float(v);
      sph[ii][jj] = h;
      spl[ii][jj] = float(v - double(h));
    }
    __syncthreads();
    for (int jj = 0; jj < 64; ++jj) {
#pragma unroll
      for (int u = 0; u < 1; ++u) {
        const float a = sph[ty + u][jj], a2 = spl[ty + u][jj];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          const int c = tx * 4 + v;
          const float b = sch[jj][c], b2 = scl[jj][c];
          // (ah, al) += (a + a2)(b + b2) in double-float, renormalised after every term
          const float pr = __fmul_rn(a, b);
          const float er = __fmaf_rn(a, b, -pr);
          const float s = __fadd_rn(ah[u][v], pr);
          const float bb = __fsub_rn(s, ah[u][v]);
          float t = __fadd_rn(__fsub_rn(ah[u][v], __fsub_rn(s, bb)), __fsub_rn(pr, bb));
          t = __fadd_rn(t, __fadd_rn(al[u][v], __fmaf_rn(a, b2, __fmaf_rn(a2, b, er))));
          ah[u][v] = __fadd_rn(s, t);
          al[u][v] = __fsub_rn(t, __fsub_rn(ah[u][v], s));
        }
      }
    }
  }
#pragma unroll
  for (int u = 0; u < 1; ++u) {
    const int i = r0 + ty + u;
    if (i >= p.N) continue;
    const double xi = p.nodes[2 * i], yi = p.nodes[2 * i + 1];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int c = tx * 4 + v;
      if (c >= R) continue;
      double s = double(ah[u][v]) + double(al[u][v]);
      for (int k = 0; k < p.M; ++k) s += monomial_terms(k, xi, yi).m * C[int64_t(p.N + k) * ldc + c];
      vals[int64_t(i) * ldv + c] = s;
    }
  }
}

// ---------------------------------------------------------------------------
// Double-float assembly of polyharmonic systems (the mixed-precision solve's K)
// ---------------------------------------------------------------------------
// GB300 runs FP64 at 1/64 of its FP32 rate, and the FP64 entries of an r^k kernel (square root, powers and
// the operator's combination, ~30 FP64 operations each) bind assemble_kernel to the FP64 pipe.  The mixed
// solve keeps K as two FP32 planes (48 significant bits) anyway, so here the entries are evaluated in
// double-float arithmetic on the FP32 pipes:
//  - node coordinates as exact triple-float expansions, so that x_i - x_j is formed exactly and rounded
//    once to double-float;
//  - for a row with operator weights w (value, d/dx, d/dy, d2/dx2, d2/dy2) and k = 2a+1,
//        K_ij = r^(k-2) (A0 r^2 + A1 dx + A2 dy + A3 + (A4 dx^2 + A5 dy^2) / r^2)
//    with A = (w0, k w1, k w2, k (w3 + w4), k (k-2) w3, k (k-2) w4) for interior rows (A3 + A4, 0, 0 in the
//    last three when w3 = w4, since the last term is then A4 exactly; the closed forms
//    phi = r^k, g1 = k r^(k-2), g2 = k (k-2) r^(k-4) of rbf_g), A = (1, 0, 0, 0, 0, 0) for Dirichlet,
//    (0, k n1x, k n1y, 0, 0, 0) for Neumann and (beta, k n1x, k n1y, 0, 0, 0) for Robin rows; the entry is
//    0 at r = 0 as in the FP64 kernel (phi(0) = 0, derivatives 0 there);
//  - monomial columns, P^T rows and periodic rows (a few per system) in FP64 through entry_rbf/entry_mono.
// The planes are written unscaled, with the row maxima of |hi|; the equilibration follows in the caller.

constexpr float kDfTiny = 7.88860905e-31f;  // 2^-100: below it an entry's low word would leave the normal range

struct __align__(16) DfRow {
  int kind, a, pad0, pad1;  // row kind (-1 interior, UPDES_ROW_*), evaluation node
  float c[12];              // A0..A5 as double-float pairs
};

// Node j's coordinates as exact triple-float expansions: tri[6j + 3d + t], d = x or y, t = 0..2.
__device__ __forceinline__ void tri_expand(const updes_problem& p, int j, float* __restrict__ tri) {
  for (int d = 0; d < 2; ++d) {
    const double x = p.nodes[2ll * j + d];
    const float x0 = __double2float_rn(x);
    const double r1 = x - double(x0);
    const float x1 = __double2float_rn(r1);
    tri[6ll * j + 3 * d] = x0;
    tri[6ll * j + 3 * d + 1] = x1;
    tri[6ll * j + 3 * d + 2] = __double2float_rn(r1 - double(x1));
  }
}

__global__ void tri_coords_kernel(updes_problem p, float* __restrict__ tri) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < p.N) tri_expand(p, j, tri);
}

__global__ void assemble_df_setup_kernel(updes_problem p, DfRow* __restrict__ rows, float* __restrict__ tri) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p.N) return;
  tri_expand(p, j, tri);
  const RowInfo ri = load_row(p, j);
  const double k = 2.0 * p.rbf_param + 1.0;
  double A[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (ri.kind == -1) {
    A[0] = ri.w0; A[1] = k * ri.w1; A[2] = k * ri.w2; A[3] = k * (ri.w3 + ri.w4);
    A[4] = k * (k - 2.0) * ri.w3; A[5] = k * (k - 2.0) * ri.w4;
    // an isotropic second-order part (A4 = A5, e.g. the Laplacian): (A4 dx^2 + A5 dy^2) / r^2 = A4 exactly,
    // folded into the constant so that the entry needs no division
    if (A[4] == A[5]) {
      A[3] += A[4];
      A[4] = A[5] = 0.0;
    }
  } else if (ri.kind == UPDES_ROW_DIRICHLET) {
    A[0] = 1.0;
  } else if (ri.kind == UPDES_ROW_NEUMANN || ri.kind == UPDES_ROW_ROBIN) {
    A[0] = ri.kind == UPDES_ROW_ROBIN ? ri.beta : 0.0;
    A[1] = k * ri.n1x; A[2] = k * ri.n1y;
  }
  DfRow o;
  o.kind = ri.kind;
  o.a = ri.a;
  o.pad0 = o.pad1 = 0;
  for (int t = 0; t < 6; ++t) {
    const F2 v = df_from_double(A[t]);
    o.c[2 * t] = v.h;
    o.c[2 * t + 1] = v.l;
  }
  rows[j] = o;
}

__global__ void __launch_bounds__(256) assemble_df_kernel(updes_problem p, int n, const DfRow* __restrict__ rows,
                                                          const float* __restrict__ tri, float* __restrict__ Khi,
                                                          float* __restrict__ Klo, int64_t ld,
                                                          unsigned* __restrict__ rowmax, int* __restrict__ range_flag) {
  const int lane = threadIdx.x, warp = threadIdx.y;
  const int64_t c0 = int64_t(blockIdx.x) * kAsmCols + 4 * lane;
  const bool live = c0 < ld;  // every lane stays for the row-maximum shuffles
  const int apow = int(p.rbf_param);  // r^(k-2) = r * (r^2)^(a-1)
  const int ip = 2 * apow + 1;
  float cx[4][3], cy[4][3];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int64_t c = c0 + u;
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      cx[u][t] = c < p.N ? tri[6 * c + t] : 0.f;
      cy[u][t] = c < p.N ? tri[6 * c + 3 + t] : 0.f;
    }
  }
  bool bad = false;
  const int rbase = blockIdx.y * kAsmRows + warp * kAsmRowsPerWarp;
  for (int i = 0; i < kAsmRowsPerWarp; ++i) {
    const int r = rbase + i;
    if (r >= n) break;
    float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
    const int kind = r < p.N ? rows[r].kind : -2;
    if (live && kind >= -1 && kind <= UPDES_ROW_ROBIN) {
      const DfRow& R = rows[r];
      const F2 A0{R.c[0], R.c[1]}, A1{R.c[2], R.c[3]}, A2{R.c[4], R.c[5]};
      const F2 A3{R.c[6], R.c[7]}, A4{R.c[8], R.c[9]}, A5{R.c[10], R.c[11]};
      const int a = R.a;
      const float ax0 = tri[6ll * a], ax1 = tri[6ll * a + 1], ax2 = tri[6ll * a + 2];
      const float ay0 = tri[6ll * a + 3], ay1 = tri[6ll * a + 4], ay2 = tri[6ll * a + 5];
      const bool interior = kind == -1;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t c = c0 + u;
        if (c < p.N) {
          const F2 dx = diff3(ax0, ax1, ax2, cx[u][0], cx[u][1], cx[u][2]);
          const F2 dy = diff3(ay0, ay1, ay2, cy[u][0], cy[u][1], cy[u][2]);
          if (dx.h == 0.f && dy.h == 0.f) continue;  // r = 0: the entry is 0
          const F2 dx2 = df_sqr(dx), dy2 = df_sqr(dy);
          const F2 r2 = df_add(dx2, dy2);
          F2 rk2 = df_sqrt(r2);
          for (int t = 1; t < apow; ++t) rk2 = df_mul(rk2, r2);
          F2 br{0.f, 0.f};
          if (A0.h != 0.f) br = df_mul(A0, r2);
          if (A1.h != 0.f) br = df_add(br, df_mul(A1, dx));
          if (A2.h != 0.f) br = df_add(br, df_mul(A2, dy));
          if (interior) {
            br = df_add(br, A3);
            if (A4.h != 0.f || A5.h != 0.f) br = df_add(br, df_div(df_add(df_mul(A4, dx2), df_mul(A5, dy2)), r2));
          }
          const F2 v = df_mul(rk2, br);
          hi[u] = v.h;
          lo[u] = v.l;
        } else if (c < n) {
          const RowInfo ri = load_row(p, r);
          const F2 v = df_from_double(entry_mono(ri, int(c - p.N)));
          hi[u] = v.h;
          lo[u] = v.l;
        }
      }
    } else if (live) {  // P^T and periodic rows in FP64
      const RowInfo ri = load_row(p, r);
      const double param = p.rbf_param;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t c = c0 + u;
        double v = 0.0;
        if (c < p.N) v = entry_rbf<UPDES_RBF_POLYHARMONIC>(ri, int(c), p.nodes[2 * c], p.nodes[2 * c + 1], param, ip,
                                                           p.self_term);
        else if (c < n) v = entry_mono(ri, int(c - p.N));
        const F2 f = df_from_double(v);
        hi[u] = f.h;
        lo[u] = f.l;
      }
    }
    float m = 0.f;
    if (live) {
      float* dh = Khi + int64_t(r) * ld + c0;
      float* dl = Klo + int64_t(r) * ld + c0;
      if (c0 + 3 < ld) {
        *reinterpret_cast<float4*>(dh) = make_float4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<float4*>(dl) = make_float4(lo[0], lo[1], lo[2], lo[3]);
      } else {
        for (int u = 0; u < 4 && c0 + u < ld; ++u) {
          dh[u] = hi[u];
          dl[u] = lo[u];
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float ah = fabsf(hi[u]);
        m = fmaxf(m, ah);
        bad |= !(ah <= 3.0e38f) || (ah != 0.f && ah < kDfTiny);
      }
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0 && m > 0.f && rowmax) atomicMax(rowmax + r, __float_as_uint(m));
  }
  if (bad && range_flag) atomicExch(range_flag, 1);
}

int check_problem(const updes_problem* p) {
  if (!p || p->N <= 0 || p->Ni < 0 || p->Ni > p->N) return UPDES_ERR_INVALID;
  if (!(p->M == 1 || p->M == 3 || p->M == 6 || p->M == 10 || p->M == 15)) return UPDES_ERR_INVALID;
  if (p->rbf < 0 || p->rbf > UPDES_RBF_THIN_PLATE) return UPDES_ERR_INVALID;
  if ((p->rbf == UPDES_RBF_POLYHARMONIC || p->rbf == UPDES_RBF_THIN_PLATE) &&
      (p->rbf_param < 1.0 || p->rbf_param > 8.0 || p->rbf_param != double(int(p->rbf_param))))
    return UPDES_ERR_INVALID;
  if (!p->nodes) return UPDES_ERR_INVALID;
  if (p->Ni > 0 && !p->op_weights) return UPDES_ERR_INVALID;
  if (p->N > p->Ni && (!p->bd_kind || !p->bd_node || !p->bd_geom)) return UPDES_ERR_INVALID;
  if (p->support_width < 0 || p->support_width >= p->N || (p->support_width > 0) != (p->supports != nullptr))
    return UPDES_ERR_INVALID;
  return UPDES_OK;
}

}  // namespace

int updes_check_problem(const updes_problem* p) { return check_problem(p); }

extern "C" int updes_assemble(const updes_problem* p, double* K64, int64_t ld64, float* K32, int64_t ld32,
                              void* stream) {
  int st = check_problem(p);
  if (st) return st;
  const int n = p->N + p->M;
  if (!K64 && !K32) return UPDES_ERR_INVALID;
  if ((K64 && (ld64 < n || ld64 % 2)) || (K32 && (ld32 < n || ld32 % 4))) return UPDES_ERR_INVALID;
  if ((K64 && (reinterpret_cast<uintptr_t>(K64) & 15)) || (K32 && (reinterpret_cast<uintptr_t>(K32) & 15)))
    return UPDES_ERR_INVALID;
  const int64_t ncols = K64 ? (K32 ? (ld64 < ld32 ? ld64 : ld32) : ld64) : ld32;
  dim3 block(32, kAsmWarps);
  dim3 grid(unsigned(ceil_div(ncols, kAsmCols)), unsigned(ceil_div(n, kAsmRows)));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  StatScope sc(kStatAssemble, s, 0.0, double(n) * ncols * ((K64 ? 8.0 : 0.0) + (K32 ? 4.0 : 0.0)));
  switch (p->rbf) {
    case UPDES_RBF_POLYHARMONIC:
      assemble_kernel<UPDES_RBF_POLYHARMONIC><<<grid, block, 0, s>>>(*p, n, K64, ld64, K32, ld32, ncols); break;
    case UPDES_RBF_GAUSSIAN:
      assemble_kernel<UPDES_RBF_GAUSSIAN><<<grid, block, 0, s>>>(*p, n, K64, ld64, K32, ld32, ncols); break;
    case UPDES_RBF_MULTIQUADRIC:
      assemble_kernel<UPDES_RBF_MULTIQUADRIC><<<grid, block, 0, s>>>(*p, n, K64, ld64, K32, ld32, ncols); break;
    case UPDES_RBF_INVERSE_MULTIQUADRIC:
      assemble_kernel<UPDES_RBF_INVERSE_MULTIQUADRIC><<<grid, block, 0, s>>>(*p, n, K64, ld64, K32, ld32, ncols); break;
    default:
      assemble_kernel<UPDES_RBF_THIN_PLATE><<<grid, block, 0, s>>>(*p, n, K64, ld64, K32, ld32, ncols); break;
  }
  UPDES_LAUNCH_CHECK();
  if (p->supports) {
    const unsigned g = unsigned(ceil_div(int64_t(p->N) * 32, 256));
    UPDES_DISPATCH_KIND(assemble_local_kernel, g, 256, s, *p, K64, ld64, K32, ld32);
    UPDES_LAUNCH_CHECK();
  }
  return UPDES_OK;
}

extern "C" int updes_assemble_df_scratch(const updes_problem* p, size_t* bytes) {
  if (check_problem(p) || !bytes) return UPDES_ERR_INVALID;
  *bytes = ((size_t(p->N) * sizeof(DfRow) + 255) & ~size_t(255)) + size_t(p->N) * 6 * sizeof(float) + 256;
  return UPDES_OK;
}

extern "C" int updes_assemble_df(const updes_problem* p, float* Khi, float* Klo, int64_t ld, uint32_t* rowmax,
                                 int32_t* range_flag, void* scratch, size_t scratch_bytes, void* stream) {
  int st = check_problem(p);
  if (st) return st;
  if (p->rbf != UPDES_RBF_POLYHARMONIC || p->supports) return UPDES_ERR_UNSUPPORTED;
  const int n = p->N + p->M;
  if (!Khi || !Klo || ld < n || ld % 4 || !scratch) return UPDES_ERR_INVALID;
  if (((reinterpret_cast<uintptr_t>(Khi) | reinterpret_cast<uintptr_t>(Klo) | reinterpret_cast<uintptr_t>(scratch)) &
       15) != 0)
    return UPDES_ERR_INVALID;
  size_t need = 0;
  updes_assemble_df_scratch(p, &need);
  if (scratch_bytes < need) return UPDES_ERR_WORKSPACE;
  DfRow* rows = static_cast<DfRow*>(scratch);
  float* tri = reinterpret_cast<float*>(static_cast<char*>(scratch) +
                                        ((size_t(p->N) * sizeof(DfRow) + 255) & ~size_t(255)));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  StatScope sc(kStatAssemble, s, 0.0, double(n) * ld * 8.0);
  assemble_df_setup_kernel<<<unsigned(ceil_div(p->N, 256)), 256, 0, s>>>(*p, rows, tri);
  UPDES_LAUNCH_CHECK();
  dim3 block(32, kAsmWarps);
  dim3 grid(unsigned(ceil_div(ld, kAsmCols)), unsigned(ceil_div(n, kAsmRows)));
  assemble_df_kernel<<<grid, block, 0, s>>>(*p, n, rows, tri, Khi, Klo, ld, rowmax, range_flag);
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

// eval_values_sym_kernel for polyharmonic kernels (phi = r^(2a+1)) in double-float arithmetic on the FP32
// pipes, for the mixed-precision solve: x_i - x_j exactly from the triple-float coordinates and rounded
// once to double-float, phi = r (r^2)^a, the products with the coefficients (rounded to double-float) and
// the 16-term partial sums of a thread in double-float (relative error a few units of 2^-48), the tile's
// row and column sums in FP64 as in the FP64 kernel.  r = 0 gives phi = 0, as phi(0) = 0.
__global__ void __launch_bounds__(256) eval_values_sym_df_kernel(updes_problem p, const double* __restrict__ coeffs,
                                                                 const float* __restrict__ tri,
                                                                 double* __restrict__ part) {
  const int J = blockIdx.x, I = blockIdx.y;
  if (I > J) return;
  __shared__ double scol[16][kSymT + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int N = p.N;
  const int apow = int(p.rbf_param);
  const int i0 = I * kSymT + ty * 4, j0 = J * kSymT + tx * 4;
  float xi[4][3], yi[4][3], xj[4][3], yj[4][3];
  F2 ci[4], cj[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int i = min(i0 + u, N - 1), j = min(j0 + u, N - 1);
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      xi[u][t] = tri[6ll * i + t];
      yi[u][t] = tri[6ll * i + 3 + t];
      xj[u][t] = tri[6ll * j + t];
      yj[u][t] = tri[6ll * j + 3 + t];
    }
    ci[u] = df_from_double(i0 + u < N ? coeffs[i] : 0.0);  // padding rows and columns carry c = 0
    cj[u] = df_from_double(j0 + u < N ? coeffs[j] : 0.0);
  }
  F2 racc[4], cacc[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) racc[u] = cacc[u] = F2{0.f, 0.f};
  const bool diag = (I == J);
#pragma unroll
  for (int u = 0; u < 4; ++u) {
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      if (diag && i0 + u == j0 + v && !p.self_term) continue;
      const F2 dx = diff3(xi[u][0], xi[u][1], xi[u][2], xj[v][0], xj[v][1], xj[v][2]);
      const F2 dy = diff3(yi[u][0], yi[u][1], yi[u][2], yj[v][0], yj[v][1], yj[v][2]);
      if (dx.h == 0.f && dy.h == 0.f) continue;
      const F2 r2 = df_add(df_sqr(dx), df_sqr(dy));
      F2 phi = df_sqrt(r2);
      for (int t = 0; t < apow; ++t) phi = df_mul(phi, r2);
      racc[u] = df_add(racc[u], df_mul(phi, cj[v]));
      cacc[v] = df_add(cacc[v], df_mul(phi, ci[u]));
    }
  }
  double rs[4], cs[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    rs[u] = double(racc[u].h) + double(racc[u].l);
    cs[u] = double(cacc[u].h) + double(cacc[u].l);
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
    for (int o = 8; o > 0; o >>= 1) rs[u] += __shfl_xor_sync(0xffffffffu, rs[u], o);
  if (tx == 0)
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (i0 + u < N) part[int64_t(J) * N + i0 + u] = rs[u];
  if (!diag) {
#pragma unroll
    for (int v = 0; v < 4; ++v) scol[ty][tx * 4 + v] = cs[v];
    __syncthreads();
    if (tid < kSymT) {
      double sum = 0.0;
#pragma unroll
      for (int q = 0; q < 16; ++q) sum += scol[q][tid];
      const int j = J * kSymT + tid;
      if (j < N) part[int64_t(I) * N + j] = sum;
    }
  }
}

size_t eval_values_sym_bytes(int N) {
  // per-tile partial sums, then the triple-float coordinates of the double-float kernel
  return size_t(ceil_div(N, kSymT)) * size_t(N) * sizeof(double) + ((size_t(N) * 6 * sizeof(float) + 255) & ~size_t(255));
}

// updes_eval_values through the symmetric kernel, with a scratch of eval_values_sym_bytes(N) bytes; df
// selects the double-float kernel for polyharmonic systems (the other kernels stay in FP64).
int eval_values_sym(const updes_problem* p, const double* coeffs, double* vals, double* part, cudaStream_t s,
                    bool df) {
  int st = check_problem(p);
  if (st) return st;
  if (!coeffs || !vals || !part) return UPDES_ERR_INVALID;
  if (p->supports) {  // local supports: Phi is sparse and not symmetric
    UPDES_DISPATCH_KIND(eval_values_local_kernel, unsigned(ceil_div(int64_t(p->N) * 32, 256)), 256, s, *p, coeffs,
                        vals);
    UPDES_LAUNCH_CHECK();
    return UPDES_OK;
  }
  const int nblk = int(ceil_div(p->N, kSymT));
  const dim3 grid{unsigned(nblk), unsigned(nblk)};
  if (df && p->rbf == UPDES_RBF_POLYHARMONIC) {
    float* tri = reinterpret_cast<float*>(part + size_t(nblk) * size_t(p->N));
    tri_coords_kernel<<<unsigned(ceil_div(p->N, 256)), 256, 0, s>>>(*p, tri);
    UPDES_LAUNCH_CHECK();
    eval_values_sym_df_kernel<<<grid, 256, 0, s>>>(*p, coeffs, tri, part);
    UPDES_LAUNCH_CHECK();
    eval_values_sym_reduce<<<unsigned(ceil_div(p->N, 256)), 256, 0, s>>>(*p, part, nblk, coeffs, vals);
    UPDES_LAUNCH_CHECK();
    return UPDES_OK;
  }
  switch (p->rbf) {
    case UPDES_RBF_POLYHARMONIC: eval_values_sym_kernel<UPDES_RBF_POLYHARMONIC><<<grid, 256, 0, s>>>(*p, coeffs, part); break;
    case UPDES_RBF_GAUSSIAN: eval_values_sym_kernel<UPDES_RBF_GAUSSIAN><<<grid, 256, 0, s>>>(*p, coeffs, part); break;
    case UPDES_RBF_MULTIQUADRIC: eval_values_sym_kernel<UPDES_RBF_MULTIQUADRIC><<<grid, 256, 0, s>>>(*p, coeffs, part); break;
    case UPDES_RBF_INVERSE_MULTIQUADRIC: eval_values_sym_kernel<UPDES_RBF_INVERSE_MULTIQUADRIC><<<grid, 256, 0, s>>>(*p, coeffs, part); break;
    default: eval_values_sym_kernel<UPDES_RBF_THIN_PLATE><<<grid, 256, 0, s>>>(*p, coeffs, part); break;
  }
  UPDES_LAUNCH_CHECK();
  eval_values_sym_reduce<<<unsigned(ceil_div(p->N, 256)), 256, 0, s>>>(*p, part, nblk, coeffs, vals);
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

extern "C" int updes_eval_values(const updes_problem* p, const double* coeffs, double* vals, void* stream) {
  int st = check_problem(p);
  if (st) return st;
  if (!coeffs || !vals) return UPDES_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->supports) {
    UPDES_DISPATCH_KIND(eval_values_local_kernel, unsigned(ceil_div(int64_t(p->N) * 32, 256)), 256, s, *p, coeffs,
                        vals);
    UPDES_LAUNCH_CHECK();
    return UPDES_OK;
  }
  const unsigned grid = unsigned(ceil_div(p->N, kEvalRows));
  switch (p->rbf) {
    case UPDES_RBF_POLYHARMONIC: eval_values_kernel<UPDES_RBF_POLYHARMONIC><<<grid, 256, 0, s>>>(*p, coeffs, vals); break;
    case UPDES_RBF_GAUSSIAN: eval_values_kernel<UPDES_RBF_GAUSSIAN><<<grid, 256, 0, s>>>(*p, coeffs, vals); break;
    case UPDES_RBF_MULTIQUADRIC: eval_values_kernel<UPDES_RBF_MULTIQUADRIC><<<grid, 256, 0, s>>>(*p, coeffs, vals); break;
    case UPDES_RBF_INVERSE_MULTIQUADRIC: eval_values_kernel<UPDES_RBF_INVERSE_MULTIQUADRIC><<<grid, 256, 0, s>>>(*p, coeffs, vals); break;
    default: eval_values_kernel<UPDES_RBF_THIN_PLATE><<<grid, 256, 0, s>>>(*p, coeffs, vals); break;
  }
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

extern "C" int updes_eval_field(int32_t m, const double* points, int32_t N, const double* centers, int32_t M,
                                int32_t rbf, double rbf_param, const double* coeffs, int32_t what, double* out,
                                void* stream) {
  if (m <= 0 || N <= 0 || !points || !centers || !coeffs || !out || what < 0 || what > 2) return UPDES_ERR_INVALID;
  if (!(M == 0 || M == 1 || M == 3 || M == 6 || M == 10 || M == 15)) return UPDES_ERR_INVALID;
  if (rbf < 0 || rbf > UPDES_RBF_THIN_PLATE) return UPDES_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const unsigned grid = unsigned(ceil_div(m, kEvalRows));
  switch (rbf) {
    case UPDES_RBF_POLYHARMONIC: eval_field_kernel<UPDES_RBF_POLYHARMONIC><<<grid, 256, 0, s>>>(m, points, N, centers, M, rbf_param, coeffs, what, out); break;
    case UPDES_RBF_GAUSSIAN: eval_field_kernel<UPDES_RBF_GAUSSIAN><<<grid, 256, 0, s>>>(m, points, N, centers, M, rbf_param, coeffs, what, out); break;
    case UPDES_RBF_MULTIQUADRIC: eval_field_kernel<UPDES_RBF_MULTIQUADRIC><<<grid, 256, 0, s>>>(m, points, N, centers, M, rbf_param, coeffs, what, out); break;
    case UPDES_RBF_INVERSE_MULTIQUADRIC: eval_field_kernel<UPDES_RBF_INVERSE_MULTIQUADRIC><<<grid, 256, 0, s>>>(m, points, N, centers, M, rbf_param, coeffs, what, out); break;
    default: eval_field_kernel<UPDES_RBF_THIN_PLATE><<<grid, 256, 0, s>>>(m, points, N, centers, M, rbf_param, coeffs, what, out); break;
  }
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

extern "C" int updes_coeff_grad(const updes_problem* p, const double* coeffs, const double* lambda, double* dW,
                                void* stream) {
  int st = check_problem(p);
  if (st) return st;
  if (!coeffs || !lambda || !dW) return UPDES_ERR_INVALID;
  if (p->Ni == 0) return UPDES_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->supports) {
    UPDES_DISPATCH_KIND(coeff_grad_local_kernel, unsigned(ceil_div(int64_t(p->Ni) * 32, 256)), 256, s, *p, coeffs,
                        lambda, dW);
    UPDES_LAUNCH_CHECK();
    return UPDES_OK;
  }
  const unsigned grid = unsigned(ceil_div(p->Ni, kEvalRows));
  switch (p->rbf) {
    case UPDES_RBF_POLYHARMONIC: coeff_grad_kernel<UPDES_RBF_POLYHARMONIC><<<grid, 256, 0, s>>>(*p, coeffs, lambda, dW); break;
    case UPDES_RBF_GAUSSIAN: coeff_grad_kernel<UPDES_RBF_GAUSSIAN><<<grid, 256, 0, s>>>(*p, coeffs, lambda, dW); break;
    case UPDES_RBF_MULTIQUADRIC: coeff_grad_kernel<UPDES_RBF_MULTIQUADRIC><<<grid, 256, 0, s>>>(*p, coeffs, lambda, dW); break;
    case UPDES_RBF_INVERSE_MULTIQUADRIC: coeff_grad_kernel<UPDES_RBF_INVERSE_MULTIQUADRIC><<<grid, 256, 0, s>>>(*p, coeffs, lambda, dW); break;
    default: coeff_grad_kernel<UPDES_RBF_THIN_PLATE><<<grid, 256, 0, s>>>(*p, coeffs, lambda, dW); break;
  }
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

extern "C" int updes_eval_values_t(const updes_problem* p, const double* g, double* out, void* stream) {
  int st = check_problem(p);
  if (st) return st;
  if (!g || !out) return UPDES_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->supports) {
    UPDES_CUDA_TRY(cudaMemsetAsync(out, 0, size_t(p->N) * sizeof(double), s));
    UPDES_DISPATCH_KIND(eval_values_local_t_kernel, unsigned(ceil_div(int64_t(p->N) * 32, 256)), 256, s, *p, g, out);
    UPDES_LAUNCH_CHECK();
    pt_matvec_kernel<<<1, 1024, 0, s>>>(*p, g, out);
    UPDES_LAUNCH_CHECK();
    return UPDES_OK;
  }
  const unsigned grid = unsigned(ceil_div(p->N, kEvalRows));
  // Phi is symmetric (radial kernel, same zero diagonal), so Phi^T g = Phi g
  switch (p->rbf) {
    case UPDES_RBF_POLYHARMONIC: eval_values_kernel<UPDES_RBF_POLYHARMONIC, false><<<grid, 256, 0, s>>>(*p, g, out); break;
    case UPDES_RBF_GAUSSIAN: eval_values_kernel<UPDES_RBF_GAUSSIAN, false><<<grid, 256, 0, s>>>(*p, g, out); break;
    case UPDES_RBF_MULTIQUADRIC: eval_values_kernel<UPDES_RBF_MULTIQUADRIC, false><<<grid, 256, 0, s>>>(*p, g, out); break;
    case UPDES_RBF_INVERSE_MULTIQUADRIC: eval_values_kernel<UPDES_RBF_INVERSE_MULTIQUADRIC, false><<<grid, 256, 0, s>>>(*p, g, out); break;
    default: eval_values_kernel<UPDES_RBF_THIN_PLATE, false><<<grid, 256, 0, s>>>(*p, g, out); break;
  }
  UPDES_LAUNCH_CHECK();
  pt_matvec_kernel<<<1, 1024, 0, s>>>(*p, g, out);
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

extern "C" int updes_eval_values_batch(const updes_problem* p, int32_t R, const double* C, int64_t ldc, double* vals,
                                       int64_t ldv, void* stream) {
  int st = check_problem(p);
  if (st) return st;
  if (!C || !vals || R <= 0 || R > 64 || ldc < R || ldv < R) return UPDES_ERR_INVALID;
  if (p->supports) return UPDES_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const unsigned grid = unsigned(ceil_div(p->N, kEvBRows));
  switch (p->rbf) {
    case UPDES_RBF_POLYHARMONIC: eval_values_batch_kernel<UPDES_RBF_POLYHARMONIC><<<grid, 256, 0, s>>>(*p, R, C, ldc, vals, ldv); break;
    case UPDES_RBF_GAUSSIAN: eval_values_batch_kernel<UPDES_RBF_GAUSSIAN><<<grid, 256, 0, s>>>(*p, R, C, ldc, vals, ldv); break;
    case UPDES_RBF_MULTIQUADRIC: eval_values_batch_kernel<UPDES_RBF_MULTIQUADRIC><<<grid, 256, 0, s>>>(*p, R, C, ldc, vals, ldv); break;
    case UPDES_RBF_INVERSE_MULTIQUADRIC: eval_values_batch_kernel<UPDES_RBF_INVERSE_MULTIQUADRIC><<<grid, 256, 0, s>>>(*p, R, C, ldc, vals, ldv); break;
    default: eval_values_batch_kernel<UPDES_RBF_THIN_PLATE><<<grid, 256, 0, s>>>(*p, R, C, ldc, vals, ldv); break;
  }
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

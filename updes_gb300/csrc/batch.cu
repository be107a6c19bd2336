// Batched right-hand sides against one factorisation, with a fixed number of refinement sweeps and no
// host synchronisation (a call only launches kernels on its stream, so time steps can be captured in a
// CUDA graph).  Time-stepped problems in the reference rebuild and refactor on every step
// (demos/Advection/00_advection_with_rbf.py:83-93); here the factors of updes_factor are reused and R
// right-hand sides (R <= 64) advance together:
//   X = M^-1 Bs;  repeat `sweeps` times:  X += M^-1 (Bs - Ks X)
// with Ks the equilibrated K (double-float planes of the solve workspace) and M^-1 the LU factors
// applied in double-float arithmetic.  FP64 factors are split once (updes_batch_prepare) into hi/lo FP32
// planes, so M^-1 is as accurate as an FP64 triangular solve while running on the FP32 pipes; FP32
// factors are used as they are (lo = 0).
//
// Every double-float accumulation renormalises after each term (fast two-sum), so its error stays at
// about 2^-48 of the running sum however many terms a thread adds.
#include <atomic>
#include <cstring>

#include "common.cuh"
#include "lu.cuh"
#include "stats.cuh"

namespace {

constexpr int kB = 64;       // block rows
constexpr int kMaxR = 64;    // right-hand sides per call
constexpr int kRG = 16;      // right-hand sides per triangular-solve CTA
constexpr int kGroups = kMaxR / kRG;
constexpr int kParts = 4;    // split of the residual's inner dimension

// (sh, sl) += (a + al) * (b + bl), dropping al * bl; renormalised
__device__ __forceinline__ void df_mac(float a, float al, float b, float bl, float& sh, float& sl) {
  const float p = __fmul_rn(a, b);
  const float e = __fmaf_rn(a, b, -p);
  const float s = __fadd_rn(sh, p);
  const float bb = __fsub_rn(s, sh);
  float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  t = __fadd_rn(t, __fadd_rn(sl, __fmaf_rn(a, bl, __fmaf_rn(al, b, e))));
  sh = __fadd_rn(s, t);
  sl = __fsub_rn(t, __fsub_rn(sh, s));
}

// (qh, ql) = (bh + bl) / (dh + dl)
__device__ __forceinline__ void df_div(float bh, float bl, float dh, float dl, float& qh, float& ql) {
  const float q1 = __fdiv_rn(bh, dh);
  const float p = __fmul_rn(q1, dh);
  const float pe = __fmaf_rn(q1, dh, -p);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(bh, p), pe), __fsub_rn(bl, __fmul_rn(q1, dl)));
  const float q2 = __fdiv_rn(r, dh);
  qh = __fadd_rn(q1, q2);
  ql = __fsub_rn(q2, __fsub_rn(qh, q1));
}

__device__ __forceinline__ void split(double v, float& h, float& l) {
  h = float(v);
  l = float(v - double(h));
}

// Header of the batch workspace: {n, precision of the factors, valid, factor generation}
struct BatchHeader {
  int32_t n, precision, valid, generation;
};

// ---------------------------------------------------------------------------
// Residual: partial[p] = Ks[rows of this block, k-range p] * X  (double-float), p = blockIdx.y
struct KxSmem {
  float Kh[kB][kB + 1], Kl[kB][kB + 1];
  float Xh[kB][kMaxR + 1], Xl[kB][kMaxR + 1];
};

__global__ void __launch_bounds__(256) batch_kx_kernel(const float* __restrict__ Khi, const float* __restrict__ Klo,
                                                       int64_t ld, int n, const double* __restrict__ X, int R,
                                                       double* __restrict__ partial) {
  extern __shared__ float4 kx_smem[];
  KxSmem& sm = *reinterpret_cast<KxSmem*>(kx_smem);
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  const int r0 = blockIdx.x * kB;
  const int ntile = int(ceil_div(n, kB));
  const int t0 = int(ceil_div(int64_t(ntile) * blockIdx.y, kParts));
  const int t1 = int(ceil_div(int64_t(ntile) * (blockIdx.y + 1), kParts));
  float ah[4][4], al[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) ah[u][v] = al[u][v] = 0.f;
  for (int tt = t0; tt < t1; ++tt) {
    const int c0 = tt * kB;
    for (int e = tid; e < kB * kB; e += blockDim.x) {
      const int i = e >> 6, j = e & 63;
      const bool ok = r0 + i < n && c0 + j < n;
      sm.Kh[i][j] = ok ? Khi[int64_t(r0 + i) * ld + c0 + j] : 0.f;
      sm.Kl[i][j] = ok ? Klo[int64_t(r0 + i) * ld + c0 + j] : 0.f;
    }
    for (int e = tid; e < kB * kMaxR; e += blockDim.x) {
      const int i = e / kMaxR, c = e % kMaxR;
      const double v = (c0 + i < n && c < R) ? X[int64_t(c0 + i) * R + c] : 0.0;
      split(v, sm.Xh[i][c], sm.Xl[i][c]);
    }
    __syncthreads();
#pragma unroll 2
    for (int kk = 0; kk < kB; ++kk) {
      float a[4], a2[4], b[4], b2[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) { a[u] = sm.Kh[ty * 4 + u][kk]; a2[u] = sm.Kl[ty * 4 + u][kk]; }
#pragma unroll
      for (int v = 0; v < 4; ++v) { b[v] = sm.Xh[kk][tx * 4 + v]; b2[v] = sm.Xl[kk][tx * 4 + v]; }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) df_mac(a[u], a2[u], b[v], b2[v], ah[u][v], al[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int r = r0 + ty * 4 + u;
    if (r >= n) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int c = tx * 4 + v;
      if (c < R) partial[(int64_t(blockIdx.y) * n + r) * R + c] = double(ah[u][v]) + double(al[u][v]);
    }
  }
}

// Res = Bs - sum_p partial[p]
__global__ void batch_residual_kernel(const double* __restrict__ Bs, const double* __restrict__ partial, int n, int R,
                                      double* __restrict__ Res) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(n) * R) return;
  double s = 0.0;
  for (int p = 0; p < kParts; ++p) s += partial[int64_t(p) * n * R + e];
  Res[e] = Bs[e] - s;
}

// Bs[i][c] = dr_i * Q[i][c] (i < N), 0 for the polynomial rows.  The solve workspace must hold factors of
// this size and the batch header must describe them (same generation); otherwise the status records
// UPDES_ERR_INVALID and the right-hand sides become NaN, so nothing downstream passes for a solution.
__global__ void batch_rhs_kernel(const double* __restrict__ Q, int64_t ldq, int N, int n, int R,
                                 const double* __restrict__ dr, double* __restrict__ Bs,
                                 const int32_t* __restrict__ state, const BatchHeader* __restrict__ hdr,
                                 DeviceStatus* st) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const bool ok = state[0] == n && state[2] == 1 && hdr->n == n && hdr->valid == 1 &&
                  hdr->precision == state[1] && hdr->generation == state[3];
  if (!ok && e == 0) status_error(st, UPDES_ERR_INVALID);
  if (e >= int64_t(n) * R) return;
  const int i = int(e / R), c = int(e % R);
  Bs[e] = !ok ? __longlong_as_double(0x7ff8000000000000ll) : (i < N ? dr[i] * Q[int64_t(i) * ldq + c] : 0.0);
}

// Y[i][c] = X[perm[i]][c]
__global__ void batch_gather_kernel(const double* __restrict__ X, double* __restrict__ Y,
                                    const int32_t* __restrict__ perm, int n, int R) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(n) * R) return;
  const int i = int(e / R), c = int(e % R);
  Y[e] = X[int64_t(perm[i]) * R + c];
}

__global__ void batch_axpy_kernel(double* __restrict__ X, const double* __restrict__ D, int64_t total) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e < total) X[e] += D[e];
}

// out[i][c] (ld = ldo) = dc_i * X[i][c]
__global__ void batch_unscale_kernel(const double* __restrict__ X, const double* __restrict__ dc, int n, int R,
                                     double* __restrict__ out, int64_t ldo) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(n) * R) return;
  const int i = int(e / R), c = int(e % R);
  out[int64_t(i) * ldo + c] = dc[i] * X[e];
}

// FP64 factors -> hi/lo FP32 planes
__global__ void split_factors_kernel(const double* __restrict__ F, float* __restrict__ Fh, float* __restrict__ Fl,
                                     int64_t total) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e < total) split(F[e], Fh[e], Fl[e]);
}

// ---------------------------------------------------------------------------
// Triangular solves of an n x R block in place (LOWER: unit lower, forward; else upper, backward).
// One CTA per (64-row block, group of 16 right-hand sides), taken in ticket order: the t-th ticket of a
// group waits (bounded) until the group's t earlier blocks are done, subtracting each finished block's
// contribution as soon as it is available, then solves its diagonal block warp by warp (two right-hand
// sides per warp, lanes own rows lane and lane + 32, x_i broadcast by shuffles).
struct TrsmSmem {
  float Fh[kB][kB + 1], Fl[kB][kB + 1];
  float Xh[kB][kRG + 1], Xl[kB][kRG + 1];
};

template <bool LOWER, bool DF>
__device__ __forceinline__ void trsm_block(const float* __restrict__ Fh, const float* __restrict__ Fl, int64_t ldf,
                                           int n, double* X, int R, int t, int g, int* done, DeviceStatus* st,
                                           TrsmSmem& sm, int& s_done) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nblk = int(ceil_div(n, kB));
  const int blk = LOWER ? t : nblk - 1 - t;
  const int r0 = blk * kB;
  const int rows = min(kB, n - r0);
  const int cbase = g * kRG;
  // off-diagonal part: thread owns row tid / 4 and columns (tid % 4) * 4 + {0..3} of the group
  const int orow = tid >> 2, ocol = (tid & 3) * 4;
  float ah[4] = {0.f, 0.f, 0.f, 0.f}, al[4] = {0.f, 0.f, 0.f, 0.f};
  for (int q = 0; q < t; ++q) {
    const int jb = LOWER ? q : nblk - 1 - q;
    const int c0 = jb * kB;
    for (int e = tid; e < kB * kB; e += blockDim.x) {
      const int i = e >> 6, j = e & 63;
      const bool ok = r0 + i < n && c0 + j < n;
      sm.Fh[i][j] = ok ? Fh[int64_t(r0 + i) * ldf + c0 + j] : 0.f;
      if (DF) sm.Fl[i][j] = ok ? Fl[int64_t(r0 + i) * ldf + c0 + j] : 0.f;
    }
    if (tid == 0 && s_done <= q) {
      volatile int* vc = done + g;
      long long it = 0;
      int d;
      while ((d = *vc) <= q) {
        if (++it > spin_limit()) {
          status_error(st, UPDES_ERR_TIMEOUT);
          atomicCAS(&st->timeout_tag, 0, 30);
          d = q + 1;
          break;
        }
        __nanosleep(20);
      }
      __threadfence();
      s_done = d;
    }
    __syncthreads();
    for (int e = tid; e < kB * kRG; e += blockDim.x) {
      const int i = e / kRG, c = e % kRG;
      double v = 0.0;
      if (c0 + i < n && cbase + c < R) v = __ldcg(X + int64_t(c0 + i) * R + cbase + c);
      split(v, sm.Xh[i][c], sm.Xl[i][c]);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kB; ++kk) {
      const float a = sm.Fh[orow][kk];
      const float a2 = DF ? sm.Fl[orow][kk] : 0.f;
#pragma unroll
      for (int v = 0; v < 4; ++v) df_mac(a, a2, sm.Xh[kk][ocol + v], sm.Xl[kk][ocol + v], ah[v], al[v]);
    }
    __syncthreads();
  }
  // right-hand side of this block minus the off-diagonal part
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const int c = ocol + v;
    double b = 0.0;
    if (orow < rows && cbase + c < R) b = X[int64_t(r0 + orow) * R + cbase + c] - (double(ah[v]) + double(al[v]));
    split(b, sm.Xh[orow][c], sm.Xl[orow][c]);
  }
  for (int e = tid; e < kB * kB; e += blockDim.x) {
    const int i = e >> 6, j = e & 63;
    const bool ok = i < rows && j < rows;
    sm.Fh[i][j] = ok ? Fh[int64_t(r0 + i) * ldf + r0 + j] : 0.f;
    if (DF) sm.Fl[i][j] = ok ? Fl[int64_t(r0 + i) * ldf + r0 + j] : 0.f;
  }
  __syncthreads();
  // diagonal block: warp w solves columns 2w, 2w + 1 of the group
  {
    float bh[2][2], bl[2][2];  // [row slot][column]
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        bh[u][v] = sm.Xh[lane + 32 * u][2 * warp + v];
        bl[u][v] = sm.Xl[lane + 32 * u][2 * warp + v];
      }
    for (int s2 = 0; s2 < rows; ++s2) {
      const int i = LOWER ? s2 : rows - 1 - s2;
      const int owner = i & 31, slot = i >> 5;
      float xh[2], xl[2];
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const float h = slot ? bh[1][v] : bh[0][v];
        const float l = slot ? bl[1][v] : bl[0][v];
        xh[v] = __shfl_sync(0xffffffffu, h, owner);
        xl[v] = __shfl_sync(0xffffffffu, l, owner);
        if (!LOWER) df_div(xh[v], xl[v], sm.Fh[i][i], DF ? sm.Fl[i][i] : 0.f, xh[v], xl[v]);
      }
      if (lane == owner) {
#pragma unroll
        for (int v = 0; v < 2; ++v) {
          if (slot) { bh[1][v] = xh[v]; bl[1][v] = xl[v]; }
          else { bh[0][v] = xh[v]; bl[0][v] = xl[v]; }
        }
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int r = lane + 32 * u;
        if (r < rows && (LOWER ? r > i : r < i)) {
          const float f = -sm.Fh[r][i];
          const float f2 = DF ? -sm.Fl[r][i] : 0.f;
#pragma unroll
          for (int v = 0; v < 2; ++v) df_mac(f, f2, xh[v], xl[v], bh[u][v], bl[u][v]);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int r = lane + 32 * u;
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const int c = cbase + 2 * warp + v;
        if (r < rows && c < R) X[int64_t(r0 + r) * R + c] = double(bh[u][v]) + double(bl[u][v]);
      }
    }
  }
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    atomicAdd(done + g, 1);
  }
}

template <bool LOWER>
__global__ void __launch_bounds__(256) batch_trsm_kernel(const float* __restrict__ F32, const float* __restrict__ Fh,
                                                         const float* __restrict__ Fl, int64_t ldf, int n, double* X,
                                                         int R, int* ticket, int* done, const BatchHeader* hdr,
                                                         DeviceStatus* st) {
  __shared__ TrsmSmem sm;
  __shared__ int s_tk, s_done;
  const int G = int(ceil_div(R, kRG));
  const int nblk = int(ceil_div(n, kB));
  if (threadIdx.x == 0) {
    s_tk = atomicAdd(ticket, 1);
    s_done = 0;
  }
  __syncthreads();
  const int tk = s_tk;
  const int t = tk / G, g = tk % G;
  if (t >= nblk) return;
  if (hdr->precision == UPDES_PREC_FP64) trsm_block<LOWER, true>(Fh, Fl, ldf, n, X, R, t, g, done, st, sm, s_done);
  else trsm_block<LOWER, false>(F32, nullptr, ldf, n, X, R, t, g, done, st, sm, s_done);
}

// ---------------------------------------------------------------------------
struct BatchWs {
  BatchHeader* hdr;
  float *Fh, *Fl;
  double *Bs, *X, *D, *T, *partial;
  int* sync;
};

size_t batch_layout(int n, char* base, BatchWs* w) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    off = (off + 255) & ~size_t(255);
    char* p = base ? base + off : nullptr;
    off += bytes;
    return p;
  };
  const int64_t ld = updes_matrix_ld(n, 8);
  const size_t v = size_t(n) * kMaxR * sizeof(double);
  BatchWs b;
  b.hdr = reinterpret_cast<BatchHeader*>(take(sizeof(BatchHeader)));
  b.Fh = reinterpret_cast<float*>(take(size_t(n) * ld * sizeof(float)));
  b.Fl = reinterpret_cast<float*>(take(size_t(n) * ld * sizeof(float)));
  b.Bs = reinterpret_cast<double*>(take(v));
  b.X = reinterpret_cast<double*>(take(v));
  b.D = reinterpret_cast<double*>(take(v));
  b.T = reinterpret_cast<double*>(take(v));
  b.partial = reinterpret_cast<double*>(take(kParts * v));
  b.sync = reinterpret_cast<int*>(take(2 * (1 + kGroups) * sizeof(int)));
  if (w) *w = b;
  return off + 256;
}

// Opt the residual kernel into its dynamic shared memory on the current device (once per device; a
// host call that is not a stream operation, made before the first launch).
int batch_kernel_setup() {
  static std::atomic<unsigned long long> ready{0};
  return smem_opt_in((const void*)batch_kx_kernel, int(sizeof(KxSmem)), ready);
}

}  // namespace

// Views of the solve workspace the batch needs (defined in solve.cu).
int solve_ws_views(const updes_problem* p, void* workspace, size_t workspace_bytes, const float** Khi,
                   const float** Klo, const float** F32, const double** F64, int64_t* ld, const int32_t** piv,
                   const double** dr, const double** dc, DeviceStatus** st, const int32_t** state);

namespace {

// Y <- M^-1 Y for an n x R block (permute, L, U).
int batch_precond(int n, int R, const float* F32, const BatchWs& b, int64_t ld, const int32_t* piv, double* Y,
                  DeviceStatus* st, cudaStream_t s) {
  const unsigned g = unsigned(ceil_div(int64_t(n) * R, 256));
  const int nblk = int(ceil_div(n, kB));
  const int G = int(ceil_div(R, kRG));
  batch_gather_kernel<<<g, 256, 0, s>>>(Y, b.T, piv + n, n, R);
  UPDES_LAUNCH_CHECK();
  StatScope sc(kStatTrsv, s, 2.0 * n * n * R, double(n) * n * 8.0);
  UPDES_CUDA_TRY(cudaMemsetAsync(b.sync, 0, 2 * (1 + kGroups) * sizeof(int), s));
  int* lo_sync = b.sync;
  int* up_sync = b.sync + 1 + kGroups;
  batch_trsm_kernel<true><<<unsigned(nblk * G), 256, 0, s>>>(F32, b.Fh, b.Fl, ld, n, b.T, R, lo_sync, lo_sync + 1,
                                                             b.hdr, st);
  UPDES_LAUNCH_CHECK();
  batch_trsm_kernel<false><<<unsigned(nblk * G), 256, 0, s>>>(F32, b.Fh, b.Fl, ld, n, b.T, R, up_sync, up_sync + 1,
                                                              b.hdr, st);
  UPDES_LAUNCH_CHECK();
  UPDES_CUDA_TRY(cudaMemcpyAsync(Y, b.T, size_t(n) * R * sizeof(double), cudaMemcpyDeviceToDevice, s));
  return UPDES_OK;
}

}  // namespace

extern "C" int updes_batch_workspace(int32_t n, size_t* bytes) {
  if (n <= 0 || !bytes) return UPDES_ERR_INVALID;
  *bytes = batch_layout(n, nullptr, nullptr);
  return UPDES_OK;
}

extern "C" int updes_batch_prepare(const updes_problem* p, void* workspace, size_t workspace_bytes, void* batch_ws,
                                   size_t batch_ws_bytes, void* stream) {
  if (!p || !batch_ws) return UPDES_ERR_INVALID;
  const int n = p->N + p->M;
  if (batch_ws_bytes < batch_layout(n, nullptr, nullptr)) return UPDES_ERR_WORKSPACE;
  const float *Khi, *Klo, *F32;
  const double *F64, *dr, *dc;
  const int32_t *piv, *state;
  int64_t ld;
  DeviceStatus* st;
  int e = solve_ws_views(p, workspace, workspace_bytes, &Khi, &Klo, &F32, &F64, &ld, &piv, &dr, &dc, &st, &state);
  if (e) return e;
  if ((e = batch_kernel_setup())) return e;
  BatchWs b;
  batch_layout(n, static_cast<char*>(batch_ws), &b);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int32_t h[4];
  UPDES_CUDA_TRY(cudaMemcpyAsync(h, state, sizeof h, cudaMemcpyDeviceToHost, s));
  UPDES_CUDA_TRY(cudaStreamSynchronize(s));
  if (h[0] != n || h[2] != 1) return UPDES_ERR_INVALID;  // no factorisation of this system in the workspace
  if (h[1] == UPDES_PREC_FP64) {
    const int64_t total = int64_t(n) * ld;
    split_factors_kernel<<<unsigned(ceil_div(total, 256)), 256, 0, s>>>(F64, b.Fh, b.Fl, total);
    UPDES_LAUNCH_CHECK();
  }
  const BatchHeader hd{n, h[1], 1, h[3]};
  UPDES_CUDA_TRY(cudaMemcpyAsync(b.hdr, &hd, sizeof hd, cudaMemcpyHostToDevice, s));
  UPDES_CUDA_TRY(cudaStreamSynchronize(s));
  return UPDES_OK;
}

extern "C" int updes_solve_batch(const updes_problem* p, int32_t R, const double* Q, int64_t ldq, double* coeffs,
                                 int64_t ldc, int32_t sweeps, void* workspace, size_t workspace_bytes,
                                 void* batch_ws, size_t batch_ws_bytes, void* stream) {
  if (!p || R <= 0 || R > kMaxR || !Q || !coeffs || ldq < R || ldc < R || sweeps < 0 || !batch_ws)
    return UPDES_ERR_INVALID;
  const int n = p->N + p->M;
  if (batch_ws_bytes < batch_layout(n, nullptr, nullptr)) return UPDES_ERR_WORKSPACE;
  const float *Khi, *Klo, *F32;
  const double *F64, *dr, *dc;
  const int32_t *piv, *state;
  int64_t ld;
  DeviceStatus* st;
  int e = solve_ws_views(p, workspace, workspace_bytes, &Khi, &Klo, &F32, &F64, &ld, &piv, &dr, &dc, &st, &state);
  if (e) return e;
  if ((e = batch_kernel_setup())) return e;
  BatchWs b;
  batch_layout(n, static_cast<char*>(batch_ws), &b);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t total = int64_t(n) * R;
  const unsigned g = unsigned(ceil_div(total, 256));
  batch_rhs_kernel<<<g, 256, 0, s>>>(Q, ldq, p->N, n, R, dr, b.Bs, state, b.hdr, st);
  UPDES_LAUNCH_CHECK();
  UPDES_CUDA_TRY(cudaMemcpyAsync(b.X, b.Bs, size_t(total) * 8, cudaMemcpyDeviceToDevice, s));
  if ((e = batch_precond(n, R, F32, b, ld, piv, b.X, st, s))) return e;
  for (int it = 0; it < sweeps; ++it) {
    {
      StatScope sc(kStatGemv, s, 2.0 * n * n * R, 8.0 * n * double(ld));
      batch_kx_kernel<<<dim3(unsigned(ceil_div(n, kB)), kParts), 256, sizeof(KxSmem), s>>>(Khi, Klo, ld, n, b.X, R,
                                                                                          b.partial);
      UPDES_LAUNCH_CHECK();
      batch_residual_kernel<<<g, 256, 0, s>>>(b.Bs, b.partial, n, R, b.D);
      UPDES_LAUNCH_CHECK();
    }
    if ((e = batch_precond(n, R, F32, b, ld, piv, b.D, st, s))) return e;
    batch_axpy_kernel<<<g, 256, 0, s>>>(b.X, b.D, total);
    UPDES_LAUNCH_CHECK();
  }
  batch_unscale_kernel<<<g, 256, 0, s>>>(b.X, dc, n, R, coeffs, ldc);
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

// Public LU / solve entry points and the GMRES-refined collocation solve.
//
// updes_solve replaces pde_solver's assemble_B -> lineax QR ->
// core_compute_coefficients sequence (updes/operators.py:602-618) by one
// factorisation of the augmented Kansa matrix K and refinement in FP64.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "gemm_tc.cuh"
#include "lu.cuh"
#include "stats.cuh"

int updes_check_problem(const updes_problem* p);
size_t eval_values_sym_bytes(int N);
int eval_values_sym(const updes_problem* p, const double* coeffs, double* vals, double* part, cudaStream_t s,
                    bool df);

namespace {

std::mutex g_err_mu;
std::string g_last_error;

constexpr int kMaxPermN = 51200;  // permutation built in shared memory

__global__ void perm_from_piv_kernel(const int32_t* __restrict__ piv, int n, int32_t* __restrict__ perm) {
  extern __shared__ int32_t sp[];
  for (int i = threadIdx.x; i < n; i += blockDim.x) sp[i] = i;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; ++i) {
      const int p = piv[i];
      if (p != i) {
        const int a = sp[i];
        sp[i] = sp[p];
        sp[p] = a;
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = sp[i];
}

// out[i] = scale[i] * in[perm[i]] (gather, scale may be null) or out[perm[i]] = in[i] (scatter)
__global__ void permute_kernel(double* __restrict__ out, const double* __restrict__ in, int64_t in_stride,
                               int64_t out_stride, const int32_t* __restrict__ perm, int n, int scatter) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (scatter) out[int64_t(perm[i]) * out_stride] = in[int64_t(i) * in_stride];
  else out[int64_t(i) * out_stride] = in[int64_t(perm[i]) * in_stride];
}

// dr[i] = 2^-round(log2(max_j |K_ij|)) (power of two, so scaling is exact)
__global__ void row_scale_kernel(const double* __restrict__ K, int64_t ld, int n, double* __restrict__ dr) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;
  double m = 0.0;
  for (int j = lane; j < n; j += 32) m = fmax(m, fabs(K[int64_t(warp) * ld + j]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) {
    int e = 0;
    if (m > 0.0 && isfinite(m)) frexp(m, &e);
    dr[warp] = ldexp(1.0, -e);
  }
}

// Column maxima of |K| diag(dr) over a chunk of rows per blockIdx.y, combined with an integer atomicMax on the
// bit patterns (non-negative doubles order like their bits); colmax must start at zero.
constexpr int kColScaleChunks = 64;
__global__ void col_max_kernel(const double* __restrict__ K, int64_t ld, int n, const double* __restrict__ dr,
                               unsigned long long* __restrict__ colmax) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int rows = int(ceil_div(n, kColScaleChunks));
  const int i0 = blockIdx.y * rows, i1 = min(n, i0 + rows);
  double m = 0.0;
  for (int i = i0; i < i1; ++i) m = fmax(m, fabs(K[int64_t(i) * ld + j]) * dr[i]);
  if (m > 0.0) atomicMax(colmax + j, (unsigned long long)__double_as_longlong(m));
}

// dc_j = 2^-e with max_i |K_ij| dr_i in [2^(e-1), 2^e)  (dc holds the maxima' bits on entry)
__global__ void col_scale_kernel(int n, double* __restrict__ dc) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double m = __longlong_as_double((long long)reinterpret_cast<unsigned long long*>(dc)[j]);
  int e = 0;
  if (m > 0.0 && isfinite(m)) frexp(m, &e);
  dc[j] = ldexp(1.0, -e);
}


// dr[i] = 2^-e with the row maximum (FP32 bit pattern in maxbits) in [2^(e-1), 2^e)
__global__ void row_scale_bits_kernel(const unsigned* __restrict__ maxbits, int n, double* __restrict__ dr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double m = double(__uint_as_float(maxbits[i]));
  int e = 0;
  if (m > 0.0 && isfinite(m)) frexp(m, &e);
  dr[i] = ldexp(1.0, -e);
}

// Column maxima of |Khi| diag(dr) (the FP32 plane of an unscaled double-float K), as col_max_kernel.
__global__ void col_max_f32_kernel(const float* __restrict__ Khi, int64_t ld, int n, const double* __restrict__ dr,
                                   unsigned long long* __restrict__ colmax) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int rows = int(ceil_div(n, kColScaleChunks));
  const int i0 = blockIdx.y * rows, i1 = min(n, i0 + rows);
  // eight independent loads in flight per thread (the column walk is otherwise one dependent load per row);
  // |hi| dr_i is formed in FP32 (dr is a power of two, exact) and widened once at the end
  float m8[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  int i = i0;
  for (; i + 8 <= i1; i += 8) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = __ldg(Khi + int64_t(i + u) * ld + j);
#pragma unroll
    for (int u = 0; u < 8; ++u) m8[u] = fmaxf(m8[u], fabsf(v[u]) * float(dr[i + u]));
  }
  for (; i < i1; ++i) m8[0] = fmaxf(m8[0], fabsf(__ldg(Khi + int64_t(i) * ld + j)) * float(dr[i]));
  float mf = m8[0];
#pragma unroll
  for (int u = 1; u < 8; ++u) mf = fmaxf(mf, m8[u]);
  const double m = double(mf);
  if (m > 0.0) atomicMax(colmax + j, (unsigned long long)__double_as_longlong(m));
}

// Both planes times dr_i dc_j in place (powers of two: exact), four columns a thread, rows strided over grid.y;
// with hi2/lo2 the scaled planes are also written there (the factorisation's working copy, in the same pass).
__global__ void __launch_bounds__(256) scale_planes_kernel(float* __restrict__ hi, float* __restrict__ lo, int64_t ld,
                                                           int n, const double* __restrict__ dr,
                                                           const double* __restrict__ dc, float* __restrict__ hi2,
                                                           float* __restrict__ lo2) {
  const int64_t j0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) * 4;
  if (j0 >= n) return;
  float cs[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) cs[u] = j0 + u < n ? float(dc[j0 + u]) : 1.f;
  for (int i = blockIdx.y; i < n; i += gridDim.y) {
    const float rs = float(dr[i]);
    float4* ph = reinterpret_cast<float4*>(hi + int64_t(i) * ld + j0);
    float4* pl = reinterpret_cast<float4*>(lo + int64_t(i) * ld + j0);
    float4 h = *ph, l = *pl;
    h.x = h.x * rs * cs[0]; h.y = h.y * rs * cs[1]; h.z = h.z * rs * cs[2]; h.w = h.w * rs * cs[3];
    l.x = l.x * rs * cs[0]; l.y = l.y * rs * cs[1]; l.z = l.z * rs * cs[2]; l.w = l.w * rs * cs[3];
    *ph = h;
    *pl = l;
    if (hi2) {
      *reinterpret_cast<float4*>(hi2 + int64_t(i) * ld + j0) = h;
      *reinterpret_cast<float4*>(lo2 + int64_t(i) * ld + j0) = l;
    }
  }
}

// out_i = dr_i * (bsign * b_i + ksign * sum_j K_ij dc_j x_j), one warp per row (dr, dc, b may be null)
// With absout != null also writes absout_i = dr_i * (sum_j |K_ij dc_j x_j| + |b_i|) (backward-error denominators).
__global__ void __launch_bounds__(256) gemv_kernel(const double* __restrict__ K, int64_t ld, int n,
                                                   const double* __restrict__ x, const double* __restrict__ b,
                                                   const double* __restrict__ dr, const double* __restrict__ dc,
                                                   double bsign, double ksign, double* __restrict__ out,
                                                   double* __restrict__ absout = nullptr) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;
  const double* row = K + int64_t(warp) * ld;
  double s = 0.0, a = 0.0;
  for (int j = lane; j < n; j += 32) {
    const double t = row[j] * (dc ? dc[j] * x[j] : x[j]);
    s += t;
    a += fabs(t);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    a += __shfl_xor_sync(0xffffffffu, a, o);
  }
  if (lane == 0) {
    double v = ksign * s + (b ? bsign * b[warp] : 0.0);
    out[warp] = dr ? dr[warp] * v : v;
    if (absout) absout[warp] = (dr ? dr[warp] : 1.0) * (a + (b ? fabs(b[warp]) : 0.0));
  }
}

// partial maxima of |r_i| / a_i (a_i = 0 with r_i = 0 counts as 0)
__global__ void bwd_partial_kernel(const double* __restrict__ r, const double* __restrict__ a, int n,
                                   double* __restrict__ partial) {
  __shared__ double red[8];
  double m = 0.0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const double rr = fabs(r[t]);
    const double v = a[t] > 0.0 ? rr / a[t] : (rr > 0.0 ? INFINITY : 0.0);
    m = fmax(m, v != v ? INFINITY : v);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < 8; ++q) t = fmax(t, red[q]);
    partial[blockIdx.x] = t;
  }
}

// Transposed: out_j = dc_j * (bsign * b_j + ksign * sum_i K_ij dr_i x_i), 256 columns per CTA.
__global__ void __launch_bounds__(256) gemv_t_kernel(const double* __restrict__ K, int64_t ld, int n,
                                                     const double* __restrict__ x, const double* __restrict__ b,
                                                     const double* __restrict__ dr, const double* __restrict__ dc,
                                                     double bsign, double ksign, double* __restrict__ out,
                                                     double* __restrict__ absout = nullptr) {
  __shared__ double part[8][33], apart[8][33];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int j = blockIdx.x * 32 + lane;
  double s = 0.0, a = 0.0;
  if (j < n)
    for (int i = w; i < n; i += 8) {
      const double t = K[int64_t(i) * ld + j] * (dr ? dr[i] * x[i] : x[i]);
      s += t;
      a += fabs(t);
    }
  part[w][lane] = s;
  apart[w][lane] = a;
  __syncthreads();
  if (w == 0 && j < n) {
    double t = 0.0, ta = 0.0;
    for (int q = 0; q < 8; ++q) {
      t += part[q][lane];
      ta += apart[q][lane];
    }
    double v = ksign * t + (b ? bsign * b[j] : 0.0);
    out[j] = dc ? dc[j] * v : v;
    if (absout) absout[j] = (dc ? dc[j] : 1.0) * (ta + (b ? fabs(b[j]) : 0.0));
  }
}

// Double-float matrix-vector products with the equilibrated K stored as FP32 planes (hi, lo):
// exact FP32 products (FMA), compensated sums; the absolute sums for the backward error in FP32.
__device__ __forceinline__ void df_acc(float kh, float kl, float a, float b, float& sh, float& sl, float& sa) {
  const float p = __fmul_rn(kh, a);
  const float e = __fmaf_rn(kh, a, -p);
  const float s = __fadd_rn(sh, p);
  const float bb = __fsub_rn(s, sh);
  float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  t = __fadd_rn(t, __fadd_rn(sl, __fmaf_rn(kh, b, __fmaf_rn(kl, a, e))));
  sh = __fadd_rn(s, t);  // renormalise, so the low word never carries more than half an ulp of sh
  sl = __fsub_rn(t, __fsub_rn(sh, s));
  sa = __fadd_rn(sa, fabsf(p));
}

// out_i = ksign * sum_j K_ij x_j (x as FP32 planes xh, xl padded with zeros to ld); absout_i = sum |K_ij x_j|
__global__ void __launch_bounds__(256) gemv_df_kernel(const float* __restrict__ Khi, const float* __restrict__ Klo,
                                                      int64_t ld, int n, const float* __restrict__ xh,
                                                      const float* __restrict__ xl, double ksign,
                                                      double* __restrict__ out, double* __restrict__ absout) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (row >= n) return;
  const float4* kh4 = reinterpret_cast<const float4*>(Khi + int64_t(row) * ld);
  const float4* kl4 = reinterpret_cast<const float4*>(Klo + int64_t(row) * ld);
  const float4* a4 = reinterpret_cast<const float4*>(xh);
  const float4* b4 = reinterpret_cast<const float4*>(xl);
  float sh = 0.f, sl = 0.f, sa = 0.f;
  for (int64_t q = lane; q < ld / 4; q += 32) {
    const float4 kh = kh4[q], kl = kl4[q], a = a4[q], b = b4[q];
    df_acc(kh.x, kl.x, a.x, b.x, sh, sl, sa);
    df_acc(kh.y, kl.y, a.y, b.y, sh, sl, sa);
    df_acc(kh.z, kl.z, a.z, b.z, sh, sl, sa);
    df_acc(kh.w, kl.w, a.w, b.w, sh, sl, sa);
  }
  double v = double(sh) + double(sl);
  for (int o = 16; o > 0; o >>= 1) {
    v += __shfl_xor_sync(0xffffffffu, v, o);
    sa += __shfl_xor_sync(0xffffffffu, sa, o);
  }
  if (lane == 0) {
    out[row] = ksign * v;
    if (absout) absout[row] = double(sa);
  }
}

// out_j = ksign * sum_i K_ij x_i (transposed), 32 columns per CTA, 8 warps over the rows
__global__ void __launch_bounds__(256) gemv_t_df_kernel(const float* __restrict__ Khi, const float* __restrict__ Klo,
                                                        int64_t ld, int n, const float* __restrict__ xh,
                                                        const float* __restrict__ xl, double ksign,
                                                        double* __restrict__ out, double* __restrict__ absout) {
  __shared__ double part[8][33];
  __shared__ float apart[8][33];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int j = blockIdx.x * 32 + lane;
  float sh = 0.f, sl = 0.f, sa = 0.f;
  if (j < n)
    for (int i = w; i < n; i += 8) {
      const int64_t idx = int64_t(i) * ld + j;
      df_acc(Khi[idx], Klo[idx], xh[i], xl[i], sh, sl, sa);
    }
  part[w][lane] = double(sh) + double(sl);
  apart[w][lane] = sa;
  __syncthreads();
  if (w == 0 && j < n) {
    double t = 0.0;
    float ta = 0.f;
    for (int q = 0; q < 8; ++q) {
      t += part[q][lane];
      ta += apart[q][lane];
    }
    out[j] = ksign * t;
    if (absout) absout[j] = double(ta);
  }
}

// (xh, xl) = FP32 planes of x (n values, zero padded to ld)
__global__ void split_vec_kernel(const double* __restrict__ x, int n, int64_t ld, float* __restrict__ xh,
                                 float* __restrict__ xl) {
  const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= ld) return;
  const double v = j < n ? x[j] : 0.0;
  const float h = float(v);
  xh[j] = h;
  xl[j] = float(v - double(h));
}

// W = double(hi) + double(lo): the FP64 working matrix from the double-float planes
__global__ void join_df_kernel(const float* __restrict__ hi, const float* __restrict__ lo, double* __restrict__ W,
                               int64_t total) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e < total) W[e] = double(hi[e]) + double(lo[e]);
}

constexpr int kDotBlocks = 120;
// Refinement stops at a componentwise backward error of 256 FP64 unit roundoffs: the residual is formed
// from the double-float planes of K (48 significant bits per entry), which by themselves put the
// measured backward error of an FP64 LU solution at roughly 50-100 unit roundoffs.
constexpr double kBwdFloor = 256.0 * 1.1102230246251565e-16;
// A restart cycle stops its inner iteration once the estimated residual has fallen by this factor, or earlier
// at the requested tolerance or at the reduction that brings the backward error to its floor (at N = 22,500
// the floor comes first and one cycle of 10 iterations converges; 1e-10 and 1e-14 here measured the same).
constexpr double kInnerReduction = 1e-6;

// partial[b * nv + i] = sum over block b's chunk of V_i . w
__global__ void __launch_bounds__(256) multi_dot_kernel(const double* __restrict__ V, int64_t ldv, int nv,
                                                        const double* __restrict__ w, int n,
                                                        double* __restrict__ partial) {
  __shared__ double red[8];
  const int chunk = int(ceil_div(n, gridDim.x));
  const int lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  for (int i = 0; i < nv; ++i) {
    double s = 0.0;
    for (int t = lo + threadIdx.x; t < hi; t += blockDim.x) s = fma(V[int64_t(i) * ldv + t], w[t], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int q = 0; q < 8; ++q) t += red[q];
      partial[blockIdx.x * nv + i] = t;
    }
    __syncthreads();
  }
}

__global__ void reduce_partials_kernel(const double* __restrict__ partial, int nblocks, int nv, double* __restrict__ h) {
  const int i = threadIdx.x;
  if (i >= nv) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += partial[b * nv + i];
  h[i] = s;
}

// w += sign * sum_i h_i V_i ; if out != null writes there instead of w (out = sign * sum_i h_i V_i)
__global__ void multi_axpy_kernel(const double* __restrict__ V, int64_t ldv, int nv, const double* __restrict__ h,
                                  double sign, double* __restrict__ w, double* __restrict__ out, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  double s = 0.0;
  for (int i = 0; i < nv; ++i) s = fma(h[i], V[int64_t(i) * ldv + t], s);
  if (out) out[t] = sign * s;
  else w[t] += sign * s;
}

__global__ void axpby_kernel(double* y, double a, const double* x, double b, int n,
                             const double* __restrict__ mul) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  double v = a * x[t] + b * y[t];
  y[t] = mul ? v * mul[t] : v;
}

__global__ void rhs_kernel(const double* __restrict__ q, int N, int n, const double* __restrict__ dr,
                           double* __restrict__ bs) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  bs[t] = (t < N ? q[t] : 0.0) * dr[t];
}

__global__ void abs_kernel(const double* __restrict__ x, double* __restrict__ y, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) y[t] = fabs(x[t]);
}

struct Carve {
  char* base;
  size_t off = 0;
  template <typename T>
  T* take(size_t count) {
    off = (off + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
    off += count * sizeof(T);
    return p;
  }
};

}  // namespace

void updes_set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
  (void)cudaGetLastError();  // the failure is reported here; later checks on this thread start clean
  std::lock_guard<std::mutex> lk(g_err_mu);
  char buf[512];
  snprintf(buf, sizeof buf, "%s: %s (%s:%d)", cudaGetErrorString(e), what, file, line);
  g_last_error = buf;
}

void updes_set_last_error_text(const std::string& text) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_last_error = text;
}

std::string updes_last_error_text() {
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_last_error;
}

extern "C" const char* updes_last_error(void) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  static thread_local std::string copy;
  copy = g_last_error;
  return copy.c_str();
}

extern "C" int updes_version(void) { return 100; }

extern "C" const char* updes_status_string(int status) {
  switch (status) {
    case UPDES_OK: return "ok";
    case UPDES_ERR_INVALID: return "invalid argument";
    case UPDES_ERR_CUDA: return "CUDA runtime error";
    case UPDES_ERR_SINGULAR: return "singular matrix (zero or non-finite pivot)";
    case UPDES_ERR_NOT_CONVERGED: return "iterative refinement did not converge";
    case UPDES_ERR_TIMEOUT: return "a bounded device-side wait timed out";
    case UPDES_ERR_UNSUPPORTED: return "unsupported by this build";
    case UPDES_ERR_WORKSPACE: return "workspace too small";
    case UPDES_ERR_TOO_LARGE: return "n exceeds UPDES_NOALLOC_MAX_N, the fixed scratch of updes_lu_solve_noalloc";
    default: return "unknown status";
  }
}

extern "C" int64_t updes_matrix_ld(int64_t n, int32_t elem_bytes) {
  (void)elem_bytes;
  return (n + 31) / 32 * 32;
}

// ---------------------------------------------------------------------------
// LU entry points
// ---------------------------------------------------------------------------
namespace {

struct LuWs {
  DeviceStatus* st;
  void* panel;
  size_t panel_bytes;
  int* sync;
  double* tmp;
  float* lo;  // lo plane of the double-float working matrix (FP32 precision, when owned here)
};

// lo_plane: reserve the n x ld FP32 lo plane (updes_lu_factor); updes_solve brings its own.
size_t lu_ws_layout(int n, int precision, char* base, LuWs* out, bool lo_plane = true) {
  Carve c{base};
  LuWs w;
  w.st = c.take<DeviceStatus>(1);
  w.panel_bytes = precision == UPDES_PREC_FP32 ? lu_df_workspace_bytes(n) : lu_panel_workspace_bytes(kLuNb);
  w.panel = c.take<char>(w.panel_bytes);
  w.sync = c.take<int>(ceil_div(n, 64) + 2);
  w.tmp = c.take<double>(n);
  w.lo = (precision == UPDES_PREC_FP32 && lo_plane) ? c.take<float>(size_t(n) * updes_matrix_ld(n, 4)) : nullptr;
  if (out) *out = w;
  return c.off + 256;
}

int read_status(DeviceStatus* st, cudaStream_t s, DeviceStatus* host) {
  UPDES_CUDA_TRY(cudaMemcpyAsync(host, st, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, s));
  UPDES_CUDA_TRY(cudaStreamSynchronize(s));
  return UPDES_OK;
}

// hi = float(v), lo = float(v - hi) with v = dr_i K_ij dc_j (scalings exact; dr, dc may be null)
// hi/lo planes of the scaled K (none when hi is null); with write_back the scaled FP64 entry also replaces
// K's (each thread reads and writes only its own entry, so K may be read and written in place; ldk == ld then).
__global__ void split_df_kernel(double* __restrict__ K, int64_t ldk, float* __restrict__ hi,
                                float* __restrict__ lo, int64_t ld, int n, const double* __restrict__ dr,
                                const double* __restrict__ dc, int write_back) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t i = e / ld, j = e % ld;
  if (i >= n) return;
  double v = 0.0;
  if (j < n) {
    v = K[i * ldk + j];
    if (dr) v *= dr[i];
    if (dc) v *= dc[j];
  }
  if (hi) {
    const float h = float(v);
    hi[i * ld + j] = h;
    lo[i * ld + j] = float(v - double(h));
  }
  if (write_back) K[i * ldk + j] = v;
}

int perm_core(int n, int32_t* piv, cudaStream_t s) {
  if (n > kMaxPermN) return UPDES_ERR_UNSUPPORTED;
  static std::atomic<unsigned long long> attr{0};
  if (int e = smem_opt_in((const void*)perm_from_piv_kernel, int(kMaxPermN * sizeof(int32_t)), attr)) return e;
  perm_from_piv_kernel<<<1, 1024, n * sizeof(int32_t), s>>>(piv, n, piv + n);
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

// Mixed LU of a double-float matrix already split into (hi = F, lo).
int factor_df_core(int n, float* hi, float* lo, int64_t ld, int32_t* piv, const LuWs& w, cudaStream_t s) {
  UPDES_CUDA_TRY(cudaMemsetAsync(w.st, 0, sizeof(DeviceStatus), s));
  int e = lu_factor_df(n, hi, lo, ld, piv, w.panel, w.panel_bytes, w.st, s);
  if (e) return e;
  return perm_core(n, piv, s);
}

int factor_core(int n, double* A, int64_t lda, int precision, void* F, int64_t ldf, int32_t* piv, const LuWs& w,
                cudaStream_t s) {
  if (precision == UPDES_PREC_FP32) {
    if (!w.lo || !F) return UPDES_ERR_INVALID;
    split_df_kernel<<<unsigned(ceil_div(int64_t(n) * ldf, 256)), 256, 0, s>>>(A, lda, static_cast<float*>(F), w.lo,
                                                                              ldf, n, nullptr, nullptr, 0);
    UPDES_LAUNCH_CHECK();
    return factor_df_core(n, static_cast<float*>(F), w.lo, ldf, piv, w, s);
  }
  UPDES_CUDA_TRY(cudaMemsetAsync(w.st, 0, sizeof(DeviceStatus), s));
  int e;
  {
    double* Fd = F ? static_cast<double*>(F) : A;
    if (Fd != A) {
      UPDES_CUDA_TRY(cudaMemcpy2DAsync(Fd, ldf * 8, A, lda * 8, size_t(n) * 8, n, cudaMemcpyDeviceToDevice, s));
      A = Fd;
      lda = ldf;
    }
    e = lu_factor_impl<double>(n, A, lda, A, lda, piv, w.panel, w.panel_bytes, w.st, s, nullptr);
  }
  if (e) return e;
  return perm_core(n, piv, s);
}

// x (contiguous, n) <- A^-1 x or A^-T x using the permutation in piv[n, 2n)
template <typename TF>
int solve_core(int n, const TF* F, int64_t ldf, const int32_t* piv, double* x, int trans, const LuWs& w,
               cudaStream_t s, const float* dinv = nullptr, float* xh = nullptr, float* xl = nullptr,
               const float* dinv128 = nullptr, unsigned long long* xtag = nullptr) {
  const int32_t* perm = piv + n;
  const unsigned g = unsigned(ceil_div(n, 256));
  if (!trans) {
    permute_kernel<<<g, 256, 0, s>>>(w.tmp, x, 1, 1, perm, n, 0);
    UPDES_LAUNCH_CHECK();
    int e = trsv_impl<TF>(n, F, ldf, w.tmp, 0, w.sync, w.st, s, dinv, xh, xl, dinv128, xtag);
    if (e) return e;
    e = trsv_impl<TF>(n, F, ldf, w.tmp, 1, w.sync, w.st, s, dinv, xh, xl, dinv128, xtag);
    if (e) return e;
    UPDES_CUDA_TRY(cudaMemcpyAsync(x, w.tmp, size_t(n) * 8, cudaMemcpyDeviceToDevice, s));
  } else {
    UPDES_CUDA_TRY(cudaMemcpyAsync(w.tmp, x, size_t(n) * 8, cudaMemcpyDeviceToDevice, s));
    int e = trsv_impl<TF>(n, F, ldf, w.tmp, 2, w.sync, w.st, s, dinv, xh, xl, dinv128, xtag);
    if (e) return e;
    e = trsv_impl<TF>(n, F, ldf, w.tmp, 3, w.sync, w.st, s, dinv, xh, xl, dinv128, xtag);
    if (e) return e;
    permute_kernel<<<g, 256, 0, s>>>(x, w.tmp, 1, 1, perm, n, 1);
    UPDES_LAUNCH_CHECK();
  }
  return UPDES_OK;
}

int solve_any(int n, const void* F, int64_t ldf, int precision, const int32_t* piv, double* x, int trans,
              const LuWs& w, cudaStream_t s) {
  if (precision == UPDES_PREC_FP64) return solve_core<double>(n, static_cast<const double*>(F), ldf, piv, x, trans, w, s);
  return solve_core<float>(n, static_cast<const float*>(F), ldf, piv, x, trans, w, s);
}

}  // namespace

extern "C" int updes_lu_workspace(int32_t n, int32_t precision, size_t* bytes) {
  if (n <= 0 || !bytes || (precision != UPDES_PREC_FP64 && precision != UPDES_PREC_FP32)) return UPDES_ERR_INVALID;
  *bytes = lu_ws_layout(n, precision, nullptr, nullptr);
  return UPDES_OK;
}

extern "C" int updes_lu_factor(int32_t n, double* A, int64_t lda, int32_t precision, void* F, int64_t ldf,
                               int32_t* piv, void* workspace, size_t workspace_bytes, int32_t* info, void* stream) {
  if (n <= 0 || !A || lda < n || !piv || !workspace) return UPDES_ERR_INVALID;
  if (precision != UPDES_PREC_FP64 && precision != UPDES_PREC_FP32) return UPDES_ERR_INVALID;
  if (precision == UPDES_PREC_FP32 && (!F || ldf < n || ldf != updes_matrix_ld(n, 4))) return UPDES_ERR_INVALID;
  if (precision == UPDES_PREC_FP64 && F && ldf < n) return UPDES_ERR_INVALID;
  if (workspace_bytes < lu_ws_layout(n, precision, nullptr, nullptr)) return UPDES_ERR_WORKSPACE;
  LuWs w;
  lu_ws_layout(n, precision, static_cast<char*>(workspace), &w);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int e = factor_core(n, A, lda, precision, F, ldf, piv, w, s);
  if (e) return e;
  DeviceStatus h;
  e = read_status(w.st, s, &h);
  if (e) return e;
  if (info) *info = h.lu_info;
  if (h.error) return h.error;
  return UPDES_OK;
}

extern "C" int updes_lu_solve(int32_t n, const void* F, int64_t ldf, int32_t precision, const int32_t* piv,
                              double* b, int32_t nrhs, int64_t ldb, int32_t trans, void* workspace,
                              size_t workspace_bytes, void* stream) {
  if (n <= 0 || !F || ldf < n || !piv || !b || nrhs <= 0 || ldb < nrhs || !workspace) return UPDES_ERR_INVALID;
  if (precision != UPDES_PREC_FP64 && precision != UPDES_PREC_FP32) return UPDES_ERR_INVALID;
  if (workspace_bytes < lu_ws_layout(n, precision, nullptr, nullptr) + size_t(n) * 8 + 256) return UPDES_ERR_WORKSPACE;
  LuWs w;
  size_t used = lu_ws_layout(n, precision, static_cast<char*>(workspace), &w);
  double* col = reinterpret_cast<double*>(static_cast<char*>(workspace) + ((used + 255) & ~size_t(255)));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  UPDES_CUDA_TRY(cudaMemsetAsync(w.st, 0, sizeof(DeviceStatus), s));
  for (int j = 0; j < nrhs; ++j) {
    double* bj = b + j;
    if (nrhs == 1) {
      int e = solve_any(n, F, ldf, precision, piv, bj, trans, w, s);
      if (e) return e;
      continue;
    }
    UPDES_CUDA_TRY(cudaMemcpy2DAsync(col, 8, bj, ldb * 8, 8, n, cudaMemcpyDeviceToDevice, s));
    int e = solve_any(n, F, ldf, precision, piv, col, trans, w, s);
    if (e) return e;
    UPDES_CUDA_TRY(cudaMemcpy2DAsync(bj, ldb * 8, col, 8, 8, n, cudaMemcpyDeviceToDevice, s));
  }
  DeviceStatus h;
  int e = read_status(w.st, s, &h);
  if (e) return e;
  return h.error;
}

extern "C" int updes_residual(int32_t n, const double* K, int64_t ldk, const double* x, const double* b, double* r,
                              int32_t trans, void* stream) {
  if (n <= 0 || !K || ldk < n || !x || !b || !r) return UPDES_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!trans) gemv_kernel<<<unsigned(ceil_div(int64_t(n) * 32, 256)), 256, 0, s>>>(K, ldk, n, x, b, nullptr, nullptr, 1.0, -1.0, r);
  else gemv_t_kernel<<<unsigned(ceil_div(n, 32)), 256, 0, s>>>(K, ldk, n, x, b, nullptr, nullptr, 1.0, -1.0, r);
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

// ---------------------------------------------------------------------------
// The full solve
// ---------------------------------------------------------------------------
namespace {

struct SolveWs {
  LuWs lu;
  double *W, *dr, *dc, *bs, *bsabs, *absr, *x, *r, *z, *wv, *V, *Z, *partial, *h;
  double* evp;  // per-tile partial sums of the symmetric value evaluation
  float *Khi, *Klo;  // equilibrated K as double-float planes (kept for the refinement's residuals)
  float *xh, *xl;    // FP32 planes of the vector a GEMV multiplies
  float* F32;  // hi plane = FP32 factors
  float* Wlo;
  float* dinv;     // inverted 64 x 64 diagonal blocks of the FP32 factors (double-float planes)
  float* dinv128;  // the same for 128 x 128 blocks
  unsigned long long* xtag;  // tagged hand-off words of the 128-row triangular solves (2n)
  int32_t* piv;
  int32_t* state;  // [0] n of the factored system, [1] precision of its factors, [2] 1 when valid
  int64_t ld;
};

size_t solve_ws_layout(int n, const updes_solve_opts& o, char* base, SolveWs* out) {
  SolveWs w;
  const int64_t ld = updes_matrix_ld(n, 8);
  Carve c{base};
  const size_t lub = lu_ws_layout(n, o.precision, nullptr, nullptr, false);
  char* lubase = c.take<char>(lub);
  if (base) lu_ws_layout(n, o.precision, lubase, &w.lu, false);
  w.ld = ld;
  w.Khi = c.take<float>(2 * size_t(n) * ld);
  w.Klo = w.Khi + size_t(n) * ld;
  w.xh = c.take<float>(ld);
  w.xl = c.take<float>(ld);
  w.W = c.take<double>(size_t(n) * ld);  // FP64 working matrix, or the hi and lo FP32 planes
  w.F32 = reinterpret_cast<float*>(w.W);
  w.Wlo = w.F32 + size_t(n) * ld;
  w.piv = c.take<int32_t>(2 * size_t(n));
  w.state = c.take<int32_t>(64);
  w.dinv = c.take<float>(diag_inverse_bytes(n) / sizeof(float));
  w.dinv128 = c.take<float>(diag_inverse128_bytes(n) / sizeof(float));
  w.evp = c.take<double>(eval_values_sym_bytes(n) / sizeof(double));
  w.dr = c.take<double>(n);
  w.dc = c.take<double>(n);
  w.bs = c.take<double>(n);
  w.bsabs = c.take<double>(n);
  w.absr = c.take<double>(n);
  w.x = c.take<double>(n);
  w.r = c.take<double>(n);
  w.z = c.take<double>(n);
  w.wv = c.take<double>(n);
  const int m = o.restart > 0 ? o.restart : 1;
  w.V = c.take<double>(size_t(m + 1) * n);
  w.partial = c.take<double>(size_t(kDotBlocks) * (m + 2));
  w.h = c.take<double>(m + 2);
  w.xtag = c.take<unsigned long long>(2 * size_t(n));
  w.Z = c.take<double>(size_t(m) * n);  // preconditioned basis vectors M^-1 V_j of a restart cycle
  if (out) *out = w;
  return c.off + 256;
}

updes_solve_opts normalise(const updes_solve_opts* o) {
  updes_solve_opts d;
  d.precision = UPDES_PREC_FP32;
  d.max_iters = 200;
  d.restart = 40;
  d.fallback_fp64 = 1;
  d.tol = 1e-13;
  if (o) {
    d = *o;
    if (d.max_iters <= 0) d.max_iters = 200;
    if (d.restart <= 0) d.restart = 40;
    if (d.restart > 200) d.restart = 200;
    if (!(d.tol > 0)) d.tol = 1e-13;
  }
  return d;
}

// h[0..nv) = V[0..nv)^T w (device), then copied to host
int multi_dot(const double* V, int64_t ldv, int nv, const double* w, int n, double* partial, double* h_dev,
              double* h_host, cudaStream_t s) {
  multi_dot_kernel<<<kDotBlocks, 256, 0, s>>>(V, ldv, nv, w, n, partial);
  UPDES_LAUNCH_CHECK();
  reduce_partials_kernel<<<1, 256, 0, s>>>(partial, kDotBlocks, nv, h_dev);
  UPDES_LAUNCH_CHECK();
  if (h_host) {
    UPDES_CUDA_TRY(cudaMemcpyAsync(h_host, h_dev, nv * sizeof(double), cudaMemcpyDeviceToHost, s));
    UPDES_CUDA_TRY(cudaStreamSynchronize(s));
  }
  return UPDES_OK;
}

struct Timer {
  cudaEvent_t a, b;
  cudaStream_t s;
  bool ok;
  explicit Timer(cudaStream_t st) : s(st) {
    ok = cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess;
    if (ok) cudaEventRecord(a, s);
  }
  double stop() {
    if (!ok) return 0.0;
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    ok = false;
    return ms;
  }
  ~Timer() {
    if (ok) {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  }
};

// Ks z = dr .* (K (dc .* z))
// (trans: Ks^T z = dc .* (K^T (dr .* z)))
int gemv_scaled(const SolveWs& w, int n, const double* z, double ksign, double* out, double* absout,
                cudaStream_t s, bool trans) {
  StatScope sc(kStatGemv, s, 2.0 * n * n, 8.0 * n * double(w.ld));
  split_vec_kernel<<<unsigned(ceil_div(w.ld, 256)), 256, 0, s>>>(z, n, w.ld, w.xh, w.xl);
  UPDES_LAUNCH_CHECK();
  if (trans)
    gemv_t_df_kernel<<<unsigned(ceil_div(n, 32)), 256, 0, s>>>(w.Khi, w.Klo, w.ld, n, w.xh, w.xl, ksign, out, absout);
  else
    gemv_df_kernel<<<unsigned(ceil_div(int64_t(n) * 32, 256)), 256, 0, s>>>(w.Khi, w.Klo, w.ld, n, w.xh, w.xl, ksign,
                                                                              out, absout);
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

int apply_K(const SolveWs& w, int n, const double* z, double* out, cudaStream_t s, bool trans = false) {
  return gemv_scaled(w, n, z, 1.0, out, nullptr, s, trans);
}

// out = bs - Ks x; also returns (on the host) the componentwise backward error
// max_i |out_i| / (|Ks| |x| + |bs|)_i.
int residual_scaled(const SolveWs& w, int n, const double* x, double* out, double* bwd, cudaStream_t s,
                    bool trans = false) {
  int e0 = gemv_scaled(w, n, x, -1.0, out, w.absr, s, trans);
  if (e0) return e0;
  axpby_kernel<<<unsigned(ceil_div(n, 256)), 256, 0, s>>>(out, 1.0, w.bs, 1.0, n, nullptr);
  UPDES_LAUNCH_CHECK();
  axpby_kernel<<<unsigned(ceil_div(n, 256)), 256, 0, s>>>(w.absr, 1.0, w.bsabs, 1.0, n, nullptr);
  UPDES_LAUNCH_CHECK();
  bwd_partial_kernel<<<kDotBlocks, 256, 0, s>>>(out, w.absr, n, w.partial);
  UPDES_LAUNCH_CHECK();
  std::vector<double> part(kDotBlocks);
  UPDES_CUDA_TRY(cudaMemcpyAsync(part.data(), w.partial, kDotBlocks * sizeof(double), cudaMemcpyDeviceToHost, s));
  UPDES_CUDA_TRY(cudaStreamSynchronize(s));
  double m = 0.0;
  for (double v : part) m = std::fmax(m, v);
  *bwd = m;
  return UPDES_OK;
}

int precond(const SolveWs& w, int n, int precision, double* x, cudaStream_t s, bool trans = false) {
  if (precision == UPDES_PREC_FP64) return solve_core<double>(n, w.W, w.ld, w.piv, x, trans ? 1 : 0, w.lu, s);
  return solve_core<float>(n, w.F32, w.ld, w.piv, x, trans ? 1 : 0, w.lu, s, w.dinv, w.xh, w.xl, w.dinv128,
                           w.xtag);
}

[[maybe_unused]] double host_norm(const std::vector<double>& v) {
  double s = 0;
  for (double a : v) s += a * a;
  return std::sqrt(s);
}

// UPDES_TRACE=1 in the environment prints the refinement history to stderr.
bool trace_on() {
  static const bool on = [] {
    const char* v = std::getenv("UPDES_TRACE");
    return v && v[0] == '1';
  }();
  return on;
}

// Restarted, right-preconditioned GMRES on Ks x = bs starting from w.x, in the flexible form: each cycle keeps
// its preconditioned vectors, so that its update x += M^-1 V y is Z y without another preconditioner solve.
int gmres(const SolveWs& w, int n, int precision, const updes_solve_opts& o, updes_solve_info* info,
          cudaStream_t s, bool trans = false) {
  const int m = o.restart;
  const unsigned g = unsigned(ceil_div(n, 256));
  std::vector<double> H(size_t(m + 1) * m), cs(m), sn(m), gv(m + 1), hcol(m + 2);
  double bnorm2;
  int e = multi_dot(w.bs, n, 1, w.bs, n, w.partial, w.h, &bnorm2, s);
  if (e) return e;
  const double bnorm = std::sqrt(bnorm2);
  int total = 0, stalls = 0;
  double last_beta = INFINITY;
  for (;;) {
    double bwd;
    if ((e = residual_scaled(w, n, w.x, w.r, &bwd, s, trans))) return e;
    double beta2;
    if ((e = multi_dot(w.r, n, 1, w.r, n, w.partial, w.h, &beta2, s))) return e;
    const double beta = std::sqrt(beta2);
    info->rel_residual = bnorm > 0 ? beta / bnorm : beta;
    info->backward_error = bwd;
    if (trace_on())
      std::fprintf(stderr, "[updes gmres n=%d prec=%d trans=%d] iters=%d rel_residual=%.3e backward_error=%.3e\n", n,
                   precision, int(trans), total, info->rel_residual, bwd);
    if (!(beta == beta)) return UPDES_ERR_NOT_CONVERGED;
    if (beta <= o.tol * bnorm || bwd <= kBwdFloor) {
      info->converged = 1;
      break;
    }
    if (total >= o.max_iters) break;
    if (beta > 0.5 * last_beta) {
      if (++stalls >= 2) break;  // two restart cycles in a row without halving the residual
    } else {
      stalls = 0;
    }
    last_beta = beta;
    // this cycle stops at whichever comes first: the requested tolerance, the reduction one cycle can
    // deliver, or (with a factor 2 to spare) the reduction that brings the backward error to its floor (the
    // ratio backward error / residual norm changes little between cycles)
    const double target = std::max(o.tol * bnorm, beta * std::max(kInnerReduction, 0.5 * kBwdFloor / bwd));
    // V0 = r / beta
    axpby_kernel<<<g, 256, 0, s>>>(w.V, 1.0 / beta, w.r, 0.0, n, nullptr);
    UPDES_LAUNCH_CHECK();
    std::fill(gv.begin(), gv.end(), 0.0);
    gv[0] = beta;
    int j = 0;
    for (; j < m && total < o.max_iters; ++j, ++total) {
      // z_j = M^-1 v_j is kept (flexible GMRES form): the cycle's update is then Z y, with no further solve
      double* vj = w.V + size_t(j) * n;
      double* zj = w.Z + size_t(j) * n;
      UPDES_CUDA_TRY(cudaMemcpyAsync(zj, vj, size_t(n) * 8, cudaMemcpyDeviceToDevice, s));
      if ((e = precond(w, n, precision, zj, s, trans))) return e;
      if ((e = apply_K(w, n, zj, w.wv, s, trans))) return e;
      // CGS2
      std::fill(hcol.begin(), hcol.end(), 0.0);
      for (int pass = 0; pass < 2; ++pass) {
        std::vector<double> hh(j + 1);
        if ((e = multi_dot(w.V, n, j + 1, w.wv, n, w.partial, w.h, hh.data(), s))) return e;
        multi_axpy_kernel<<<g, 256, 0, s>>>(w.V, n, j + 1, w.h, -1.0, w.wv, nullptr, n);
        UPDES_LAUNCH_CHECK();
        for (int i = 0; i <= j; ++i) hcol[i] += hh[i];
      }
      double hn2;
      if ((e = multi_dot(w.wv, n, 1, w.wv, n, w.partial, w.h, &hn2, s))) return e;
      const double hn = std::sqrt(hn2);
      hcol[j + 1] = hn;
      if (hn > 0) {
        axpby_kernel<<<g, 256, 0, s>>>(w.V + size_t(j + 1) * n, 1.0 / hn, w.wv, 0.0, n, nullptr);
        UPDES_LAUNCH_CHECK();
      }
      // Givens
      for (int i = 0; i < j; ++i) {
        const double t = cs[i] * hcol[i] + sn[i] * hcol[i + 1];
        hcol[i + 1] = -sn[i] * hcol[i] + cs[i] * hcol[i + 1];
        hcol[i] = t;
      }
      const double d = std::hypot(hcol[j], hcol[j + 1]);
      cs[j] = d > 0 ? hcol[j] / d : 1.0;
      sn[j] = d > 0 ? hcol[j + 1] / d : 0.0;
      hcol[j] = d;
      hcol[j + 1] = 0.0;
      gv[j + 1] = -sn[j] * gv[j];
      gv[j] = cs[j] * gv[j];
      for (int i = 0; i <= j; ++i) H[size_t(i) * m + j] = hcol[i];
      if (trace_on())
        std::fprintf(stderr, "[updes gmres]   j=%d estimate=%.3e h_next=%.3e\n", j, std::fabs(gv[j + 1]) / bnorm, hn);
      if (std::fabs(gv[j + 1]) <= target || hn == 0.0) {
        ++j;
        ++total;
        break;
      }
    }
    // y = R^-1 g
    std::vector<double> y(j);
    for (int i = j - 1; i >= 0; --i) {
      double t = gv[i];
      for (int k = i + 1; k < j; ++k) t -= H[size_t(i) * m + k] * y[k];
      y[i] = H[size_t(i) * m + i] != 0 ? t / H[size_t(i) * m + i] : 0.0;
    }
    if (j > 0) {
      UPDES_CUDA_TRY(cudaMemcpyAsync(w.h, y.data(), j * sizeof(double), cudaMemcpyHostToDevice, s));
      multi_axpy_kernel<<<g, 256, 0, s>>>(w.Z, n, j, w.h, 1.0, nullptr, w.z, n);
      UPDES_LAUNCH_CHECK();
      axpby_kernel<<<g, 256, 0, s>>>(w.x, 1.0, w.z, 1.0, n, nullptr);
      UPDES_LAUNCH_CHECK();
      UPDES_CUDA_TRY(cudaStreamSynchronize(s));
    }
  }
  if (precision == UPDES_PREC_FP32) info->iters = total;
  return UPDES_OK;
}

}  // namespace

extern "C" int updes_solve_workspace(const updes_problem* p, const updes_solve_opts* opts, size_t* bytes) {
  if (updes_check_problem(p) || !bytes) return UPDES_ERR_INVALID;
  const updes_solve_opts o = normalise(opts);
  updes_solve_opts o64 = o;
  o64.precision = UPDES_PREC_FP32;  // the FP64 fallback fits in the same layout
  *bytes = solve_ws_layout(p->N + p->M, o64, nullptr, nullptr);
  return UPDES_OK;
}

namespace {

// Factors of the equilibrated K (double-float planes) at `precision`; records the factored state.
// planes_ready: the working copy already holds the equilibrated K, written by the assembly: for FP32 factors
// the planes F32 and Wlo (double-float assembly), for FP64 factors the FP64 matrix W.
int factor_stage(const SolveWs& w, int n, int precision, updes_solve_info* info, cudaStream_t s,
                 bool planes_ready = false) {
  Timer t(s);
  int e;
  UPDES_CUDA_TRY(cudaMemsetAsync(w.state, 0, 4 * sizeof(int32_t), s));  // invalid until the factors are complete
  const int64_t total = int64_t(n) * w.ld;
  if (precision == UPDES_PREC_FP64) {
    if (!planes_ready) {  // a fallback after the FP32 attempt: W was overwritten, K is rebuilt from its planes
      join_df_kernel<<<unsigned(ceil_div(total, 256)), 256, 0, s>>>(w.Khi, w.Klo, w.W, total);
      UPDES_LAUNCH_CHECK();
    }
    e = factor_core(n, w.W, w.ld, precision, nullptr, w.ld, w.piv, w.lu, s);
  } else {
    if (!planes_ready) {
      UPDES_CUDA_TRY(cudaMemcpyAsync(w.F32, w.Khi, size_t(total) * 4, cudaMemcpyDeviceToDevice, s));
      UPDES_CUDA_TRY(cudaMemcpyAsync(w.Wlo, w.Klo, size_t(total) * 4, cudaMemcpyDeviceToDevice, s));
    }
    e = factor_df_core(n, w.F32, w.Wlo, w.ld, w.piv, w.lu, s);
    if (!e) e = diag_inverse(n, w.F32, w.ld, w.dinv, s);
    if (!e) e = diag_inverse128(n, w.F32, w.ld, w.dinv, w.dinv128, s);
  }
  if (e) return e;
  DeviceStatus h;
  if ((e = read_status(w.lu.st, s, &h))) return e;
  if (h.error) return h.error;
  info->lu_info = h.lu_info;
  info->t_factor_ms += t.stop();
  // {n, precision, valid, generation}: the generation tells derived copies of these factors (the batched
  // solves' double-float planes) that they are stale after a refactorisation
  static std::atomic<int32_t> generation{0};
  const int32_t st4[4] = {n, precision, 1, generation.fetch_add(1) + 1};
  UPDES_CUDA_TRY(cudaMemcpyAsync(w.state, st4, sizeof st4, cudaMemcpyHostToDevice, s));
  UPDES_CUDA_TRY(cudaStreamSynchronize(s));
  return UPDES_OK;
}

int read_state(const SolveWs& w, int n, int* precision, cudaStream_t s) {
  int32_t st3[3] = {0, 0, 0};
  UPDES_CUDA_TRY(cudaMemcpyAsync(st3, w.state, sizeof st3, cudaMemcpyDeviceToHost, s));
  UPDES_CUDA_TRY(cudaStreamSynchronize(s));
  if (st3[2] != 1 || st3[0] != n) return UPDES_ERR_INVALID;
  *precision = st3[1];
  return UPDES_OK;
}

// K of a polyharmonic system in double-float (updes_assemble_df) with the power-of-two equilibration of the
// FP64 path: row maxima from the assembly, column maxima of the row-scaled hi plane, both planes scaled in
// place.  UNSUPPORTED when an entry falls outside the range in which double-float keeps its 48 bits (the
// caller then assembles in FP64).
int assemble_df_stage(const updes_problem* p, const SolveWs& w, int n, cudaStream_t s) {
  unsigned* rowmax = reinterpret_cast<unsigned*>(w.dc);  // float bits, then the column maxima, then dc
  int32_t* flag = reinterpret_cast<int32_t*>(w.r);       // free until the refinement
  UPDES_CUDA_TRY(cudaMemsetAsync(rowmax, 0, size_t(n) * sizeof(unsigned), s));
  UPDES_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int32_t), s));
  // the FP64 working matrix is free until the factorisation: the assembly's row records and coordinates
  int e = updes_assemble_df(p, w.Khi, w.Klo, w.ld, rowmax, flag, w.W, size_t(n) * w.ld * sizeof(double), s);
  if (e) return e;
  row_scale_bits_kernel<<<unsigned(ceil_div(n, 256)), 256, 0, s>>>(rowmax, n, w.dr);
  UPDES_LAUNCH_CHECK();
  UPDES_CUDA_TRY(cudaMemsetAsync(w.dc, 0, size_t(n) * sizeof(double), s));
  col_max_f32_kernel<<<dim3(unsigned(ceil_div(n, 256)), kColScaleChunks), 256, 0, s>>>(
      w.Khi, w.ld, n, w.dr, reinterpret_cast<unsigned long long*>(w.dc));
  UPDES_LAUNCH_CHECK();
  col_scale_kernel<<<unsigned(ceil_div(n, 256)), 256, 0, s>>>(n, w.dc);
  UPDES_LAUNCH_CHECK();
  {
    StatScope sc(kStatOther, s, 0.0, double(n) * n * 24.0);
    // the factorisation's working copy (F32, Wlo) in the same pass: the assembly's scratch there is done with
    scale_planes_kernel<<<dim3(unsigned(ceil_div(n, 1024)), unsigned(std::min(n, 4096))), 256, 0, s>>>(
        w.Khi, w.Klo, w.ld, n, w.dr, w.dc, w.F32, w.Wlo);
    UPDES_LAUNCH_CHECK();
  }
  int32_t hflag = 0;
  UPDES_CUDA_TRY(cudaMemcpyAsync(&hflag, flag, sizeof hflag, cudaMemcpyDeviceToHost, s));
  UPDES_CUDA_TRY(cudaStreamSynchronize(s));
  return hflag ? UPDES_ERR_UNSUPPORTED : UPDES_OK;
}

// Assemble K and its power-of-two equilibration into the double-float planes: in double-float arithmetic for
// a polyharmonic system factored in FP32, else in FP64.
// *planes_ready: the factorisation's working copy holds the equilibrated K as well (the planes of a
// double-float assembly, or the FP64 K of an FP64 solve).
int assemble_stage(const updes_problem* p, const SolveWs& w, int n, int precision, updes_solve_info* info,
                   cudaStream_t s, bool* planes_ready) {
  Timer t(s);
  int e;
  *planes_ready = false;
  // UPDES_DF_ASSEMBLY=0 assembles every system in FP64
  static const bool df_assembly = [] {
    const char* v = std::getenv("UPDES_DF_ASSEMBLY");
    return !(v && v[0] == '0');
  }();
  if (df_assembly && precision == UPDES_PREC_FP32 && p->rbf == UPDES_RBF_POLYHARMONIC) {
    e = assemble_df_stage(p, w, n, s);
    if (e != UPDES_ERR_UNSUPPORTED) {
      if (e) return e;
      *planes_ready = true;
      info->t_assemble_ms += t.stop();
      return UPDES_OK;
    }
  }
  if ((e = updes_assemble(p, w.W, w.ld, nullptr, 0, s))) return e;  // FP64 K, staged in the working buffer
  row_scale_kernel<<<unsigned(ceil_div(int64_t(n) * 32, 256)), 256, 0, s>>>(w.W, w.ld, n, w.dr);
  UPDES_LAUNCH_CHECK();
  UPDES_CUDA_TRY(cudaMemsetAsync(w.dc, 0, size_t(n) * sizeof(double), s));
  col_max_kernel<<<dim3(unsigned(ceil_div(n, 256)), kColScaleChunks), 256, 0, s>>>(
      w.W, w.ld, n, w.dr, reinterpret_cast<unsigned long long*>(w.dc));
  UPDES_LAUNCH_CHECK();
  col_scale_kernel<<<unsigned(ceil_div(n, 256)), 256, 0, s>>>(n, w.dc);
  UPDES_LAUNCH_CHECK();
  // the FP64 path factors the equilibrated FP64 K itself (written back in place), not the 48-bit sum of its
  // planes: on systems near the FP64 limit (r^5 at N = 10,000) the planes' rounding alone would be 32x the
  // FP64 rounding of K
  const int fp64 = precision == UPDES_PREC_FP64;
  split_df_kernel<<<unsigned(ceil_div(int64_t(n) * w.ld, 256)), 256, 0, s>>>(w.W, w.ld, w.Khi, w.Klo, w.ld, n, w.dr,
                                                                             w.dc, fp64);
  UPDES_LAUNCH_CHECK();
  *planes_ready = fp64 != 0;  // for the FP64 factorisation: W holds the equilibrated K
  info->t_assemble_ms += t.stop();
  return UPDES_OK;
}

// One right-hand side against the stored factors: refinement, FP64 fallback, coeffs and vals.
int solve_stage(const updes_problem* p, const SolveWs& w, int n, const double* q, int64_t qstride, double* coeffs,
                int64_t cstride, double* vals, int64_t vstride, const updes_solve_opts& o, updes_solve_info* info,
                cudaStream_t s) {
  const unsigned g = unsigned(ceil_div(n, 256));
  int precision, e;
  if ((e = read_state(w, n, &precision, s))) return e;
  for (int attempt = 0; attempt < 2; ++attempt) {
    Timer t(s);
    if (qstride == 1) {
      rhs_kernel<<<g, 256, 0, s>>>(q, p->N, n, w.dr, w.bs);
      UPDES_LAUNCH_CHECK();
    } else {
      UPDES_CUDA_TRY(cudaMemsetAsync(w.r, 0, size_t(n) * 8, s));
      UPDES_CUDA_TRY(cudaMemcpy2DAsync(w.r, 8, q, qstride * 8, 8, p->N, cudaMemcpyDeviceToDevice, s));
      rhs_kernel<<<g, 256, 0, s>>>(w.r, p->N, n, w.dr, w.bs);
      UPDES_LAUNCH_CHECK();
    }
    abs_kernel<<<g, 256, 0, s>>>(w.bs, w.bsabs, n);
    UPDES_LAUNCH_CHECK();
    UPDES_CUDA_TRY(cudaMemcpyAsync(w.x, w.bs, size_t(n) * 8, cudaMemcpyDeviceToDevice, s));
    if ((e = precond(w, n, precision, w.x, s))) return e;
    updes_solve_opts oi = o;
    if (precision == UPDES_PREC_FP64) oi.max_iters = 0;  // plain FP64 LU: report the residual only
    if ((e = gmres(w, n, precision, oi, info, s))) return e;
    DeviceStatus h;
    if ((e = read_status(w.lu.st, s, &h))) return e;
    if (h.error) return h.error;
    info->t_refine_ms += t.stop();
    if (precision == UPDES_PREC_FP64) {
      info->converged = 1;
      break;
    }
    if (info->converged || !o.fallback_fp64) break;
    precision = UPDES_PREC_FP64;
    info->fell_back = 1;
    // the FP32 attempt overwrote the working matrix: K is assembled again in FP64 and scaled in place with the
    // same powers of two, so the fallback factors the FP64 K (not the 48-bit sum of its planes); the planes,
    // the residuals' operator, stay as they are
    if ((e = updes_assemble(p, w.W, w.ld, nullptr, 0, s))) return e;
    split_df_kernel<<<unsigned(ceil_div(int64_t(n) * w.ld, 256)), 256, 0, s>>>(w.W, w.ld, nullptr, nullptr, w.ld, n,
                                                                               w.dr, w.dc, 1);
    UPDES_LAUNCH_CHECK();
    if ((e = factor_stage(w, n, precision, info, s, true))) return e;
  }
  Timer t(s);
  // the values of a mixed-precision solve in double-float (polyharmonic kernels; UPDES_DF_EVAL=0: FP64)
  static const bool df_eval_on = [] {
    const char* v = std::getenv("UPDES_DF_EVAL");
    return !(v && v[0] == '0');
  }();
  const bool df_eval = df_eval_on && precision == UPDES_PREC_FP32;
  axpby_kernel<<<g, 256, 0, s>>>(w.x, 1.0, w.x, 0.0, n, w.dc);  // coeffs = dc .* x
  UPDES_LAUNCH_CHECK();
  if (cstride == 1) {
    UPDES_CUDA_TRY(cudaMemcpyAsync(coeffs, w.x, size_t(n) * 8, cudaMemcpyDeviceToDevice, s));
    if (vals && vstride == 1 && (e = eval_values_sym(p, coeffs, vals, w.evp, s, df_eval))) return e;
  } else {
    UPDES_CUDA_TRY(cudaMemcpy2DAsync(coeffs, cstride * 8, w.x, 8, 8, n, cudaMemcpyDeviceToDevice, s));
  }
  if (vals && (cstride != 1 || vstride != 1)) {
    if ((e = eval_values_sym(p, w.x, w.wv, w.evp, s, df_eval))) return e;
    UPDES_CUDA_TRY(cudaMemcpy2DAsync(vals, vstride * 8, w.wv, 8, 8, p->N, cudaMemcpyDeviceToDevice, s));
  }
  info->t_eval_ms += t.stop();
  return UPDES_OK;
}

int solve_setup(const updes_problem* p, const updes_solve_opts* opts, void* workspace, size_t workspace_bytes,
                SolveWs* w, updes_solve_opts* o) {
  if (updes_check_problem(p) || !workspace) return UPDES_ERR_INVALID;
  *o = normalise(opts);
  if (o->precision != UPDES_PREC_FP64 && o->precision != UPDES_PREC_FP32) return UPDES_ERR_INVALID;
  const int n = p->N + p->M;
  updes_solve_opts olay = *o;
  olay.precision = UPDES_PREC_FP32;
  if (workspace_bytes < solve_ws_layout(n, olay, nullptr, nullptr)) return UPDES_ERR_WORKSPACE;
  solve_ws_layout(n, olay, static_cast<char*>(workspace), w);
  return UPDES_OK;
}

}  // namespace

extern "C" int updes_factor(const updes_problem* p, const updes_solve_opts* opts, updes_solve_info* info,
                            void* workspace, size_t workspace_bytes, void* stream) {
  SolveWs w;
  updes_solve_opts o;
  int e = solve_setup(p, opts, workspace, workspace_bytes, &w, &o);
  if (e) return e;
  updes_solve_info dummy;
  if (!info) info = &dummy;
  std::memset(info, 0, sizeof *info);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int n = p->N + p->M;
  bool planes_ready = false;
  if ((e = assemble_stage(p, w, n, o.precision, info, s, &planes_ready))) return e;
  if ((e = factor_stage(w, n, o.precision, info, s, planes_ready))) return e;
  return info->lu_info ? UPDES_ERR_SINGULAR : UPDES_OK;
}

extern "C" int updes_solve_factored(const updes_problem* p, int32_t nrhs, const double* Q, int64_t ldq,
                                    double* coeffs, int64_t ldc, double* vals, int64_t ldv,
                                    const updes_solve_opts* opts, updes_solve_info* info, void* workspace,
                                    size_t workspace_bytes, void* stream) {
  SolveWs w;
  updes_solve_opts o;
  int e = solve_setup(p, opts, workspace, workspace_bytes, &w, &o);
  if (e) return e;
  if (nrhs <= 0 || !Q || !coeffs || ldq < nrhs || ldc < nrhs || (vals && ldv < nrhs)) return UPDES_ERR_INVALID;
  updes_solve_info dummy;
  if (!info) info = &dummy;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int n = p->N + p->M;
  updes_solve_info agg;
  std::memset(&agg, 0, sizeof agg);
  agg.converged = 1;
  for (int j = 0; j < nrhs; ++j) {
    updes_solve_info one;
    std::memset(&one, 0, sizeof one);
    if ((e = solve_stage(p, w, n, Q + j, ldq, coeffs + j, ldc, vals ? vals + j : nullptr, ldv, o, &one, s))) return e;
    agg.iters += one.iters;
    agg.fell_back |= one.fell_back;
    agg.lu_info = one.lu_info ? one.lu_info : agg.lu_info;
    agg.converged &= one.converged;
    agg.rel_residual = std::fmax(agg.rel_residual, one.rel_residual);
    agg.backward_error = std::fmax(agg.backward_error, one.backward_error);
    agg.t_factor_ms += one.t_factor_ms;
    agg.t_refine_ms += one.t_refine_ms;
    agg.t_eval_ms += one.t_eval_ms;
  }
  *info = agg;
  return agg.converged ? UPDES_OK : UPDES_ERR_NOT_CONVERGED;
}

extern "C" int updes_solve(const updes_problem* p, const double* q, double* coeffs, double* vals,
                           const updes_solve_opts* opts, updes_solve_info* info, void* workspace,
                           size_t workspace_bytes, void* stream) {
  SolveWs w;
  updes_solve_opts o;
  int e = solve_setup(p, opts, workspace, workspace_bytes, &w, &o);
  if (e) return e;
  if (!q || !coeffs) return UPDES_ERR_INVALID;
  updes_solve_info dummy;
  if (!info) info = &dummy;
  std::memset(info, 0, sizeof *info);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int n = p->N + p->M;
  bool planes_ready = false;
  if ((e = assemble_stage(p, w, n, o.precision, info, s, &planes_ready))) return e;
  if ((e = factor_stage(w, n, o.precision, info, s, planes_ready))) return e;
  if ((e = solve_stage(p, w, n, q, 1, coeffs, 1, vals, 1, o, info, s))) return e;
  if (info->lu_info) return UPDES_ERR_SINGULAR;
  if (!info->converged) return UPDES_ERR_NOT_CONVERGED;
  return UPDES_OK;
}

// ---------------------------------------------------------------------------
// Triangular solves with a fixed, library-owned scratch (no allocation at all)
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoallocSyncOff = 256;                                   // after the status word
constexpr size_t kNoallocVecOff = 2304;                                   // after (n/64 + 2) flags
constexpr size_t kNoallocBytes = kNoallocVecOff + 2 * size_t(UPDES_NOALLOC_MAX_N) * sizeof(double);
static_assert(kNoallocVecOff - kNoallocSyncOff >= sizeof(int) * (UPDES_NOALLOC_MAX_N / 64 + 2), "flag region");

// The only scratch of updes_lu_solve_noalloc, shared by all its calls on a device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

std::mutex g_noalloc_mu;
constexpr int kMaxDevices = 64;
void* g_noalloc_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once per device, by the first call
// there).  Devices with ordinal 64 or more are not supported; a lookup that fails while `s` is being captured
// says so, since that first call has to be made outside capture.
int noalloc_scratch(void** out, cudaStream_t s) {
  int dev = 0;
  UPDES_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    updes_set_last_cuda_error(cudaErrorInvalidDevice, "updes_lu_solve_noalloc supports device ordinals 0..63",
                              __FILE__, __LINE__);
    return UPDES_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      const bool capturing = cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
      updes_set_last_cuda_error(e, capturing ? "cudaGetSymbolAddress(g_noalloc_scratch) during stream capture: make "
                                               "the first updes_lu_solve_noalloc call on a device before any capture"
                                             : "cudaGetSymbolAddress(g_noalloc_scratch)",
                                __FILE__, __LINE__);
      return UPDES_ERR_CUDA;
    }
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return UPDES_OK;
}

}  // namespace

extern "C" int updes_lu_solve_noalloc(int32_t n, const void* F, int64_t ldf, int32_t precision, const int32_t* piv,
                                      double* b, int32_t nrhs, int64_t ldb, int32_t trans, void* stream) {
  if (n <= 0 || !F || ldf < n || !piv || !b || nrhs <= 0 || ldb < nrhs) return UPDES_ERR_INVALID;
  if (precision != UPDES_PREC_FP64 && precision != UPDES_PREC_FP32) return UPDES_ERR_INVALID;
  if (n > UPDES_NOALLOC_MAX_N) return UPDES_ERR_TOO_LARGE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void* base = nullptr;
  int e = noalloc_scratch(&base, s);
  if (e) return e;
  char* c = static_cast<char*>(base);
  LuWs w{};
  w.st = reinterpret_cast<DeviceStatus*>(c);
  w.sync = reinterpret_cast<int*>(c + kNoallocSyncOff);
  w.tmp = reinterpret_cast<double*>(c + kNoallocVecOff);
  double* col = w.tmp + UPDES_NOALLOC_MAX_N;
  UPDES_CUDA_TRY(cudaMemsetAsync(w.st, 0, sizeof(DeviceStatus), s));  // the flags are cleared by each solve
  for (int j = 0; j < nrhs; ++j) {
    double* bj = b + j;
    if (nrhs == 1) {
      if ((e = solve_any(n, F, ldf, precision, piv, bj, trans, w, s))) return e;
      continue;
    }
    UPDES_CUDA_TRY(cudaMemcpy2DAsync(col, 8, bj, ldb * 8, 8, n, cudaMemcpyDeviceToDevice, s));
    if ((e = solve_any(n, F, ldf, precision, piv, col, trans, w, s))) return e;
    UPDES_CUDA_TRY(cudaMemcpy2DAsync(bj, ldb * 8, col, 8, 8, n, cudaMemcpyDeviceToDevice, s));
  }
  DeviceStatus h;
  if ((e = read_status(w.st, s, &h))) return e;
  return h.error;
}

// Views into a solve workspace (after updes_factor) for the batched solves.
int solve_ws_views(const updes_problem* p, void* workspace, size_t workspace_bytes, const float** Khi,
                   const float** Klo, const float** F32, const double** F64, int64_t* ld, const int32_t** piv,
                   const double** dr, const double** dc, DeviceStatus** st, const int32_t** state) {
  SolveWs w;
  updes_solve_opts o;
  int e = solve_setup(p, nullptr, workspace, workspace_bytes, &w, &o);
  if (e) return e;
  *Khi = w.Khi;
  *Klo = w.Klo;
  *F32 = w.F32;
  *F64 = w.W;
  *ld = w.ld;
  *piv = w.piv;
  *dr = w.dr;
  *dc = w.dc;
  *st = w.lu.st;
  *state = w.state;
  return UPDES_OK;
}

extern "C" int updes_workspace_status(const updes_problem* p, void* workspace, size_t workspace_bytes,
                                      int32_t* error, void* stream) {
  SolveWs w;
  updes_solve_opts o;
  int e = solve_setup(p, nullptr, workspace, workspace_bytes, &w, &o);
  if (e) return e;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DeviceStatus h;
  if ((e = read_status(w.lu.st, s, &h))) return e;
  if (error) *error = h.error;
  UPDES_CUDA_TRY(cudaMemsetAsync(w.lu.st, 0, sizeof(DeviceStatus), s));
  return UPDES_OK;
}

// ---------------------------------------------------------------------------
// Adjoint: K^T lambda = g with the factors left in the workspace by updes_solve
// ---------------------------------------------------------------------------
extern "C" int updes_solve_transpose(const updes_problem* p, const double* g, double* lambda,
                                     const updes_solve_opts* opts, updes_solve_info* info, void* workspace,
                                     size_t workspace_bytes, void* stream) {
  if (updes_check_problem(p) || !g || !lambda || !workspace) return UPDES_ERR_INVALID;
  updes_solve_opts o = normalise(opts);
  const int n = p->N + p->M;
  updes_solve_opts olay = o;
  olay.precision = UPDES_PREC_FP32;
  if (workspace_bytes < solve_ws_layout(n, olay, nullptr, nullptr)) return UPDES_ERR_WORKSPACE;
  SolveWs w;
  solve_ws_layout(n, olay, static_cast<char*>(workspace), &w);
  updes_solve_info dummy;
  if (!info) info = &dummy;
  std::memset(info, 0, sizeof *info);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int precision = 0;
  if (int e0 = read_state(w, n, &precision, s)) return e0;  // no factorisation of this system in the workspace
  const unsigned gr = unsigned(ceil_div(n, 256));
  Timer t(s);
  UPDES_CUDA_TRY(cudaMemsetAsync(w.lu.st, 0, sizeof(DeviceStatus), s));
  // K^T lambda = g  <=>  Ks^T mu = dc .* g,  lambda = dr .* mu
  UPDES_CUDA_TRY(cudaMemcpyAsync(w.bs, g, size_t(n) * 8, cudaMemcpyDeviceToDevice, s));
  axpby_kernel<<<gr, 256, 0, s>>>(w.bs, 1.0, w.bs, 0.0, n, w.dc);
  UPDES_LAUNCH_CHECK();
  abs_kernel<<<gr, 256, 0, s>>>(w.bs, w.bsabs, n);
  UPDES_LAUNCH_CHECK();
  UPDES_CUDA_TRY(cudaMemcpyAsync(w.x, w.bs, size_t(n) * 8, cudaMemcpyDeviceToDevice, s));
  int e;
  if ((e = precond(w, n, precision, w.x, s, true))) return e;
  updes_solve_opts oi = o;
  if (precision == UPDES_PREC_FP64) oi.max_iters = 0;
  if ((e = gmres(w, n, precision, oi, info, s, true))) return e;
  if (precision == UPDES_PREC_FP64) info->converged = 1;
  info->fell_back = precision == UPDES_PREC_FP64 && o.precision == UPDES_PREC_FP32;
  axpby_kernel<<<gr, 256, 0, s>>>(w.x, 1.0, w.x, 0.0, n, w.dr);
  UPDES_LAUNCH_CHECK();
  UPDES_CUDA_TRY(cudaMemcpyAsync(lambda, w.x, size_t(n) * 8, cudaMemcpyDeviceToDevice, s));
  DeviceStatus h;
  if ((e = read_status(w.lu.st, s, &h))) return e;
  if (h.error) return h.error;
  info->t_refine_ms = t.stop();
  return info->converged ? UPDES_OK : UPDES_ERR_NOT_CONVERGED;
}

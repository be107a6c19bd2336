// Many independent collocation systems of uneven size in ONE persistent launch (updes_solve_batched).
//
// The reference solves each system with its own pde_solver call (updes/operators.py:559-618).  Systems of a
// few hundred to a few thousand nodes leave most of a GB300 idle one at a time, and a solve made of hundreds
// of small launches per system is bound by launch and synchronisation latency.  Here one CTA per SM takes
// systems from a device work queue (largest first) and runs the whole solve of each inside the CTA:
//
//   assembly   K (FP64, closed forms of entries.cuh), equilibrated by powers of two (rows, then columns);
//              the value matrix A[:N] = [Phi P] for vals, in FP64
//   LU         right-looking, partial pivoting (LAPACK's pivot rule), panel width nb chosen per system size
//              by the autotuner (updes_batched_tune); the elimination in double-float arithmetic on the FP32
//              pipes (UPDES_PREC_FP32: about 48-bit factors, GB300's FP64 pipe is 1/64 of its FP32 rate) or
//              in FP64 (UPDES_PREC_FP64)
//   refinement y = (LU)^-1 b, then classical refinement sweeps y += (LU)^-1 (b - K y) with an FP64 residual
//              while the componentwise backward error still halves (down to 2 FP64 unit roundoffs; 32
//              count as converged) and the sweep cap is not met; with 48-bit factors each sweep gains a factor of about 1 / (cond(K) 2^-48),
//              so one or two sweeps reach the floor wherever cond(K) 2^-48 is small
//   values     coeffs = Dc y, vals = A[:N] coeffs
//
// The CTA's scratch (its slice of the workspace) holds K, the working matrix and A for the largest system.
// Every wait is a CTA barrier; there is no wait between CTAs, so nothing can hang on another CTA.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "df.cuh"
#include "entries.cuh"
#include "rbf.cuh"
#include "stats.cuh"

int updes_check_problem(const updes_problem* p);

namespace {

constexpr int kBT = 512;                 // threads per CTA
constexpr int kWarps = kBT / 32;
constexpr int kTM = 128, kTN = 64;       // trailing-update tile: 4 x 4 entries per thread
constexpr int kMaxNB = 64;               // widest panel
constexpr int kMaxBatchN = 4096;         // the solve's vectors live in shared memory
// A solve counts as converged at a componentwise backward error of 32 FP64 unit roundoffs (the residual is
// FP64 here, K being kept in FP64), but refinement goes on while the error still halves, down to 2 unit
// roundoffs: on the r^5 systems of a few hundred nodes the vals only agree with an FP64 LU's to within
// FP64's own spread once the backward error is a few unit roundoffs.
constexpr double kBwdFloorB = 32.0 * 1.1102230246251565e-16;
constexpr double kBwdStop = 2.0 * 1.1102230246251565e-16;

struct BatchSys {
  updes_problem p;
  const double* q;
  double* coeffs;
  double* vals;
  int32_t n, nb, precision, max_sweeps;
};

struct BatchOut {
  int32_t lu_info, sweeps, converged, done;
  double backward_error;
};

// Shared memory of one CTA: the LU's staged tiles, or the solve's two vectors.
struct SmemLU {
  double L[kTM][kMaxNB];      // L21 rows of the current row chunk (8-byte elements of either type)
  double U[kMaxNB][kTN];      // U12 columns of the current column chunk
  double L11[kMaxNB][kMaxNB]; // unit lower diagonal block of the panel
  double prow[kMaxNB];        // pivot row of the panel column being eliminated
};
constexpr size_t kSmemBytes = sizeof(SmemLU) > 2 * kMaxBatchN * sizeof(double) ? sizeof(SmemLU)
                                                                                 : 2 * kMaxBatchN * sizeof(double);

// Element arithmetic of the elimination: FP64, or double-float (F2, 8 bytes like a double).
struct OpsF64 {
  using T = double;
  static __device__ __forceinline__ T from_d(double v) { return v; }
  static __device__ __forceinline__ double to_d(T a) { return a; }
  static __device__ __forceinline__ void fms(T& c, T a, T b) { c = fma(-a, b, c); }  // c -= a b
  static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
  // acc[a][b] -= sum_k L[a][k] U[k][16 b] over a 4 x 4 register tile (L rows ldl apart, U rows ldu apart)
  static __device__ __forceinline__ void tile_update(T (&acc)[4][4], const T* L, int ldl, const T* U, int ldu,
                                                     int kb) {
    for (int k = 0; k < kb; ++k) {
      T la[4], ub[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) la[a] = L[a * ldl + k];
#pragma unroll
      for (int b = 0; b < 4; ++b) ub[b] = U[k * ldu + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) fms(acc[a][b], la[a], ub[b]);
    }
  }
};

struct OpsDF {
  using T = F2;
  static __device__ __forceinline__ T from_d(double v) { return df_from_double(v); }
  static __device__ __forceinline__ double to_d(T a) { return double(a.h) + double(a.l); }
  // c -= a b: the exact product of the high parts by FMA plus the cross terms, subtracted by TwoSum, then
  // renormalised (every operation an _rn intrinsic, so the compiler cannot contract the error terms away)
  static __device__ __forceinline__ void fms(T& c, T a, T b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e));
    const float s = __fsub_rn(c.h, p);
    const float v = __fsub_rn(s, c.h);
    float t = __fsub_rn(__fsub_rn(c.h, __fsub_rn(s, v)), __fadd_rn(p, v));
    t = __fadd_rn(t, __fsub_rn(c.l, e));
    const float h = __fadd_rn(s, t);
    c.l = __fsub_rn(t, __fsub_rn(h, s));
    c.h = h;
  }
  static __device__ __forceinline__ T mul(T a, T b) { return df_mul(a, b); }
  // fms on two columns at once with the packed FP32x2 instructions of sm_100+ (one issue slot per pair): the
  // same operations in the same order as fms, so bitwise the same results; y - x is fma(x, -1, y), which
  // rounds once like the subtraction
  static __device__ __forceinline__ float2 sub2(float2 y, float2 x) {
    return __ffma2_rn(x, make_float2(-1.f, -1.f), y);
  }
  static __device__ __forceinline__ void fms2(float2& ch, float2& cl, T a, float2 bh, float2 bl) {
    const float2 ah = make_float2(a.h, a.h), al = make_float2(a.l, a.l);
    const float2 p = __fmul2_rn(ah, bh);
    float2 e = __ffma2_rn(ah, bh, make_float2(-p.x, -p.y));
    e = __ffma2_rn(ah, bl, __ffma2_rn(al, bh, e));
    const float2 s = sub2(ch, p);
    const float2 v = sub2(s, ch);
    float2 t = sub2(sub2(ch, sub2(s, v)), __fadd2_rn(p, v));
    t = __fadd2_rn(t, sub2(cl, e));
    const float2 h = __fadd2_rn(s, t);
    cl = sub2(t, sub2(h, s));
    ch = h;
  }
  static __device__ __forceinline__ void tile_update(T (&acc)[4][4], const T* L, int ldl, const T* U, int ldu,
                                                     int kb) {
    float2 ch[4][2], cl[4][2];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        ch[a][q] = make_float2(acc[a][2 * q].h, acc[a][2 * q + 1].h);
        cl[a][q] = make_float2(acc[a][2 * q].l, acc[a][2 * q + 1].l);
      }
    for (int k = 0; k < kb; ++k) {
      T la[4];
      float2 ubh[2], ubl[2];
#pragma unroll
      for (int a = 0; a < 4; ++a) la[a] = L[a * ldl + k];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const T u0 = U[k * ldu + 32 * q], u1 = U[k * ldu + 32 * q + 16];
        ubh[q] = make_float2(u0.h, u1.h);
        ubl[q] = make_float2(u0.l, u1.l);
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int q = 0; q < 2; ++q) fms2(ch[a][q], cl[a][q], la[a], ubh[q], ubl[q]);
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        acc[a][2 * q] = {ch[a][q].x, cl[a][q].x};
        acc[a][2 * q + 1] = {ch[a][q].y, cl[a][q].y};
      }
  }
};

__device__ __forceinline__ double pow2_scale(double m) {
  // 2^-e with m = f 2^e, f in [0.5, 1): scales m into [0.5, 1) exactly; 1 for m = 0 or non-finite m
  int e = 0;
  if (m > 0.0 && isfinite(m)) frexp(m, &e);
  return ldexp(1.0, -e);
}

// max over the CTA of (value, -index): the largest value, the smallest index on ties.
__device__ __forceinline__ void cta_argmax(double& v, int& i, double* red_v, int* red_i) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, v, o);
    const int oi = __shfl_xor_sync(0xffffffffu, i, o);
    if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; }
  }
  if (lane == 0) { red_v[w] = v; red_i[w] = i; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < kWarps; ++k)
      if (red_v[k] > red_v[0] || (red_v[k] == red_v[0] && red_i[k] < red_i[0])) { red_v[0] = red_v[k]; red_i[0] = red_i[k]; }
  }
  __syncthreads();
  v = red_v[0];
  i = red_i[0];
  __syncthreads();
}

__device__ __forceinline__ double cta_max(double v, double* red_v) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (lane == 0) red_v[w] = v;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 1; k < kWarps; ++k) red_v[0] = fmax(red_v[0], red_v[k]);
  __syncthreads();
  v = red_v[0];
  __syncthreads();
  return v;
}

// ---- assembly ---------------------------------------------------------------------------------------------

// K (n x ld, FP64) and A[:N] (N x ld, FP64) of one system, K equilibrated in place: dr (rows) and dc
// (columns) are the powers of two applied, b = Dr [q; 0].  One warp per row.
template <int KIND>
__device__ void assemble_system(const BatchSys& sys, double* K, double* A, int64_t ld, double* dr, double* dc,
                                double* b, double* red_v) {
  const updes_problem& p = sys.p;
  const int n = sys.n, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ip = (KIND == UPDES_RBF_POLYHARMONIC) ? 2 * int(p.rbf_param) + 1 : int(p.rbf_param);
  for (int r = warp; r < n; r += kWarps) {
    const RowInfo ri = load_row(p, r);
    double* Kr = K + int64_t(r) * ld;
    double* Ar = A + int64_t(r) * ld;
    // the value row of node r, A[r] = [phi(x_r - x_j) (0 at j = r), m_k(x_r)], from the same kernel
    // evaluations as K's row where the row's evaluation node is r
    const bool fused = r < p.N && ri.a == r;
    double mx = 0.0;
    for (int c = lane; c < n; c += 32) {
      double v;
      if (c < p.N) {
        const double xc = p.nodes[2ll * c], yc = p.nodes[2ll * c + 1];
        if (fused) {
          double phi;
          v = entry_rbf_phi<KIND>(ri, c, xc, yc, p.rbf_param, ip, p.self_term, &phi);
          Ar[c] = phi;
        } else {
          v = entry_rbf<KIND>(ri, c, xc, yc, p.rbf_param, ip, p.self_term);
        }
      } else {
        v = entry_mono(ri, c - p.N);
      }
      Kr[c] = v;
      mx = fmax(mx, fabs(v));
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const double s = pow2_scale(mx);
    for (int c = lane; c < n; c += 32) Kr[c] *= s;
    if (lane == 0) {
      dr[r] = s;
      b[r] = r < p.N ? s * sys.q[r] : 0.0;
    }
    if (r < p.N) {
      const double xr = p.nodes[2ll * r], yr = p.nodes[2ll * r + 1];
      for (int c = lane; c < n; c += 32) {
        if (c >= p.N) Ar[c] = monomial_terms(c - p.N, xr, yr).m;
        else if (!fused)
          Ar[c] = (c == r && !p.self_term) ? 0.0 : rbf_value<KIND>(xr - p.nodes[2ll * c], yr - p.nodes[2ll * c + 1], p.rbf_param, ip);
      }
    }
  }
  __syncthreads();
  // column powers of two over the row-scaled K, applied in place
  for (int c = threadIdx.x; c < n; c += kBT) {
    double mx = 0.0;
    for (int r = 0; r < n; ++r) mx = fmax(mx, fabs(K[int64_t(r) * ld + c]));
    dc[c] = pow2_scale(mx);
  }
  __syncthreads();
  (void)red_v;
}

// W = K (scaled) converted to the elimination's type.
template <class Ops>
__device__ void scale_columns_to_w(const BatchSys& sys, double* K, typename Ops::T* W, int64_t ld, const double* dc) {
  const int n = sys.n;
  for (int r = threadIdx.x >> 5; r < n; r += kWarps) {
    double* Kr = K + int64_t(r) * ld;
    typename Ops::T* Wr = W + int64_t(r) * ld;
    for (int c = threadIdx.x & 31; c < n; c += 32) {
      const double v = Kr[c] * dc[c];
      Kr[c] = v;
      Wr[c] = Ops::from_d(v);
    }
  }
  __syncthreads();
}

// ---- LU -----------------------------------------------------------------------------------------------------

template <class Ops>
__device__ int cta_lu(typename Ops::T* W, int64_t ld, int n, int nb, int32_t* piv, SmemLU& sm, double* red_v,
                      int* red_i) {
  using T = typename Ops::T;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int info = 0;
  T* L = reinterpret_cast<T*>(&sm.L[0][0]);
  T* U = reinterpret_cast<T*>(&sm.U[0][0]);
  T* L11 = reinterpret_cast<T*>(&sm.L11[0][0]);
  T* prow = reinterpret_cast<T*>(&sm.prow[0]);
  for (int k0 = 0; k0 < n; k0 += nb) {
    const int kb = min(nb, n - k0);
    const int k1 = k0 + kb;
    // ---- panel: columns [k0, k1), rows [k0, n).  One thread per row for the scaling and the rank-1
    // update (its row's panel entries are adjacent, so after the first access they come from L1, and the
    // CTA's 512 rows are in flight at once); the candidate for the next column's pivot is taken on the way.
    double bv = -1.0;
    int bi = n;
    for (int i = k0 + tid; i < n; i += kBT) {
      double v = fabs(Ops::to_d(W[int64_t(i) * ld + k0]));
      if (v != v) v = INFINITY;  // NaN wins, so it surfaces as a bad pivot
      if (v > bv) { bv = v; bi = i; }
    }
    for (int j = k0; j < k1; ++j) {
      cta_argmax(bv, bi, red_v, red_i);
      const int p = bi < n ? bi : j;
      if (p != j)
        for (int c = tid; c < n; c += kBT) {
          T* a = W + int64_t(j) * ld + c;
          T* b = W + int64_t(p) * ld + c;
          const T t = *a;
          *a = *b;
          *b = t;
        }
      __syncthreads();
      const double pv = Ops::to_d(W[int64_t(j) * ld + j]);
      const bool ok = pv != 0.0 && isfinite(pv);
      if (tid == 0) {
        piv[j] = p;
        if (!ok && info == 0) info = j + 1;
      }
      for (int c = j + 1 + tid; c < k1; c += kBT) prow[c - k0] = W[int64_t(j) * ld + c];
      __syncthreads();
      bv = -1.0;
      bi = n;
      const T inv = Ops::from_d(ok ? 1.0 / pv : 0.0);
      // rows below: scale column j and update the panel's columns (j, k1), one thread per row; the row's
      // remaining panel entries are loaded together (one round trip), updated in a local copy and stored
      // back, and the candidate for the next column's pivot is taken on the way.  (A warp-per-row mapping
      // with coalesced accesses and eight rows in flight per warp measured slower on GB300.)
      for (int i = j + 1 + tid; i < n; i += kBT) {
        T* Wi = W + int64_t(i) * ld;
        if (ok) {
          T rowv[kMaxNB];
          const int cnt = k1 - j;  // columns j .. k1 - 1
          for (int c = 0; c < cnt; ++c) rowv[c] = Wi[j + c];
          const T l = Ops::mul(rowv[0], inv);
          rowv[0] = l;
          for (int c = 1; c < cnt; ++c) Ops::fms(rowv[c], l, prow[j + c - k0]);
          for (int c = 0; c < cnt; ++c) Wi[j + c] = rowv[c];
          if (cnt > 1) {
            double v = fabs(Ops::to_d(rowv[1]));
            if (v != v) v = INFINITY;
            if (v > bv) { bv = v; bi = i; }
          }
        } else if (j + 1 < k1) {
          double v = fabs(Ops::to_d(Wi[j + 1]));
          if (v != v) v = INFINITY;
          if (v > bv) { bv = v; bi = i; }
        }
      }
      __syncthreads();
    }
    if (k1 >= n) break;
    // ---- U12 = L11^-1 A12 (rows [k0, k1), columns [k1, n))
    for (int e = tid; e < kb * kb; e += kBT) {
      const int r = e / kb, c = e % kb;
      L11[r * kMaxNB + c] = W[int64_t(k0 + r) * ld + k0 + c];
    }
    __syncthreads();
    for (int c = k1 + tid; c < n; c += kBT) {
      T col[kMaxNB];
      for (int r = 0; r < kb; ++r) col[r] = W[int64_t(k0 + r) * ld + c];
      for (int r = 1; r < kb; ++r)
        for (int t = 0; t < r; ++t) Ops::fms(col[r], L11[r * kMaxNB + t], col[t]);
      for (int r = 1; r < kb; ++r) W[int64_t(k0 + r) * ld + c] = col[r];
    }
    __syncthreads();
    // ---- A22 -= L21 U12 in 128 x 64 tiles, 4 x 4 entries per thread
    const int tr = tid >> 4, tc = tid & 15;
    for (int r0 = k1; r0 < n; r0 += kTM) {
      const int rows = min(kTM, n - r0);
      for (int e = tid; e < kTM * kb; e += kBT) {
        const int r = e / kb, c = e % kb;
        if (r < rows) L[r * kMaxNB + c] = W[int64_t(r0 + r) * ld + k0 + c];
      }
      for (int c0 = k1; c0 < n; c0 += kTN) {
        const int cols = min(kTN, n - c0);
        __syncthreads();  // the previous tile is done with U (and L has been staged)
        for (int e = tid; e < kb * kTN; e += kBT) {
          const int r = e / kTN, c = e % kTN;
          if (c < cols) U[r * kTN + c] = W[int64_t(k0 + r) * ld + c0 + c];
        }
        __syncthreads();
        // thread (tr, tc) owns rows 4 tr .. 4 tr + 3 and columns tc + 16 b: a warp's loads of a U row are then
        // 16 consecutive entries (no shared-memory bank conflicts), and its C accesses 128-byte row segments
        T acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int r = 4 * tr + a, c = tc + 16 * b;
            acc[a][b] = (r < rows && c < cols) ? W[int64_t(r0 + r) * ld + c0 + c] : Ops::from_d(0.0);
          }
        Ops::tile_update(acc, L + (4 * tr) * kMaxNB, kMaxNB, U + tc, kTN, kb);
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int r = 4 * tr + a, c = tc + 16 * b;
            if (r < rows && c < cols) W[int64_t(r0 + r) * ld + c0 + c] = acc[a][b];
          }
      }
      __syncthreads();  // L is restaged for the next row chunk
    }
  }
  __syncthreads();
  return info;
}

// ---- triangular solves on a shared-memory vector ------------------------------------------------------------

// v = U^-1 L^-1 P v with the factors in W (LAPACK layout: piv[j] is the row swapped with j at step j).  The
// forward and backward substitutions go by blocks of 32 rows: warp 0 solves a block's diagonal part, then all
// warps subtract the block's columns from the rows still to come (one warp per row, lanes over the block's
// columns, coalesced).
template <class Ops>
__device__ void cta_lu_solve(const typename Ops::T* W, int64_t ld, int n, const int32_t* piv, double* v) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0)
    for (int j = 0; j < n; ++j) {
      const int p = piv[j];
      if (p != j) { const double t = v[j]; v[j] = v[p]; v[p] = t; }
    }
  __syncthreads();
  // forward: unit lower
  for (int b0 = 0; b0 < n; b0 += 32) {
    const int bs = min(32, n - b0);
    if (warp == 0) {
      double xv = lane < bs ? v[b0 + lane] : 0.0;
      for (int r = 1; r < bs; ++r) {
        const double lr = lane < r ? Ops::to_d(W[int64_t(b0 + r) * ld + b0 + lane]) : 0.0;
        double s = lr * xv;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == r) xv -= s;
      }
      if (lane < bs) v[b0 + lane] = xv;
    }
    __syncthreads();
    const double xb = lane < bs ? v[b0 + lane] : 0.0;
    for (int i = b0 + bs + warp; i < n; i += kWarps) {
      double s = lane < bs ? Ops::to_d(W[int64_t(i) * ld + b0 + lane]) * xb : 0.0;
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) v[i] -= s;
    }
    __syncthreads();
  }
  // backward: upper with its diagonal
  const int nblk = (n + 31) / 32;
  for (int bb = nblk - 1; bb >= 0; --bb) {
    const int b0 = bb * 32, bs = min(32, n - b0);
    if (warp == 0) {
      double xv = lane < bs ? v[b0 + lane] : 0.0;
      for (int r = bs - 1; r >= 0; --r) {
        const double ur = (lane > r && lane < bs) ? Ops::to_d(W[int64_t(b0 + r) * ld + b0 + lane]) : 0.0;
        double s = ur * xv;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == r) xv = (xv - s) / Ops::to_d(W[int64_t(b0 + r) * ld + b0 + r]);
      }
      if (lane < bs) v[b0 + lane] = xv;
    }
    __syncthreads();
    const double xb = lane < bs ? v[b0 + lane] : 0.0;
    for (int i = warp; i < b0; i += kWarps) {
      double s = lane < bs ? Ops::to_d(W[int64_t(i) * ld + b0 + lane]) * xb : 0.0;
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) v[i] -= s;
    }
    __syncthreads();
  }
}

// r = b - K y (FP64, K the equilibrated matrix), returns max_i |r_i| / max_i (|K| |y| + |b|)_i.
__device__ double cta_residual(const double* K, int64_t ld, int n, const double* y, const double* b, double* r,
                               double* red_v) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double rmax = 0.0, smax = 0.0;
  for (int i = warp; i < n; i += kWarps) {
    const double* Ki = K + int64_t(i) * ld;
    double s = 0.0, a = 0.0;
    for (int c = lane; c < n; c += 32) {
      const double kv = Ki[c];
      s = fma(kv, y[c], s);
      a = fma(fabs(kv), fabs(y[c]), a);
    }
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_xor_sync(0xffffffffu, s, o);
      a += __shfl_xor_sync(0xffffffffu, a, o);
    }
    if (lane == 0) {
      const double ri = b[i] - s;
      r[i] = ri;
      rmax = fmax(rmax, fabs(ri));
      smax = fmax(smax, a + fabs(b[i]));
    }
  }
  rmax = cta_max(rmax, red_v);
  smax = cta_max(smax, red_v);
  return smax > 0.0 ? rmax / smax : rmax;
}

// ---- one system -------------------------------------------------------------------------------------------------

template <class Ops>
__device__ void solve_system(const BatchSys& sys, char* slice, int64_t ld_max, SmemLU& sm, double* red_v, int* red_i,
                             BatchOut* out) {
  using T = typename Ops::T;
  const int n = sys.n;
  const int64_t ld = (int64_t(n) + 3) & ~int64_t(3);
  (void)ld_max;
  double* K = reinterpret_cast<double*>(slice);
  T* W = reinterpret_cast<T*>(K + int64_t(n) * ld);
  double* A = reinterpret_cast<double*>(W + int64_t(n) * ld);
  double* dr = A + int64_t(n) * ld;
  double* dc = dr + n;
  double* b = dc + n;
  double* rv = b + n;
  int32_t* piv = reinterpret_cast<int32_t*>(rv + n);
  switch (sys.p.rbf) {
    case UPDES_RBF_POLYHARMONIC: assemble_system<UPDES_RBF_POLYHARMONIC>(sys, K, A, ld, dr, dc, b, red_v); break;
    case UPDES_RBF_GAUSSIAN: assemble_system<UPDES_RBF_GAUSSIAN>(sys, K, A, ld, dr, dc, b, red_v); break;
    case UPDES_RBF_MULTIQUADRIC: assemble_system<UPDES_RBF_MULTIQUADRIC>(sys, K, A, ld, dr, dc, b, red_v); break;
    case UPDES_RBF_INVERSE_MULTIQUADRIC:
      assemble_system<UPDES_RBF_INVERSE_MULTIQUADRIC>(sys, K, A, ld, dr, dc, b, red_v); break;
    default: assemble_system<UPDES_RBF_THIN_PLATE>(sys, K, A, ld, dr, dc, b, red_v); break;
  }
  scale_columns_to_w<Ops>(sys, K, W, ld, dc);
  const int info = cta_lu<Ops>(W, ld, n, sys.nb, piv, sm, red_v, red_i);
  // the solve's vectors: y and the correction, in shared memory
  double* y = reinterpret_cast<double*>(&sm);
  double* d = y + kMaxBatchN;
  for (int i = threadIdx.x; i < n; i += kBT) y[i] = b[i];
  __syncthreads();
  cta_lu_solve<Ops>(W, ld, n, piv, y);
  int sweeps = 0;
  double bwd = cta_residual(K, ld, n, y, b, rv, red_v);
  double last = INFINITY;
  while (bwd > kBwdStop && sweeps < sys.max_sweeps && bwd < 0.5 * last) {
    for (int i = threadIdx.x; i < n; i += kBT) d[i] = rv[i];
    __syncthreads();
    cta_lu_solve<Ops>(W, ld, n, piv, d);
    for (int i = threadIdx.x; i < n; i += kBT) y[i] += d[i];
    __syncthreads();
    last = bwd;
    bwd = cta_residual(K, ld, n, y, b, rv, red_v);
    ++sweeps;
  }
  // coeffs = Dc y; vals = A[:N] coeffs
  for (int i = threadIdx.x; i < n; i += kBT) {
    const double c = dc[i] * y[i];
    sys.coeffs[i] = c;
    y[i] = c;
  }
  __syncthreads();
  if (sys.vals) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = warp; i < sys.p.N; i += kWarps) {
      const double* Ai = A + int64_t(i) * ld;
      double s = 0.0;
      for (int c = lane; c < n; c += 32) s = fma(Ai[c], y[c], s);
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) sys.vals[i] = s;
    }
  }
  if (threadIdx.x == 0) {
    out->lu_info = info;
    out->sweeps = sweeps;
    out->backward_error = bwd;
    out->converged = (info == 0 && bwd <= kBwdFloorB) ? 1 : 0;
    out->done = 1;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kBT) batched_solve_kernel(const BatchSys* __restrict__ systems,
                                                            const int32_t* __restrict__ order, int count,
                                                            int* __restrict__ queue, char* __restrict__ scratch,
                                                            size_t slice_bytes, int64_t ld_max,
                                                            BatchOut* __restrict__ outs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemLU& sm = *reinterpret_cast<SmemLU*>(smem_raw);
  __shared__ double red_v[kWarps];
  __shared__ int red_i[kWarps];
  __shared__ int s_next;
  char* slice = scratch + size_t(blockIdx.x) * slice_bytes;
  for (;;) {
    if (threadIdx.x == 0) s_next = atomicAdd(queue, 1);
    __syncthreads();
    const int k = s_next;
    __syncthreads();
    if (k >= count) break;
    const int i = order[k];
    const BatchSys sys = systems[i];
    if (sys.precision == UPDES_PREC_FP64) solve_system<OpsF64>(sys, slice, ld_max, sm, red_v, red_i, outs + i);
    else solve_system<OpsDF>(sys, slice, ld_max, sm, red_v, red_i, outs + i);
  }
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Bytes of one CTA's slice for systems of at most n_max unknowns: K, W and A (n x ld, 8 bytes each),
// four n-vectors and the pivots.
size_t slice_bytes_for(int n_max) {
  const size_t ld = (size_t(n_max) + 3) & ~size_t(3);
  return align256(3 * size_t(n_max) * ld * 8 + 4 * size_t(n_max) * 8 + size_t(n_max) * 4);
}

int batch_n_max(const updes_problem* problems, int32_t count, int* n_max) {
  int mx = 0;
  for (int32_t i = 0; i < count; ++i) {
    const int e = updes_check_problem(&problems[i]);
    if (e) return e;
    if (problems[i].supports) return UPDES_ERR_UNSUPPORTED;
    mx = std::max(mx, problems[i].N + problems[i].M);
  }
  if (mx > kMaxBatchN) return UPDES_ERR_UNSUPPORTED;
  *n_max = mx;
  return UPDES_OK;
}

int sm_count() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  return sms;
}

std::atomic<unsigned long long> g_batched_smem_done{0};

}  // namespace

extern "C" int updes_solve_batched_workspace(const updes_problem* problems, int32_t count, int32_t ctas,
                                             size_t* bytes) {
  if (!problems || count <= 0 || ctas < 0 || !bytes) return UPDES_ERR_INVALID;
  int n_max = 0;
  const int e = batch_n_max(problems, count, &n_max);
  if (e) return e;
  const int c = std::min<int>(ctas > 0 ? ctas : sm_count(), count);
  if (c <= 0) return UPDES_ERR_CUDA;
  *bytes = slice_bytes_for(n_max) * size_t(c) + align256(size_t(count) * (sizeof(BatchSys) + sizeof(BatchOut) + 4)) +
           1024;
  return UPDES_OK;
}

extern "C" int updes_solve_batched(const updes_problem* problems, int32_t count, const double* const* q,
                                   double* const* coeffs, double* const* vals, const int32_t* precision,
                                   const int32_t* panel_width, int32_t max_sweeps, int32_t ctas,
                                   updes_solve_info* infos, void* workspace, size_t workspace_bytes, void* stream) {
  if (!problems || count <= 0 || !q || !coeffs || !workspace || ctas < 0 || max_sweeps < 0) return UPDES_ERR_INVALID;
  int n_max = 0;
  int e = batch_n_max(problems, count, &n_max);
  if (e) return e;
  const int nctas = std::min<int>(ctas > 0 ? ctas : sm_count(), count);
  if (nctas <= 0) return UPDES_ERR_CUDA;
  size_t need = 0;
  if ((e = updes_solve_batched_workspace(problems, count, nctas, &need))) return e;
  if (workspace_bytes < need) return UPDES_ERR_WORKSPACE;
  std::vector<BatchSys> sys(count);
  for (int32_t i = 0; i < count; ++i) {
    if (!q[i] || !coeffs[i]) return UPDES_ERR_INVALID;
    const int pr = precision ? precision[i] : UPDES_PREC_FP32;
    const int nb = panel_width ? panel_width[i] : 16;
    if ((pr != UPDES_PREC_FP32 && pr != UPDES_PREC_FP64) || nb < 1 || nb > kMaxNB) return UPDES_ERR_INVALID;
    sys[i].p = problems[i];
    sys[i].q = q[i];
    sys[i].coeffs = coeffs[i];
    sys[i].vals = vals ? vals[i] : nullptr;
    sys[i].n = problems[i].N + problems[i].M;
    sys[i].nb = nb;
    sys[i].precision = pr;
    sys[i].max_sweeps = max_sweeps;
  }
  // largest systems first (their solves are the longest)
  std::vector<int32_t> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
    const double ca = double(sys[a].n) * sys[a].n * sys[a].n * (sys[a].precision == UPDES_PREC_FP64 ? 6.0 : 1.0);
    const double cb = double(sys[b].n) * sys[b].n * sys[b].n * (sys[b].precision == UPDES_PREC_FP64 ? 6.0 : 1.0);
    return ca > cb;
  });
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  const size_t slice = slice_bytes_for(n_max);
  char* scratch = base;
  char* meta = base + slice * size_t(nctas);
  BatchSys* d_sys = reinterpret_cast<BatchSys*>(meta);
  BatchOut* d_out = reinterpret_cast<BatchOut*>(meta + align256(size_t(count) * sizeof(BatchSys)));
  int32_t* d_order = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(d_out) + align256(size_t(count) * sizeof(BatchOut)));
  int* d_queue = d_order + count;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  UPDES_CUDA_TRY(cudaMemcpyAsync(d_sys, sys.data(), sizeof(BatchSys) * count, cudaMemcpyHostToDevice, s));
  UPDES_CUDA_TRY(cudaMemcpyAsync(d_order, order.data(), sizeof(int32_t) * count, cudaMemcpyHostToDevice, s));
  UPDES_CUDA_TRY(cudaMemsetAsync(d_out, 0, sizeof(BatchOut) * count, s));
  UPDES_CUDA_TRY(cudaMemsetAsync(d_queue, 0, sizeof(int), s));
  if ((e = smem_opt_in(reinterpret_cast<const void*>(&batched_solve_kernel), int(kSmemBytes), g_batched_smem_done)))
    return e;
  {
    double flops = 0.0;
    for (const auto& x : sys) flops += 2.0 / 3.0 * double(x.n) * x.n * x.n;
    StatScope sc(kStatOther, s, flops, 0.0);
    batched_solve_kernel<<<nctas, kBT, kSmemBytes, s>>>(d_sys, d_order, count, d_queue, scratch, slice,
                                                         int64_t((n_max + 3) & ~3), d_out);
    UPDES_LAUNCH_CHECK();
  }
  std::vector<BatchOut> outs(count);
  UPDES_CUDA_TRY(cudaMemcpyAsync(outs.data(), d_out, sizeof(BatchOut) * count, cudaMemcpyDeviceToHost, s));
  UPDES_CUDA_TRY(cudaStreamSynchronize(s));
  int status = UPDES_OK;
  for (int32_t i = 0; i < count; ++i) {
    if (infos) {
      std::memset(&infos[i], 0, sizeof(updes_solve_info));
      infos[i].iters = outs[i].sweeps;
      infos[i].lu_info = outs[i].lu_info;
      infos[i].converged = outs[i].converged;
      infos[i].backward_error = outs[i].backward_error;
    }
    if (!outs[i].done) status = UPDES_ERR_CUDA;
    else if (status == UPDES_OK && outs[i].lu_info) status = UPDES_ERR_SINGULAR;
  }
  return status;
}

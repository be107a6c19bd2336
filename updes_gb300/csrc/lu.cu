// Blocked right-looking LU with partial pivoting and triangular solves.
//
// Two storage schemes share the kernels:
//   * FP64 LU: the working matrix W (FP64) is factored in place (F == W).
//   * mixed LU: W (FP64) holds the not-yet-factored trailing matrix; the
//     factors are stored in FP32 in F.  Every product of factor entries is
//     formed from the FP32 values and accumulated in FP64 into W, so the
//     Schur complements keep FP64 accuracy while L and U are FP32.
// Replaces the LAPACK getrf behind jnp.linalg.inv (updes/assembly.py:87-90)
// and the lineax QR factorisation (updes/operators.py:612-613).
#include <cooperative_groups.h>

#include <algorithm>
#include <cstdlib>
#include <type_traits>
#include <vector>

#include <atomic>

#include "common.cuh"
#include "lu.cuh"
#include "stats.cuh"
#include "gemm_tc.cuh"

namespace {

constexpr int kPanelThreads = 256;

struct Cand {
  double absval;
  int idx;
  int tag;  // column index + 1 this candidate belongs to (written last)
};

// Cooperative panel factorisation of W[k:n, k:k+nb] (FP64), result to F.
// DF_IN: the input is a double-float pair of FP32 planes (W = hi plane, Wlo = lo plane).
// swap_map (optional): [0] count, [1..128] destination rows, [129..256] source rows of the
// net row permutation of this panel's interchanges (row dst receives old row src).
template <typename TF, bool DF_IN>
__global__ void __launch_bounds__(kPanelThreads) panel_kernel(void* W, const float* Wlo, int64_t ldw, TF* F,
                                                              int64_t ldf, int n, int k, int nb, int rows_per_cta,
                                                              int32_t* __restrict__ piv, unsigned int* bar,
                                                              Cand* cand, double* cand_row, double* diag_row,
                                                              int32_t* swap_map, DeviceStatus* st) {
  // The FP64 path factors in FP64; the mixed path's panel reads the FP32 rounding (hi plane) of the
  // double-float trailing matrix and works in FP32 (each update one rounding, like an FMA).
  using TT = typename std::conditional<DF_IN, float, double>::type;
  extern __shared__ __align__(16) unsigned char panel_smem[];
  TT* tile = reinterpret_cast<TT*>(panel_smem);          // rows_per_cta x nb
  TT* prow = tile + int64_t(rows_per_cta) * nb;          // nb
  TT* drow = prow + nb;                                  // nb
  __shared__ double red_v[kPanelThreads / 32];
  __shared__ int red_i[kPanelThreads / 32];
  __shared__ int s_best_local, s_gw, s_p;
  __shared__ double s_pivval;

  const int G = gridDim.x, g = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int rbase = k + g * rows_per_cta;
  const int rcount = max(0, min(rows_per_cta, n - rbase));

  // rows over warps, columns over lanes (no division by the runtime panel width)
  for (int l = wid; l < rcount; l += kPanelThreads / 32)
    for (int c = lane; c < nb; c += 32) {
      const int64_t idx = int64_t(rbase + l) * ldw + k + c;
      if constexpr (DF_IN) tile[int64_t(l) * nb + c] = static_cast<const float*>(W)[idx];
      else tile[int64_t(l) * nb + c] = static_cast<const double*>(W)[idx];
    }
  __syncthreads();

  for (int j = 0; j < nb; ++j) {
    const int par = j & 1;
    const int diag = k + j;
    // 1. local candidate: max |a| over owned rows >= diag (smallest index on ties)
    double bv = -1.0;
    int bi = 0x7fffffff;
    for (int l = tid; l < rcount; l += blockDim.x) {
      const int gr = rbase + l;
      if (gr < diag) continue;
      const double v = fabs(double(tile[int64_t(l) * nb + j]));
      const double vv = (v != v) ? INFINITY : v;  // NaN wins, so it surfaces as a bad pivot
      if (vv > bv || (vv == bv && gr < bi)) { bv = vv; bi = gr; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    if (lane == 0) { red_v[wid] = bv; red_i[wid] = bi; }
    __syncthreads();
    if (tid == 0) {
      for (int w = 1; w < kPanelThreads / 32; ++w)
        if (red_v[w] > bv || (red_v[w] == bv && red_i[w] < bi)) { bv = red_v[w]; bi = red_i[w]; }
      s_best_local = (bi == 0x7fffffff) ? -1 : bi - rbase;
      red_v[0] = bv;
      red_i[0] = bi;
    }
    __syncthreads();
    if (s_best_local >= 0)
      for (int c = tid; c < nb; c += blockDim.x)
        __stcg(cand_row + (int64_t(par) * G + g) * nb + c, double(tile[int64_t(s_best_local) * nb + c]));
    if (diag >= rbase && diag < rbase + rcount)
      for (int c = tid; c < nb; c += blockDim.x)
        __stcg(diag_row + par * nb + c, double(tile[int64_t(diag - rbase) * nb + c]));
    __threadfence();
    __syncthreads();
    if (tid == 0) {
      // publish: value, then (index, tag) as one 8-byte word after a fence
      Cand* slot = cand + par * G + g;
      __stcg(&slot->absval, red_v[0]);
      __threadfence();
      const unsigned long long it = (unsigned long long)(unsigned)red_i[0] |
                                    ((unsigned long long)(unsigned)(diag + 1) << 32);
      atomicExch(reinterpret_cast<unsigned long long*>(&slot->idx), it);
    }
    // wait until every CTA has published its candidate for this column (bounded)
    for (int w = tid; w < G; w += blockDim.x) {
      volatile unsigned long long* tw = reinterpret_cast<volatile unsigned long long*>(&(cand + par * G + w)->idx);
      long long it = 0;
      while (int((*tw) >> 32) != diag + 1) {
        if (++it > spin_limit()) {
          status_error(st, UPDES_ERR_TIMEOUT);
          atomicCAS(&st->timeout_tag, 0, 1);
          break;
        }
        __nanosleep(20);
      }
      __threadfence();
    }
    // one answer for the whole CTA (another CTA may set the status word at any moment)
    if (__syncthreads_or(*reinterpret_cast<volatile int*>(&st->error) != 0)) return;
    // 2. global pivot
    bv = -1.0;
    bi = 0x7fffffff;
    int bw = -1;
    for (int w = tid; w < G; w += blockDim.x) {
      double2 raw = __ldcg(reinterpret_cast<const double2*>(cand + par * G + w));
      const Cand c = *reinterpret_cast<Cand*>(&raw);
      if (c.idx != 0x7fffffff && (c.absval > bv || (c.absval == bv && c.idx < bi))) { bv = c.absval; bi = c.idx; bw = w; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      const int ow = __shfl_xor_sync(0xffffffffu, bw, o);
      if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; bw = ow; }
    }
    if (lane == 0) { red_v[wid] = bv; red_i[wid] = bi; }
    __shared__ int red_w[kPanelThreads / 32];
    if (lane == 0) red_w[wid] = bw;
    __syncthreads();
    if (tid == 0) {
      for (int w = 1; w < kPanelThreads / 32; ++w)
        if (red_v[w] > bv || (red_v[w] == bv && red_i[w] < bi)) { bv = red_v[w]; bi = red_i[w]; bw = red_w[w]; }
      s_gw = bw;
      s_p = bi;
    }
    __syncthreads();
    const int gw = s_gw, p = s_p;
    for (int c = tid; c < nb; c += blockDim.x) {
      prow[c] = TT(__ldcg(cand_row + (int64_t(par) * G + gw) * nb + c));
      drow[c] = TT(__ldcg(diag_row + par * nb + c));
    }
    __syncthreads();
    if (tid == 0) {
      s_pivval = prow[j];
      if (g == 0) piv[diag] = p;
      const double pv = prow[j];
      if (g == 0 && (pv == 0.0 || !isfinite(pv))) atomicCAS(&st->lu_info, 0, diag + 1);
    }
    // 3. swap rows diag <-> p inside the panel
    if (diag >= rbase && diag < rbase + rcount)
      for (int c = tid; c < nb; c += blockDim.x) tile[int64_t(diag - rbase) * nb + c] = prow[c];
    if (p != diag && p >= rbase && p < rbase + rcount)
      for (int c = tid; c < nb; c += blockDim.x) tile[int64_t(p - rbase) * nb + c] = drow[c];
    __syncthreads();
    // 4. scale the column and update the rest of the panel
    const double pv = s_pivval;
    if (pv != 0.0 && isfinite(pv)) {
      const TT rinv = TT(1.0 / pv);
      const int l0 = max(0, diag + 1 - rbase);
      for (int l = l0 + tid; l < rcount; l += blockDim.x) tile[int64_t(l) * nb + j] *= rinv;
      __syncthreads();
      if (j + 1 < nb) {
        // rank-1 update of the panel's remaining columns: rows over warps, columns over lanes
        for (int l = l0 + wid; l < rcount; l += kPanelThreads / 32) {
          TT* row = tile + int64_t(l) * nb;
          const TT a = row[j];
          for (int c = j + 1 + lane; c < nb; c += 32) row[c] -= a * prow[c];
        }
      }
    }
    __syncthreads();
  }
  for (int l = wid; l < rcount; l += kPanelThreads / 32)
    for (int c = lane; c < nb; c += 32) F[int64_t(rbase + l) * ldf + k + c] = TF(tile[int64_t(l) * nb + c]);
  if (swap_map && g == 0 && tid < 32) {
    // net permutation of the interchanges piv[k, k+nb): content tracking over <= 2 nb rows
    __shared__ int rows_s[128], cont_s[128];
    for (int i = tid; i < nb; i += 32) rows_s[i] = cont_s[i] = k + i;
    int cnt = nb;
    __syncwarp();
    for (int i = 0; i < nb; ++i) {
      const int p = piv[k + i];
      if (p == k + i) continue;
      int found = -1;
      for (int q = tid; q < cnt; q += 32)
        if (rows_s[q] == p) found = q;
      found = __reduce_max_sync(0xffffffffu, found);
      if (found < 0) {
        if (tid == 0) { rows_s[cnt] = p; cont_s[cnt] = p; }
        found = cnt++;
        __syncwarp();
      }
      if (tid == 0) {
        const int a = cont_s[i];
        cont_s[i] = cont_s[found];
        cont_s[found] = a;
      }
      __syncwarp();
    }
    for (int q = tid; q < cnt; q += 32) {
      swap_map[1 + q] = rows_s[q];
      swap_map[129 + q] = cont_s[q];
    }
    if (tid == 0) swap_map[0] = cnt;
  }
}

// Row interchanges of up to 3 (plane, column range) jobs.
struct SwapJobs {
  float* plane[3];
  int64_t c0[3], c1[3];
  int njobs;
};

// All row interchanges of a panel in one pass: a CTA per (64-column chunk, job) reads the moved rows of its
// columns into shared memory, then writes each to its destination (the net permutation from the panel's swap
// map), so a launch touches only the rows that move.
__global__ void __launch_bounds__(256) swap_rows_kernel(SwapJobs jobs, int64_t ld, const int32_t* __restrict__ map) {
  __shared__ float buf[128][64];
  const int j = blockIdx.y;
  if (j >= jobs.njobs) return;
  const int cnt = map[0];
  const int col = threadIdx.x & 63, r0 = threadIdx.x >> 6;
  const int64_t c = jobs.c0[j] + int64_t(blockIdx.x) * 64 + col;
  const bool ok = c < jobs.c1[j];
  float* plane = jobs.plane[j];
  for (int q = r0; q < cnt; q += 4)
    if (ok) buf[q][col] = plane[int64_t(map[129 + q]) * ld + c];
  __syncthreads();
  for (int q = r0; q < cnt; q += 4)
    if (ok) plane[int64_t(map[1 + q]) * ld + c] = buf[q][col];
}

// The interchanges of nmaps consecutive panels (swap maps kSwapMapStride ints apart) in one launch: each CTA
// applies the maps to its columns in panel order, the order in which separate launches would apply them.
constexpr int kSwapMapStride = 512;
__global__ void __launch_bounds__(256) swap_rows_maps_kernel(SwapJobs jobs, int64_t ld, const int32_t* __restrict__ maps,
                                                             int nmaps) {
  __shared__ float buf[128][64];
  const int j = blockIdx.y;
  if (j >= jobs.njobs) return;
  const int col = threadIdx.x & 63, r0 = threadIdx.x >> 6;
  const int64_t c = jobs.c0[j] + int64_t(blockIdx.x) * 64 + col;
  const bool ok = c < jobs.c1[j];
  float* plane = jobs.plane[j];
  for (int m = 0; m < nmaps; ++m) {
    const int32_t* map = maps + m * kSwapMapStride;
    const int cnt = map[0];
    for (int q = r0; q < cnt; q += 4)
      if (ok) buf[q][col] = plane[int64_t(map[129 + q]) * ld + c];
    __syncthreads();
    for (int q = r0; q < cnt; q += 4)
      if (ok) plane[int64_t(map[1 + q]) * ld + c] = buf[q][col];
    __syncthreads();  // this map's rows are in place (and buf free) before the next map reads them
  }
}

// U = L^-1 W on rows [k, k+nb), columns [c0, c1): L unit lower from F (FP32), W double-float.  Each row is
// w_i - sum_j L_ij x_j accumulated in double-float (exact FP32 products, compensated sums) and rounded once
// to FP32 into F: FP32 ALU only.
__global__ void __launch_bounds__(64) trsm_df_kernel(float* Whi, const float* Wlo, int64_t ld, int k, int nb,
                                                     int64_t c0, int64_t c1) {
  __shared__ float sL[64][65];
  __shared__ float sX[64][65];
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    sL[i][j] = (j < i) ? Whi[int64_t(k + i) * ld + k + j] : 0.f;
  }
  __syncthreads();
  const int t = threadIdx.x;
  const int64_t c = c0 + int64_t(blockIdx.x) * blockDim.x + t;
  if (c >= c1) return;
  for (int i = 0; i < nb; ++i) {
    const int64_t idx = int64_t(k + i) * ld + c;
    float sh = Whi[idx], sl = Wlo[idx];
    for (int j = 0; j < i; ++j) {
      const float f = -sL[i][j], xj = sX[j][t];
      const float p = __fmul_rn(f, xj);
      const float e = __fmaf_rn(f, xj, -p);
      const float s2 = __fadd_rn(sh, p);
      const float bb = __fsub_rn(s2, sh);
      const float tt = __fadd_rn(__fsub_rn(sh, __fsub_rn(s2, bb)), __fsub_rn(p, bb));
      sh = s2;
      sl = __fadd_rn(sl, __fadd_rn(tt, e));
    }
    const float xi = __fadd_rn(sh, sl);
    sX[i][t] = xi;
    Whi[idx] = xi;
  }
}

// U12 = L11^-1 W12 for a full 64-row panel: 64 columns per CTA, 4 lanes per column.  The right-hand sides
// (double-float planes) are staged in shared memory in one coalesced pass; lane s of a column's group keeps
// rows s, s+4, ..., s+60 in registers, as eight pairs (s + 8q, s + 8q + 4) on the packed FP32x2 instructions
// of sm_100+ (one issue slot per pair; the same operations as scalar code, so bitwise the same results).
// Step j (unrolled): the owner of row j rounds it to FP32 (the factor entry), broadcasts it by shuffle, and
// every lane subtracts L[i][j] * x_j from its rows i > j in double-float arithmetic; the chain is one
// shuffle per row instead of a 2016-term dependent sum.
struct TrsmDfSmem {
  float L[64][65];
  float Xh[64][65], Xl[64][65];
};

__device__ __forceinline__ float2 trsm_sub2(float2 y, float2 x) { return __ffma2_rn(x, make_float2(-1.f, -1.f), y); }

__global__ void __launch_bounds__(256) trsm_df64_kernel(float* Whi, const float* Wlo, int64_t ld, int k, int64_t c0,
                                                        int64_t c1) {
  extern __shared__ float4 trsm_df_smem[];
  TrsmDfSmem& sm = *reinterpret_cast<TrsmDfSmem*>(trsm_df_smem);
  const int tid = threadIdx.x, lane = tid & 31;
  const int64_t cb = c0 + int64_t(blockIdx.x) * 64;
  for (int e = tid; e < 64 * 64; e += blockDim.x) {
    const int i = e >> 6, j = e & 63;
    sm.L[i][j] = (j < i) ? Whi[int64_t(k + i) * ld + k + j] : 0.f;
    const int64_t c = cb + j;
    const bool ok = c < c1;
    sm.Xh[i][j] = ok ? Whi[int64_t(k + i) * ld + c] : 0.f;
    sm.Xl[i][j] = ok ? Wlo[int64_t(k + i) * ld + c] : 0.f;
  }
  __syncthreads();
  const int col = tid >> 2, s = tid & 3;
  const int gbase = lane & ~3;
  float2 ah[8], al[8];  // pair q: rows s + 8q (.x) and s + 8q + 4 (.y)
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    ah[q] = make_float2(sm.Xh[s + 8 * q][col], sm.Xh[s + 8 * q + 4][col]);
    al[q] = make_float2(sm.Xl[s + 8 * q][col], sm.Xl[s + 8 * q + 4][col]);
  }
#pragma unroll
  for (int j = 0; j < 64; ++j) {
    // row j lives in slot j / 4 of lane j % 4: pair j / 8, half (j / 4) & 1
    const int q0 = j >> 3;
    const float mine = ((j >> 2) & 1) ? __fadd_rn(ah[q0].y, al[q0].y) : __fadd_rn(ah[q0].x, al[q0].x);
    const float xj = __shfl_sync(0xffffffffu, mine, gbase | (j & 3));
    if (s == (j & 3)) sm.Xh[j][col] = xj;
    const float2 x2 = make_float2(xj, xj);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      if (8 * q + 7 <= j) continue;  // both rows of this pair are <= j
      const int i0 = s + 8 * q, i1 = i0 + 4;
      const float2 f = make_float2(-sm.L[i0][j], -sm.L[i1][j]);
      const float2 p = __fmul2_rn(f, x2);
      const float2 e = __ffma2_rn(f, x2, make_float2(-p.x, -p.y));
      const float2 t0 = __fadd2_rn(ah[q], p);
      const float2 bb = trsm_sub2(t0, ah[q]);
      const float2 tt = __fadd2_rn(trsm_sub2(ah[q], trsm_sub2(t0, bb)), trsm_sub2(p, bb));
      const float2 nl = __fadd2_rn(al[q], __fadd2_rn(tt, e));
      // rows i <= j keep their values (only a pair straddling j has one)
      if (i0 > j) { ah[q].x = t0.x; al[q].x = nl.x; }
      if (i1 > j) { ah[q].y = t0.y; al[q].y = nl.y; }
    }
  }
  __syncthreads();
  for (int e = tid; e < 64 * 64; e += blockDim.x) {
    const int i = e >> 6, j = e & 63;
    const int64_t c = cb + j;
    if (c < c1) Whi[int64_t(k + i) * ld + c] = sm.Xh[i][j];
  }
}

// Apply the row interchanges piv[k0, k0+cnt) to columns [c0, c1) of M.
template <typename T>
__global__ void laswp_kernel(T* __restrict__ M, int64_t ld, const int32_t* __restrict__ piv, int k0, int cnt,
                             int64_t c0, int64_t c1) {
  const int64_t c = c0 + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (c >= c1) return;
  for (int i = k0; i < k0 + cnt; ++i) {
    const int p = piv[i];
    if (p != i) {
      T a = M[int64_t(i) * ld + c];
      M[int64_t(i) * ld + c] = M[int64_t(p) * ld + c];
      M[int64_t(p) * ld + c] = a;
    }
  }
}

// U12 = L11^-1 W12 (L11 unit lower from F), one thread per column, FP64 arithmetic.
template <typename TF>
__global__ void __launch_bounds__(64) trsm_kernel(double* W, int64_t ldw, TF* F,
                                                  int64_t ldf, int n, int k, int nb) {
  extern __shared__ double sL[];  // nb x nb
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    sL[e] = (j < i) ? double(F[int64_t(k + i) * ldf + k + j]) : 0.0;
  }
  __syncthreads();
  const int64_t c = int64_t(k) + nb + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (c >= n) return;
  double x[128];
  for (int i = 0; i < nb; ++i) {
    double s = W[int64_t(k + i) * ldw + c];
    for (int j = 0; j < i; ++j) s -= sL[i * nb + j] * x[j];
    x[i] = s;
  }
  for (int i = 0; i < nb; ++i) F[int64_t(k + i) * ldf + c] = TF(x[i]);
}

// W[r0:n, c0:n] -= F[r0:n, k:k+nb] * F[k:k+nb, c0:n], FP64 accumulation (SIMT reference path).
template <typename TF>
__global__ void __launch_bounds__(256) gemm_update_kernel(double* W, int64_t ldw,
                                                          const TF* F, int64_t ldf, int n, int k,
                                                          int nb) {
  __shared__ double As[32][65];
  __shared__ double Bs[32][65];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int r0 = k + nb + blockIdx.y * 64, c0 = k + nb + blockIdx.x * 64;
  double acc[4][4] = {};
  for (int kb = 0; kb < nb; kb += 32) {
    for (int e = threadIdx.x; e < 64 * 32; e += 256) {
      const int i = e >> 5, j = e & 31;           // A: row i, k-column j
      const int ra = r0 + i;
      As[j][i] = (ra < n && kb + j < nb) ? double(F[int64_t(ra) * ldf + k + kb + j]) : 0.0;
      const int kr = e >> 6, cj = e & 63;         // B: k-row kr, column cj
      const int cb = c0 + cj;
      Bs[kr][cj] = (kb + kr < nb && cb < n) ? double(F[int64_t(k + kb + kr) * ldf + cb]) : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < 32; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) { a[u] = As[kk][ty + 16 * u]; b[u] = Bs[kk][tx + 16 * u]; }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int r = r0 + ty + 16 * u;
    if (r >= n) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int c = c0 + tx + 16 * v;
      if (c < n) W[int64_t(r) * ldw + c] -= acc[u][v];
    }
  }
}

std::atomic<int> g_num_sms{0};

int num_sms() {
  if (!g_num_sms.load()) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    g_num_sms.store(v > 0 ? v : 1);
  }
  return g_num_sms.load();
}

}  // namespace

// ---------------------------------------------------------------------------------------------------
// FP32 panel of the mixed LU with one exchange per column and look-ahead.
//
// G <= 32 CTAs each hold a block of the panel's rows in shared memory.  For every column j, each CTA
// publishes one record: its best candidate (|a|, row) together with that row's values, and the owner of the
// diagonal position publishes the row sitting there.  Every entry of a record is an 8-byte word holding the
// column's tag (global column + 1) in its high half and a 32-bit value in its low half, stored and loaded as
// one single-copy-atomic access, so an entry whose tag matches is that column's value: the publisher needs
// no fence.  A record's header (the (idx, |a|) pair) is stored after the CTA barrier that follows its row
// stores.  G + 1 reader threads wait for the headers, from which every warp finds the pivot; the CTA then
// fetches only the pivot's row and the diagonal row, re-reading (bounded) an entry whose tag is not yet the
// column's.  A CTA that gives up on a wait records a timeout and returns; the others then give up on their
// own bounded waits for its records.
//
// The records are published right after the look-ahead step (column j+1 updated and searched), before the
// rank-1 update of the other columns, which then overlaps the exchange; a published row therefore still
// lacks that last update for columns >= j+2, and readers apply it with the same fused multiply-add (bitwise
// the same values as the owner's).  Records alternate between two slots by column parity: a CTA publishes
// column j+2 into column j's slot only after it has seen every header of column j+1, which each CTA
// publishes only after its reads of column j's slot have returned.
struct alignas(16) PanelRec {
  unsigned long long idx;         // candidate row (INT_MAX: none); the diagonal record: the diagonal row
  unsigned long long absval;      // |a| of the candidate
  unsigned long long row[kLuNb];  // the candidate's row (the diagonal record: the row at the diagonal)
};

__device__ __forceinline__ void st_tagged(unsigned long long* p, unsigned long long tag, uint32_t bits) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(tag | bits) : "memory");
}

// Tagged entries loaded from L2 (bypassing L1, so a re-read sees new stores): one entry, or two adjacent
// ones in a 16-byte load, each 8-byte half validated by its own tag.
__device__ __forceinline__ unsigned long long ld_tagged_cg(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.global.cg.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ ulonglong2 ld_tagged_pair(const unsigned long long* p) {
  ulonglong2 v;
  asm volatile("ld.global.cg.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p) : "memory");
  return v;
}

// Order key of a pivot candidate's |a| (-1: no candidate; NaN has been mapped to +inf): 0 for none, else
// the float's bits + 1, which orders non-negative floats as unsigned integers.
__device__ __forceinline__ unsigned cand_key(float v) { return v < 0.f ? 0u : __float_as_uint(v) + 1u; }
__device__ __forceinline__ float cand_val(unsigned key) { return key ? __uint_as_float(key - 1u) : -1.f; }
constexpr int kMaxPanelCtas = 32;
constexpr int kPanelF32Threads = 512;  // 16 warps: the rank-1 update and the searches split over more rows

__global__ void __launch_bounds__(kPanelF32Threads) panel_f32_kernel(float* W, int64_t ld, int n, int k, int nb,
                                                                  int rows_per_cta, int32_t* __restrict__ piv,
                                                                  PanelRec* recs, int32_t* swap_map,
                                                                  DeviceStatus* st) {
  extern __shared__ __align__(16) unsigned char pf_smem[];
  float(*crow)[kLuNb] = reinterpret_cast<float(*)[kLuNb]>(pf_smem);      // 32 x 64 (row 0: the pivot's row)
  float* wrow = crow[0];  // the pivot's row as its record holds it
  // rows_per_cta x nb with row stride nb + 1: consecutive rows of one column fall in different banks
  float* tile = reinterpret_cast<float*>(pf_smem) + (kMaxPanelCtas + 3) * kLuNb;
  const int ldt = nb + 1;
  float* drow = crow[kMaxPanelCtas];                                      // 64: row at the diagonal position
  float* prow = drow + kLuNb;                                             // 64: this column's pivot row
  float* pprev = prow + kLuNb;                                            // 64: the previous column's pivot row
  __shared__ unsigned s_ckey[kMaxPanelCtas];
  __shared__ int s_cidx[kMaxPanelCtas];
  __shared__ unsigned red_k[kPanelF32Threads / 32];
  __shared__ unsigned red_i[kPanelF32Threads / 32];

  const int G = gridDim.x, g = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int rbase = k + g * rows_per_cta;
  const int rcount = max(0, min(rows_per_cta, n - rbase));
  constexpr int kW = kPanelF32Threads / 32;

  for (int l = wid; l < rcount; l += kW)
    for (int c = lane; c < nb; c += 32) tile[int64_t(l) * ldt + c] = W[int64_t(rbase + l) * ld + k + c];
  __syncthreads();

  // this thread's candidate for column j over its rows l (local) in [l_from, rcount), stepping by the CTA's
  // threads: the largest |a| (NaN counts as +inf), the smallest row on ties
  auto scan = [&](int j, int l_from, unsigned& key, unsigned& row) {
    for (int l = l_from + tid; l < rcount; l += blockDim.x) {
      const float v = fabsf(tile[int64_t(l) * ldt + j]);
      const unsigned kv = cand_key((v != v) ? INFINITY : v);
      if (kv > key) { key = kv; row = unsigned(rbase + l); }
    }
  };
  // The CTA's candidate for column j from every thread's (key, row), and the records of column j: the
  // candidate (header and row) and, by the owner of position k + j, the row there.  Warps 0 and 1 finish the
  // argmax over the 16 warp results themselves and publish the candidate's row; warps 2 and 3 publish the
  // diagonal row.  The barrier after the row stores keeps the published rows from being changed by the
  // rank-1 update before they are read, and the headers, which readers wait for, are stored after it.
  auto publish = [&](int j, unsigned key, unsigned row) {
    unsigned km = __reduce_max_sync(0xffffffffu, key);
    unsigned rm = __reduce_min_sync(0xffffffffu, key == km ? row : 0xffffffffu);
    if (lane == 0) { red_k[wid] = km; red_i[wid] = rm; }
    __syncthreads();
    const int par = j & 1, diag = k + j;
    const unsigned long long tag = static_cast<unsigned long long>(unsigned(diag + 1)) << 32;
    PanelRec* mine = recs + par * (kMaxPanelCtas + 1) + g;
    PanelRec* drec = recs + par * (kMaxPanelCtas + 1) + kMaxPanelCtas;
    if (tid < 64) {
      const unsigned k2 = lane < kW ? red_k[lane] : 0u, r2 = lane < kW ? red_i[lane] : 0x7fffffffu;
      km = __reduce_max_sync(0xffffffffu, k2);
      rm = __reduce_min_sync(0xffffffffu, k2 == km ? r2 : 0xffffffffu);
      const int best = (rm == 0x7fffffffu) ? -1 : int(rm) - rbase;  // local row; -1: no candidate (zero row)
      if (tid < nb) st_tagged(&mine->row[tid], tag, __float_as_uint(best >= 0 ? tile[int64_t(best) * ldt + tid] : 0.f));
    } else if (tid < 128 && diag >= rbase && diag < rbase + rcount) {
      const int c = tid - 64;
      if (c < nb) st_tagged(&drec->row[c], tag, __float_as_uint(tile[int64_t(diag - rbase) * ldt + c]));
    }
    __syncthreads();
    if (tid == 0) {
      st_tagged(&mine->absval, tag, __float_as_uint(cand_val(km)));
      st_tagged(&mine->idx, tag, rm);
    } else if (tid == 64 && diag >= rbase && diag < rbase + rcount) {
      st_tagged(&drec->idx, tag, unsigned(diag));
    }
  };

  {
    unsigned key = 0u, row = 0x7fffffffu;
    scan(0, 0, key, row);
    publish(0, key, row);
  }
  bool prev_ok = false;  // the previous column's pivot was usable, so its update is pending in published rows
  for (int j = 0; j < nb; ++j) {
    const int par = j & 1, diag = k + j;
    const PanelRec* base = recs + par * (kMaxPanelCtas + 1);
    const unsigned want = unsigned(diag + 1);
    // wait (bounded) for the headers: each candidate record's (idx, |a|) pair, the diagonal record's idx
    bool gave_up = false;
    if (tid <= G) {
      const unsigned long long* hp = (tid < G) ? &base[tid].idx : &base[kMaxPanelCtas].idx;
      ulonglong2 h = ld_tagged_pair(hp);
      long long it = 0;
      while (unsigned(h.x >> 32) != want || (tid < G && unsigned(h.y >> 32) != want)) {
        if (++it > spin_limit()) {
          status_error(st, UPDES_ERR_TIMEOUT);
          atomicCAS(&st->timeout_tag, 0, 2);
          gave_up = true;
          break;
        }
        if (it > 64) __nanosleep(20);  // the exchange normally lands within a few round trips: poll hot first
        h = ld_tagged_pair(hp);
      }
      if (tid < G) {
        s_cidx[tid] = int(unsigned(h.x));
        s_ckey[tid] = cand_key(__uint_as_float(unsigned(h.y)));
      }
    }
    if (__syncthreads_or(gave_up)) return;
    // pivot: the largest |a| over the G candidates, the smallest row on ties (every warp computes it)
    int p, gw;
    {
      const unsigned ck = lane < G ? s_ckey[lane] : 0u, ci = lane < G ? unsigned(s_cidx[lane]) : 0x7fffffffu;
      const unsigned km = __reduce_max_sync(0xffffffffu, ck);
      const unsigned im = __reduce_min_sync(0xffffffffu, ck == km ? ci : 0xffffffffu);
      p = int(im);
      gw = __ffs(__ballot_sync(0xffffffffu, ck == km && ci == im)) - 1;
    }
    // the pivot's row from record gw (threads 0-63) and the diagonal row (threads 64-127), each entry
    // re-read (bounded) until it carries the column's tag
    if (tid < 128 && (tid & 63) < nb) {
      const int c = tid & 63;
      const unsigned long long* q = tid < 64 ? &base[gw].row[c] : &base[kMaxPanelCtas].row[c];
      unsigned long long x = ld_tagged_cg(q);
      long long it = 0;
      while (unsigned(x >> 32) != want) {
        if (++it > spin_limit()) {
          status_error(st, UPDES_ERR_TIMEOUT);
          atomicCAS(&st->timeout_tag, 0, 3);
          gave_up = true;
          break;
        }
        if (it > 64) __nanosleep(20);
        x = ld_tagged_cg(q);
      }
      (tid < 64 ? wrow : drow)[c] = __uint_as_float(unsigned(x));
    }
    if (__syncthreads_or(gave_up)) return;
    // the published rows still lack the previous column's update for columns >= j + 1
    if (tid < nb) {
      float pr = wrow[tid], dr = drow[tid];
      if (prev_ok && tid > j) {
        pr = __fmaf_rn(-wrow[j - 1], pprev[tid], pr);
        dr = __fmaf_rn(-drow[j - 1], pprev[tid], dr);
      }
      prow[tid] = pr;
      drow[tid] = dr;
    }
    __syncthreads();
    const float pv = prow[j];
    if (tid == 0 && g == 0) {
      piv[diag] = (p == 0x7fffffff) ? diag : p;
      if (pv == 0.f || !isfinite(pv)) atomicCAS(&st->lu_info, 0, diag + 1);
    }
    // interchange rows diag <-> p inside the panel
    if (diag >= rbase && diag < rbase + rcount && tid < nb) tile[int64_t(diag - rbase) * ldt + tid] = prow[tid];
    if (p != diag && p >= rbase && p < rbase + rcount && tid < nb) tile[int64_t(p - rbase) * ldt + tid] = drow[tid];
    __syncthreads();
    const int l0 = max(0, diag + 1 - rbase);
    const bool ok = (pv != 0.f && isfinite(pv));
    // scale column j, update the look-ahead column j + 1 and take this thread's candidate for it on the way
    unsigned key = 0u, crow_i = 0x7fffffffu;
    if (ok) {
      const float rinv = 1.0f / pv;
      for (int l = l0 + tid; l < rcount; l += blockDim.x) {
        float* row = tile + int64_t(l) * ldt;
        row[j] *= rinv;
        if (j + 1 < nb) {
          const float x = __fmaf_rn(-row[j], prow[j + 1], row[j + 1]);  // look-ahead column
          row[j + 1] = x;
          const float ax = fabsf(x);
          const unsigned kv = cand_key((ax != ax) ? INFINITY : ax);
          if (kv > key) { key = kv; crow_i = unsigned(rbase + l); }
        }
      }
    } else if (j + 1 < nb) {
      scan(j + 1, l0, key, crow_i);
    }
    if (j + 1 < nb) publish(j + 1, key, crow_i);
    // rank-1 update of the remaining columns, overlapping the exchange of the next column
    if (ok && j + 2 < nb) {
      // warp w takes rows l0 + w + 8i, four at a time for independent shared-memory traffic; lanes span columns
      const float p0 = (j + 2 + lane < nb) ? prow[j + 2 + lane] : 0.f;
      const float p1 = (j + 34 + lane < nb) ? prow[j + 34 + lane] : 0.f;
      const int c0 = j + 2 + lane, c1 = j + 34 + lane;
      int l = l0 + wid;
      for (; l + 3 * kW < rcount; l += 4 * kW) {
        float* r0 = tile + int64_t(l) * ldt;
        float* r1 = r0 + kW * ldt;
        float* r2 = r1 + kW * ldt;
        float* r3 = r2 + kW * ldt;
        const float a0 = r0[j], a1 = r1[j], a2 = r2[j], a3 = r3[j];
        if (c0 < nb) {
          const float x0 = r0[c0], x1 = r1[c0], x2 = r2[c0], x3 = r3[c0];
          r0[c0] = __fmaf_rn(-a0, p0, x0);
          r1[c0] = __fmaf_rn(-a1, p0, x1);
          r2[c0] = __fmaf_rn(-a2, p0, x2);
          r3[c0] = __fmaf_rn(-a3, p0, x3);
        }
        if (c1 < nb) {
          const float x0 = r0[c1], x1 = r1[c1], x2 = r2[c1], x3 = r3[c1];
          r0[c1] = __fmaf_rn(-a0, p1, x0);
          r1[c1] = __fmaf_rn(-a1, p1, x1);
          r2[c1] = __fmaf_rn(-a2, p1, x2);
          r3[c1] = __fmaf_rn(-a3, p1, x3);
        }
      }
      for (; l < rcount; l += kW) {
        float* r0 = tile + int64_t(l) * ldt;
        const float a0 = r0[j];
        if (c0 < nb) r0[c0] = __fmaf_rn(-a0, p0, r0[c0]);
        if (c1 < nb) r0[c1] = __fmaf_rn(-a0, p1, r0[c1]);
      }
    }
    if (tid < nb) pprev[tid] = prow[tid];
    prev_ok = ok;
    __syncthreads();
  }
  for (int l = wid; l < rcount; l += kW)
    for (int c = lane; c < nb; c += 32) W[int64_t(rbase + l) * ld + k + c] = tile[int64_t(l) * ldt + c];
  if (swap_map && g == 0 && tid < 32) {
    // net permutation of the interchanges piv[k, k+nb): content tracking over <= 2 nb rows
    __shared__ int rows_s[128], cont_s[128];
    for (int i = tid; i < nb; i += 32) rows_s[i] = cont_s[i] = k + i;
    int cnt = nb;
    __syncwarp();
    for (int i = 0; i < nb; ++i) {
      const int pp = piv[k + i];
      if (pp == k + i) continue;
      int found = -1;
      for (int q = tid; q < cnt; q += 32)
        if (rows_s[q] == pp) found = q;
      found = __reduce_max_sync(0xffffffffu, found);
      if (found < 0) {
        if (tid == 0) { rows_s[cnt] = pp; cont_s[cnt] = pp; }
        found = cnt++;
        __syncwarp();
      }
      if (tid == 0) {
        const int a = cont_s[i];
        cont_s[i] = cont_s[found];
        cont_s[found] = a;
      }
      __syncwarp();
    }
    for (int q = tid; q < cnt; q += 32) {
      swap_map[1 + q] = rows_s[q];
      swap_map[129 + q] = cont_s[q];
    }
    if (tid == 0) swap_map[0] = cnt;
  }
}

// Launch the FP32 panel with G <= 32 CTAs when its rows fit; returns UPDES_ERR_UNSUPPORTED otherwise.
int launch_panel_f32(float* W, int64_t ld, int n, int k, int w, int32_t* piv, PanelRec* recs, int32_t* swap_map,
                     DeviceStatus* st, cudaStream_t s) {
  const int m = n - k;
  const int G = std::min(kMaxPanelCtas, int(ceil_div(m, 32)));
  const int rows = int(ceil_div(m, G));
  const size_t smem = (size_t(rows) * (w + 1) + size_t(kMaxPanelCtas + 3) * kLuNb) * sizeof(float);
  if (smem > 200 * 1024) return UPDES_ERR_UNSUPPORTED;
  static std::atomic<unsigned long long> attr{0};
  if (int e = smem_opt_in((const void*)panel_f32_kernel, 200 * 1024, attr)) return e;
  int per_sm = 0;
  UPDES_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, panel_f32_kernel, kPanelF32Threads, smem));
  if (per_sm * num_sms() < G) return UPDES_ERR_UNSUPPORTED;
  int k_ = k, nb_ = w, rows_ = rows, n_ = n;
  int64_t ld_ = ld;
  void* args[] = {&W, &ld_, &n_, &k_, &nb_, &rows_, &piv, &recs, &swap_map, &st};
  StatScope sc(kStatPanel, s, double(m) * w * w, double(m) * w * 8.0);
  UPDES_CUDA_TRY(cudaLaunchCooperativeKernel((void*)panel_f32_kernel, dim3(G), dim3(kPanelF32Threads), args, smem, s));
  stats_count_launch(1);
  return UPDES_OK;
}

size_t lu_panel_workspace_bytes(int nb) {
  const int G = 1024;  // upper bound on panel CTAs
  return 256 + sizeof(DeviceStatus) + 2 * G * sizeof(Cand) + 2ull * G * nb * sizeof(double) + 2ull * nb * sizeof(double);
}

template <typename TF, bool DF_IN>
int launch_panel(void* W, const float* Wlo, int64_t ldw, TF* F, int64_t ldf, int n, int k, int w, int32_t* piv,
                 unsigned int* bar, Cand* cand, double* cand_row, double* diag_row, int32_t* swap_map,
                 DeviceStatus* st, cudaStream_t s) {
  const int sms = num_sms();
  const int m = n - k;
  const size_t esz = DF_IN ? sizeof(float) : sizeof(double);
  // fewer CTAs make each column's candidate exchange cheaper; the FP32 panel fits in 32 CTAs up to ~24k rows
  int G = std::min(DF_IN ? 32 : sms, int(ceil_div(m, 32)));
  int rows = int(ceil_div(m, G));
  size_t smem = (size_t(rows) * w + 2 * w) * esz;
  while (smem > 200 * 1024 && G < 2 * sms) {
    ++G;
    rows = int(ceil_div(m, G));
    smem = (size_t(rows) * w + 2 * w) * esz;
  }
  if (smem > 200 * 1024) return UPDES_ERR_UNSUPPORTED;
  auto kern = panel_kernel<TF, DF_IN>;
  static std::atomic<unsigned long long> attr{0};
  if (int e = smem_opt_in((const void*)kern, 200 * 1024, attr)) return e;
  int per_sm = 0;
  UPDES_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPanelThreads, smem));
  if (per_sm * sms < G) return UPDES_ERR_UNSUPPORTED;
  int k_ = k, nb_ = w, rows_ = rows, n_ = n;
  int64_t ldw_ = ldw, ldf_ = ldf;
  void* args[] = {&W, &Wlo, &ldw_, &F, &ldf_, &n_, &k_, &nb_, &rows_, &piv, &bar, &cand, &cand_row, &diag_row,
                  &swap_map, &st};
  StatScope sc(kStatPanel, s, double(m) * w * w, double(m) * w * 8.0 * 2);
  UPDES_CUDA_TRY(cudaLaunchCooperativeKernel((void*)kern, dim3(G), dim3(kPanelThreads), args, smem, s));
  stats_count_launch(1);
  return UPDES_OK;
}

constexpr int kOuterNb = 4 * kLuNb;   // 256: width of the big exact trailing updates
constexpr int kSwapMapInts = kSwapMapStride;  // one panel's swap map (257 ints used): 2 KB per slot
constexpr int kLookaheadMinN = 1024;  // smaller factorisations run their steps in order on one stream
constexpr int kLookaheadCtas = kMaxPanelCtas;  // SMs kept for the look-ahead block beside the trailing update
// Below this many trailing rows the next block's factorisation (linear in the rows) outlasts the trailing
// update (quadratic): the side stream then forks as soon as the next block's own columns are ready, and the
// rest of the step's interchanges and U row follow beside it.  Above it they stay before the fork, on all
// SMs, where they shorten the update stream that bounds the step.
constexpr int kEarlyForkRows = 12288;

size_t lu_df_workspace_bytes(int n) {
  // panel scratch (rounded up to 256 B), the swap maps of two 256-column blocks' panels, the digit scratch of
  // the trailing update and that of the look-ahead block's own updates (the two run at the same time)
  return ((lu_panel_workspace_bytes(kLuNb) + 255) & ~size_t(255)) + 2 * size_t(kOuterNb / kLuNb) * kSwapMapInts * 4 +
         ozaki3_scratch_bytes(n, n, kOuterNb) + ozaki3_scratch_bytes(n, kOuterNb, kLuNb);
}

namespace {

// The second stream of the look-ahead and the two events that fork it from and join it back to the caller's
// stream.  The destructor joins as well, so that every return path leaves the caller's stream ordered after
// all work of the factorisation.
struct SideStream {
  cudaStream_t main = nullptr, side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  int create(cudaStream_t s) {
    main = s;
    int least = 0, greatest = 0;
    UPDES_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    UPDES_CUDA_TRY(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, greatest));
    UPDES_CUDA_TRY(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    UPDES_CUDA_TRY(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
    return UPDES_OK;
  }
  int start() {  // the side stream waits for all work issued on the caller's stream so far
    UPDES_CUDA_TRY(cudaEventRecord(fork, main));
    UPDES_CUDA_TRY(cudaStreamWaitEvent(side, fork, 0));
    return UPDES_OK;
  }
  int finish() {  // the caller's stream waits for all work issued on the side stream so far
    UPDES_CUDA_TRY(cudaEventRecord(join, side));
    UPDES_CUDA_TRY(cudaStreamWaitEvent(main, join, 0));
    return UPDES_OK;
  }
  ~SideStream() {
    bool bad = false;
    if (side && join) {
      bad |= cudaEventRecord(join, side) != cudaSuccess;
      bad |= cudaStreamWaitEvent(main, join, 0) != cudaSuccess;
    }
    if (fork) bad |= cudaEventDestroy(fork) != cudaSuccess;
    if (join) bad |= cudaEventDestroy(join) != cudaSuccess;
    if (side) bad |= cudaStreamDestroy(side) != cudaSuccess;
    if (bad) (void)cudaGetLastError();
  }
};

void add_swap_job(SwapJobs& j, int64_t& maxc, float* plane, int64_t c0, int64_t c1) {
  if (c1 <= c0) return;
  j.plane[j.njobs] = plane;
  j.c0[j.njobs] = c0;
  j.c1[j.njobs] = c1;
  ++j.njobs;
  maxc = std::max(maxc, c1 - c0);
}

}  // namespace

// Mixed LU of the double-float matrix (Whi, Wlo) with FP32 factors overwriting Whi.  Blocks of 256 columns:
// each block's 64-wide panels are factored with their own updates, then the block row of U is solved and the
// trailing matrix updated by the exact tensor-core update with K = 256.
//
// Look-ahead (n >= kLookaheadMinN): the trailing update after block j is split into the next block's 256
// columns, done first, and the rest.  The next block is then factored on a second stream on kLookaheadCtas
// SMs while the rest of the update runs on the other SMs.  The two touch disjoint data as long as the next
// block's row interchanges stay within its own columns; the interchanges of the columns outside it (the
// factored L to its left, the trailing columns to its right) are kept as one swap map per panel and applied
// in panel order once the update is done, the order in which the serial algorithm applies them.  Every
// entry therefore sees the same operations in the same order and the factors are bitwise those of the
// serial order.
int lu_factor_df(int n, float* Whi, float* Wlo, int64_t ld, int32_t* piv, void* ws, size_t ws_bytes, DeviceStatus* st,
                 cudaStream_t s) {
  const int nb = kLuNb;
  if (ws_bytes < lu_df_workspace_bytes(n)) return UPDES_ERR_WORKSPACE;
  char* base = static_cast<char*>(ws);
  unsigned int* bar = reinterpret_cast<unsigned int*>(base);
  Cand* cand = reinterpret_cast<Cand*>(base + 256);
  double* cand_row = reinterpret_cast<double*>(base + 256 + 2 * 1024 * sizeof(Cand));
  double* diag_row = cand_row + 2ll * 1024 * nb;
  char* after = base + ((lu_panel_workspace_bytes(nb) + 255) & ~size_t(255));
  int32_t* swap_maps = reinterpret_cast<int32_t*>(after);
  char* digits = after + 2 * size_t(kOuterNb / kLuNb) * kSwapMapInts * 4;
  // The swap maps of block [K0, K0 + 256) sit in the half of swap_maps chosen by the block's parity: the
  // look-ahead block's panels write their maps while the caller's stream still applies the previous block's.
  auto block_maps = [&](int K0) { return swap_maps + ((K0 / kOuterNb) & 1) * (kOuterNb / kLuNb) * kSwapMapInts; };
  const size_t digits_bytes = ozaki3_scratch_bytes(n, n, kOuterNb);
  char* digits_la = digits + digits_bytes;
  const size_t digits_la_bytes = ozaki3_scratch_bytes(n, kOuterNb, kLuNb);
  // the persistent TMA-fed update (gemm_tc3.cu); UPDES_OZAKI=2 selects the per-tile kernel of gemm_tc.cu, which
  // also serves updates whose C planes are not 16-byte aligned
  static const bool use_v2 = [] {
    const char* v = std::getenv("UPDES_OZAKI");
    return v && v[0] == '2';
  }();
  // UPDES_LOOKAHEAD=0 runs the block steps in order on the caller's stream (same factors, no overlap)
  static const bool lookahead_on = [] {
    const char* v = std::getenv("UPDES_LOOKAHEAD");
    return !(v && v[0] == '0');
  }();
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  UPDES_CUDA_TRY(cudaStreamIsCapturing(s, &cs));
  const bool lookahead = lookahead_on && !use_v2 && n >= kLookaheadMinN && cs == cudaStreamCaptureStatusNone;
  UPDES_CUDA_TRY(cudaMemsetAsync(bar, 0, 256 + 2 * 1024 * sizeof(Cand), s));  // barrier words and candidate tags
  // the single-exchange panel's records live in the candidate-row area (tags must start at zero)
  PanelRec* recs = reinterpret_cast<PanelRec*>(cand_row);
  static_assert(2 * (kMaxPanelCtas + 1) * sizeof(PanelRec) <= 2 * 1024 * kLuNb * sizeof(double), "panel records");
  UPDES_CUDA_TRY(cudaMemsetAsync(recs, 0, 2 * (kMaxPanelCtas + 1) * sizeof(PanelRec), s));
  constexpr int kOuter = kOuterNb;

  auto swap_launch = [&](const SwapJobs& j, int64_t maxc, const int32_t* map, cudaStream_t us) -> int {
    if (!j.njobs) return UPDES_OK;
    StatScope sc(kStatOther, us, 0.0, 2.0 * 2 * nb * maxc * 4.0 * j.njobs);
    swap_rows_kernel<<<dim3(unsigned(ceil_div(maxc, 64)), j.njobs), 256, 0, us>>>(j, ld, map);
    UPDES_LAUNCH_CHECK();
    return UPDES_OK;
  };
  auto trsm = [&](int k, int w, int64_t c0, int64_t c1, cudaStream_t us) -> int {
    if (c1 <= c0) return UPDES_OK;
    StatScope sc(kStatTrsm, us, double(w) * w * (c1 - c0), double(w) * (c1 - c0) * 12.0);
    if (w == 64) {
      static std::atomic<unsigned long long> attr{0};
      if (int e = smem_opt_in((const void*)trsm_df64_kernel, int(sizeof(TrsmDfSmem)), attr)) return e;
      trsm_df64_kernel<<<unsigned(ceil_div(c1 - c0, 64)), 256, sizeof(TrsmDfSmem), us>>>(Whi, Wlo, ld, k, c0, c1);
    } else {
      trsm_df_kernel<<<unsigned(ceil_div(c1 - c0, 64)), 64, 0, us>>>(Whi, Wlo, ld, k, w, c0, c1);
    }
    UPDES_LAUNCH_CHECK();
    return UPDES_OK;
  };
  // W[r0:r1, c0:c1] -= F[r0:r1, kk0:kk1] * F[kk0:kk1, c0:c1] on stream us with digit scratch dg, at most ctas CTAs
  // The digits of the last A written into each scratch (the update after a block writes them for the next
  // block's columns, and the rest of the trailing matrix has the same A: the block's L rows below it, which
  // nothing changes in between; any other update on that scratch replaces them).
  struct ADigits {
    const void* dg = nullptr;
    int r0 = -1, r1 = -1, kk0 = -1, kk1 = -1;
  } a_main, a_side;
  auto upd = [&](int r0, int r1, int c0, int c1, int kk0, int kk1, cudaStream_t us, void* dg, size_t dgb,
                 int ctas) -> int {
    if (!use_v2) {
      ADigits& last = (dg == digits) ? a_main : a_side;
      const bool a_ready = last.dg == dg && last.r0 == r0 && last.r1 == r1 && last.kk0 == kk0 && last.kk1 == kk1;
      const int e3 = ozaki3_update(Whi + int64_t(r0) * ld + c0, Wlo + int64_t(r0) * ld + c0, ld,
                                   Whi + int64_t(r0) * ld + kk0, ld, Whi + int64_t(kk0) * ld + c0, ld, r1 - r0,
                                   c1 - c0, kk1 - kk0, dg, dgb, st, us, ctas, a_ready);
      last = e3 == UPDES_OK ? ADigits{dg, r0, r1, kk0, kk1} : ADigits{};
      if (e3 != UPDES_ERR_UNSUPPORTED) return e3;
    }
    return ozaki_update(Whi + int64_t(r0) * ld + c0, Wlo + int64_t(r0) * ld + c0, ld, Whi + int64_t(r0) * ld + kk0,
                        ld, Whi + int64_t(kk0) * ld + c0, ld, r1 - r0, c1 - c0, kk1 - kk0, st, us);
  };
  // Columns [K0, KE): panels, their interchanges and the block's own updates.  `deferred`: the interchanges
  // touch only the block's columns, and panel p's swap map stays in slot p for the columns outside.
  auto factor_block = [&](int K0, int KE, bool deferred, cudaStream_t us, int ctas) -> int {
    int e;
    for (int k = K0, p = 0; k < KE; k += nb, ++p) {
      const int w = std::min(nb, KE - k);
      int32_t* map = block_maps(K0) + p * kSwapMapInts;
      e = launch_panel_f32(Whi, ld, n, k, w, piv, recs, map, st, us);
      if (e == UPDES_ERR_UNSUPPORTED)
        e = launch_panel<float, true>(Whi, Wlo, ld, Whi, ld, n, k, w, piv, bar, cand, cand_row, diag_row, map, st,
                                      us);
      if (e) return e;
      SwapJobs j{};
      int64_t maxc = 0;
      add_swap_job(j, maxc, Whi, k + w, deferred ? KE : n);
      add_swap_job(j, maxc, Wlo, k + w, deferred ? KE : n);
      add_swap_job(j, maxc, Whi, deferred ? K0 : 0, k);  // factored columns: the FP32 factors only
      if ((e = swap_launch(j, maxc, map, us))) return e;
      if (k + w < KE) {
        if ((e = trsm(k, w, k + w, KE, us))) return e;
        if ((e = upd(k + w, n, k + w, KE, k, k + w, us, deferred ? digits_la : digits,
                     deferred ? digits_la_bytes : digits_bytes, ctas)))
          return e;
      }
    }
    return UPDES_OK;
  };
  // The deferred interchanges of block [K0, KE), panel by panel, on trailing columns [c0, c1) (both planes)
  // and, with left, on the factored columns [0, K0) (the FP32 factors).
  // All the block's panels in one launch: each column chunk applies their maps in panel order.
  auto swaps_deferred = [&](int K0, int KE, int c0, int c1, bool left) -> int {
    SwapJobs j{};
    int64_t maxc = 0;
    if (left) add_swap_job(j, maxc, Whi, 0, K0);
    add_swap_job(j, maxc, Whi, c0, c1);
    add_swap_job(j, maxc, Wlo, c0, c1);
    if (!j.njobs) return UPDES_OK;
    const int nmaps = int(ceil_div(KE - K0, nb));
    StatScope sc(kStatOther, s, 0.0, 2.0 * 2 * nb * maxc * 4.0 * j.njobs * nmaps);
    swap_rows_maps_kernel<<<dim3(unsigned(ceil_div(maxc, 64)), j.njobs), 256, 0, s>>>(j, ld, block_maps(K0), nmaps);
    UPDES_LAUNCH_CHECK();
    return UPDES_OK;
  };
  // Block row of U for block [K0, KE) on trailing columns [c0, c1), the updates on at most ctas CTAs.
  auto block_row = [&](int K0, int KE, int c0, int c1, int ctas) -> int {
    for (int b = K0; b < KE; b += nb) {
      const int w = std::min(nb, KE - b);
      if (int e = trsm(b, w, c0, c1, s)) return e;
      if (b + w < KE)
        if (int e = upd(b + w, KE, c0, c1, b, b + w, s, digits, digits_bytes, ctas)) return e;
    }
    return UPDES_OK;
  };

  SideStream side;
  int e;
  if (lookahead && (e = side.create(s))) return e;
  const int rest_ctas = std::max(num_sms() - kLookaheadCtas, num_sms() / 2);
  // UPDES_EARLY_FORK_ROWS overrides kEarlyForkRows (same factors either way)
  static const int early_rows = [] {
    const char* v = std::getenv("UPDES_EARLY_FORK_ROWS");
    return v ? std::atoi(v) : kEarlyForkRows;
  }();
  int K0 = 0, KE = std::min(kOuter, n);
  if ((e = factor_block(K0, KE, false, s, 0))) return e;
  bool pending = false;  // block [K0, KE) was factored beside the update: its outside interchanges are due
  while (KE < n) {
    const int KE2 = std::min(KE + kOuter, n);
    const bool early_fork = lookahead && KE2 < n && n - KE <= early_rows;
    // what the next block [KE, KE2) needs before it can be factored: this block's interchanges, U row and
    // update on its columns (with an early fork), or on all trailing columns
    const int c1 = early_fork ? KE2 : n;
    if (pending && (e = swaps_deferred(K0, KE, KE, c1, !early_fork))) return e;
    if ((e = block_row(K0, KE, KE, c1, 0))) return e;
    if ((e = upd(KE, n, KE, KE2, K0, KE, s, digits, digits_bytes, 0))) return e;
    if (lookahead && KE2 < n) {
      // the next block on the side stream; the rest of this step on this stream, on the SMs it leaves
      if ((e = side.start())) return e;
      if ((e = factor_block(KE, KE2, true, side.side, kLookaheadCtas))) return e;
      if (early_fork) {
        if (pending && (e = swaps_deferred(K0, KE, KE2, n, true))) return e;
        if ((e = block_row(K0, KE, KE2, n, rest_ctas))) return e;
      }
      if ((e = upd(KE, n, KE2, n, K0, KE, s, digits, digits_bytes, rest_ctas))) return e;
      if ((e = side.finish())) return e;
      pending = true;
    } else {
      if (KE2 < n && (e = upd(KE, n, KE2, n, K0, KE, s, digits, digits_bytes, 0))) return e;
      if ((e = factor_block(KE, KE2, false, s, 0))) return e;
      pending = false;
    }
    K0 = KE;
    KE = KE2;
  }
  return UPDES_OK;
}

template <typename TF>
int lu_factor_impl(int n, double* W, int64_t ldw, TF* F, int64_t ldf, int32_t* piv, void* ws, size_t ws_bytes,
                   DeviceStatus* st, cudaStream_t s, const LuHooks* hooks) {
  const int nb = kLuNb;
  if (ws_bytes < lu_panel_workspace_bytes(nb)) return UPDES_ERR_WORKSPACE;
  char* base = static_cast<char*>(ws);
  unsigned int* bar = reinterpret_cast<unsigned int*>(base);
  Cand* cand = reinterpret_cast<Cand*>(base + 256);
  double* cand_row = reinterpret_cast<double*>(base + 256 + 2 * 1024 * sizeof(Cand));
  double* diag_row = cand_row + 2ll * 1024 * nb;
  UPDES_CUDA_TRY(cudaMemsetAsync(bar, 0, 256 + 2 * 1024 * sizeof(Cand), s));  // barrier words and candidate tags
  // the single-exchange panel's records live in the candidate-row area (tags must start at zero)
  PanelRec* recs = reinterpret_cast<PanelRec*>(cand_row);
  static_assert(2 * (kMaxPanelCtas + 1) * sizeof(PanelRec) <= 2 * 1024 * kLuNb * sizeof(double), "panel records");
  UPDES_CUDA_TRY(cudaMemsetAsync(recs, 0, 2 * (kMaxPanelCtas + 1) * sizeof(PanelRec), s));
  for (int k = 0; k < n; k += nb) {
    const int w = std::min(nb, n - k);
    {
      int e = launch_panel<TF, false>(W, nullptr, ldw, F, ldf, n, k, w, piv, bar, cand, cand_row, diag_row,
                                      nullptr, st, s);
      if (e) return e;
    }
    // row interchanges: factored columns [0, k) of F, trailing columns [k+w, n) of W
    if (k > 0) {
      laswp_kernel<TF><<<unsigned(ceil_div(k, 256)), 256, 0, s>>>(F, ldf, piv, k, w, 0, k);
      UPDES_LAUNCH_CHECK();
    }
    if (k + w < n) {
      laswp_kernel<double><<<unsigned(ceil_div(n - k - w, 256)), 256, 0, s>>>(W, ldw, piv, k, w, k + w, n);
      UPDES_LAUNCH_CHECK();
      {
        StatScope sc(kStatTrsm, s, double(w) * w * (n - k - w), double(w) * (n - k - w) * (8.0 + sizeof(TF)));
        trsm_kernel<TF><<<unsigned(ceil_div(n - k - w, 64)), 64, size_t(w) * w * sizeof(double), s>>>(W, ldw, F, ldf, n, k, w);
        UPDES_LAUNCH_CHECK();
      }
      const double mm = double(n - k - w);
      StatScope sc(kStatGemm, s, 2.0 * mm * mm * w, mm * mm * 16.0 + 2.0 * mm * w * sizeof(TF));
      if (hooks && hooks->gemm) {
        int e = hooks->gemm(hooks->ctx, n, k, w, W, ldw, F, ldf, s);
        if (e) return e;
      } else {
        dim3 grid(unsigned(ceil_div(n - k - w, 64)), unsigned(ceil_div(n - k - w, 64)));
        gemm_update_kernel<TF><<<grid, 256, 0, s>>>(W, ldw, F, ldf, n, k, w);
        UPDES_LAUNCH_CHECK();
      }
    }
  }
  return UPDES_OK;
}

template int lu_factor_impl<double>(int, double*, int64_t, double*, int64_t, int32_t*, void*, size_t, DeviceStatus*,
                                    cudaStream_t, const LuHooks*);
template int lu_factor_impl<float>(int, double*, int64_t, float*, int64_t, int32_t*, void*, size_t, DeviceStatus*,
                                   cudaStream_t, const LuHooks*);

// ---------------------------------------------------------------------------
// Triangular solves (single right-hand side, FP64 arithmetic on TF factors).
// One launch per triangle; CTAs take block rows in ticket order and wait
// (bounded) on the flags of the blocks they depend on.
// ---------------------------------------------------------------------------
namespace {

constexpr int kTB = 64;

// mode: 0 = L (unit lower, forward), 1 = U (upper, backward),
//       2 = U^T (lower with U's diagonal, forward), 3 = L^T (unit upper, backward)
// Off-diagonal 64 x 64 tiles are read coalesced (transposed through shared memory for modes 2/3) with the
// next tile prefetched into registers while the current one is used.  FP32 factors are applied in
// double-float arithmetic (exact products via FMA, compensated sums), FP64 factors in FP64.
__device__ __forceinline__ void df_fma(float f, float xh, float xl, float& sh, float& sl) {
  const float p = __fmul_rn(f, xh);
  const float e = __fmaf_rn(f, xh, -p);  // exact error of the product
  const float s = __fadd_rn(sh, p);
  const float bb = __fsub_rn(s, sh);
  float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  t = __fadd_rn(t, __fadd_rn(sl, __fmaf_rn(f, xl, e)));
  sh = __fadd_rn(s, t);  // renormalised after every term
  sl = __fsub_rn(t, __fsub_rn(sh, s));
}

// Warp-wide sum of a double-float pair with FP32 instructions (FP64 adds would queue on the SM's few FP64
// units): every lane ends with the total.
__device__ __forceinline__ void df_warp_sum(float& h, float& l) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, h, o), ol = __shfl_xor_sync(0xffffffffu, l, o);
    const float s = __fadd_rn(h, oh);
    const float bb = __fsub_rn(s, h);
    float t = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(oh, bb));
    t = __fadd_rn(t, __fadd_rn(l, ol));
    h = __fadd_rn(s, t);
    l = __fsub_rn(t, __fsub_rn(h, s));
  }
}

// (qh, ql) = (bh + bl) / d for an FP32 divisor d
__device__ __forceinline__ void df_div1(float bh, float bl, float d, float& qh, float& ql) {
  const float q1 = __fdiv_rn(bh, d);
  const float p = __fmul_rn(q1, d);
  const float pe = __fmaf_rn(q1, d, -p);  // q1 * d = p + pe exactly
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(bh, p), pe), bl);
  const float q2 = __fdiv_rn(r, d);
  qh = __fadd_rn(q1, q2);
  ql = __fsub_rn(q2, __fsub_rn(qh, q1));
}

template <typename TF, int MODE>
__global__ void __launch_bounds__(256) trsv_kernel(const TF* __restrict__ F, int64_t ldf, int n, double* x,
                                                   int* ticket, int* flags, DeviceStatus* st,
                                                   const float* __restrict__ dinv) {
  extern __shared__ __align__(16) unsigned char trsv_smem[];
  TF(*sT)[kTB + 1] = reinterpret_cast<TF(*)[kTB + 1]>(trsv_smem);
  double* sxd = reinterpret_cast<double*>(trsv_smem + sizeof(TF) * kTB * (kTB + 1));  // 64
  float* sxh = reinterpret_cast<float*>(sxd + kTB);                                    // 64
  float* sxl = sxh + kTB;                                                              // 64
  double* sacc = reinterpret_cast<double*>(sxl + kTB);                                 // 64
  float(*sDl)[kTB + 1] = reinterpret_cast<float(*)[kTB + 1]>(sacc + kTB);              // 64 x 65 (dinv only)
  float(*sDh)[kTB + 1] = sDl + kTB;                                                    // 64 x 65 (dinv only)
  __shared__ int s_blk;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nblk = int(ceil_div(n, kTB));
  if (tid == 0) s_blk = atomicAdd(ticket, 1);
  __syncthreads();
  const int t = s_blk;
  if (t >= nblk) return;
  constexpr bool fwd = (MODE == 0 || MODE == 2);
  constexpr bool trans = (MODE >= 2);
  const int blk = fwd ? t : nblk - 1 - t;
  const int r0 = blk * kTB;
  const int rows = min(kTB, n - r0);
  // inputs that no other block writes, fetched before any wait: this block's right-hand side and, with
  // dinv, its inverted diagonal block (modes 2 and 3 use the transposes of the U and L inverses)
  const double b_own = (tid < rows) ? x[r0 + tid] : 0.0;
  if constexpr (sizeof(TF) == 4) {
    if (dinv) {
      constexpr int which = (MODE == 0 || MODE == 3) ? 0 : 1;  // 0: inv(L_bb), 1: inv(U_bb)
      constexpr bool tr = (MODE >= 2);
      const float* Dh = dinv + (size_t(blk) * 4 + which * 2) * kTB * kTB;
      const float* Dlo = Dh + kTB * kTB;
      for (int e = tid; e < kTB * kTB; e += blockDim.x) {
        const int a = e >> 6, b = e & 63;
        const int ra = tr ? b : a, cb = tr ? a : b;
        sDh[ra][cb] = __ldg(Dh + e);
        sDl[ra][cb] = __ldg(Dlo + e);
      }
    }
  }

  auto load_tile = [&](int c0, TF (&pre)[16]) {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int e = tid + 256 * i;
      const int a = e >> 6, b = e & 63;  // a: source row in the tile, b: source column
      TF v = TF(0);
      if (!trans) {
        if (r0 + a < n && c0 + b < n) v = F[int64_t(r0 + a) * ldf + c0 + b];
      } else {
        if (c0 + a < n && r0 + b < n) v = F[int64_t(c0 + a) * ldf + r0 + b];
      }
      pre[i] = v;
    }
  };
  auto store_tile = [&](const TF (&pre)[16]) {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int e = tid + 256 * i;
      const int a = e >> 6, b = e & 63;
      if (!trans) sT[a][b] = pre[i];
      else sT[b][a] = pre[i];
    }
  };

  // per-warp rows w*8 .. w*8+7, lane columns lane, lane+32
  float ah[8], al[8];
  double ad[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) { ah[i] = 0.f; al[i] = 0.f; ad[i] = 0.0; }
  TF pre[16];
  if (t > 0) load_tile((fwd ? 0 : nblk - 1) * kTB, pre);
  // Blocks finish in ticket order (each waits for all earlier ones), so flags[nblk] counts finished
  // blocks: a CTA re-reads it only when it needs a block beyond the last count it saw.
  __shared__ int s_done;
  if (tid == 0) s_done = 0;
  for (int q = 0; q < t; ++q) {
    const int jb = fwd ? q : nblk - 1 - q;
    const int c0 = jb * kTB;
    const int cols = min(kTB, n - c0);
    if (tid == 0 && s_done <= q) {
      volatile int* vc = flags + nblk;
      long long it = 0;
      int d;
      while ((d = *vc) <= q) {
        if (++it > spin_limit()) {
          status_error(st, UPDES_ERR_TIMEOUT);
          atomicCAS(&st->timeout_tag, 0, 10 + MODE);
          d = q + 1;
          break;
        }
        __nanosleep(20);
      }
      __threadfence();
      s_done = d;
    }
    __syncthreads();
    store_tile(pre);
    if (tid < kTB) {
      const double v = tid < cols ? __ldcg(x + c0 + tid) : 0.0;
      sxd[tid] = v;
      const float h = float(v);
      sxh[tid] = h;
      sxl[tid] = float(v - double(h));
    }
    __syncthreads();
    if (q + 1 < t) load_tile((fwd ? q + 1 : nblk - 2 - q) * kTB, pre);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int rr = warp * 8 + i;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int cc = lane + 32 * h;
        if constexpr (sizeof(TF) == 4) df_fma(float(sT[rr][cc]), sxh[cc], sxl[cc], ah[i], al[i]);
        else ad[i] = fma(double(sT[rr][cc]), sxd[cc], ad[i]);
      }
    }
    __syncthreads();
  }
  if constexpr (sizeof(TF) == 4) {
    if (dinv) {
      // row sums of the off-diagonal part in double-float (FP32 pipes), kept as two FP32 words
      float* sacc_h = reinterpret_cast<float*>(sacc);
      float* sacc_l = sacc_h + kTB;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        float h = ah[i], l = al[i];
        df_warp_sum(h, l);
        if (lane == 0) {
          sacc_h[warp * 8 + i] = h;
          sacc_l[warp * 8 + i] = l;
        }
      }
      // x_blk = D (b - off-diagonal part), D the inverted diagonal block (double-float planes, prefetched):
      // a matvec, no dependent chain
      __syncthreads();
      if (tid < kTB) {
        // b - acc in double-float: b split once, then a two-sum
        const float bh = float(b_own), bl = float(b_own - double(bh));
        float rh = 0.f, rl = 0.f;
        if (tid < rows) {
          const float ch = -sacc_h[tid], cl = -sacc_l[tid];
          const float s0 = __fadd_rn(bh, ch);
          const float bb = __fsub_rn(s0, bh);
          float t = __fadd_rn(__fsub_rn(bh, __fsub_rn(s0, bb)), __fsub_rn(ch, bb));
          t = __fadd_rn(t, __fadd_rn(bl, cl));
          rh = __fadd_rn(s0, t);
          rl = __fsub_rn(t, __fsub_rn(rh, s0));
        }
        sxh[tid] = rh;
        sxl[tid] = rl;
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int rr = warp * 8 + i;
        float ph = 0.f, pl = 0.f;
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          const int cc = lane + 32 * hh;
          const float dh = sDh[rr][cc], dl = sDl[rr][cc];
          // (ph, pl) += (dh + dl)(xh + xl), dropping dl * xl
          const float p = __fmul_rn(dh, sxh[cc]);
          const float pe = __fmaf_rn(dh, sxh[cc], -p);
          const float s0 = __fadd_rn(ph, p);
          const float bb = __fsub_rn(s0, ph);
          float t = __fadd_rn(__fsub_rn(ph, __fsub_rn(s0, bb)), __fsub_rn(p, bb));
          t = __fadd_rn(t, __fadd_rn(pl, __fmaf_rn(dh, sxl[cc], __fmaf_rn(dl, sxh[cc], pe))));
          ph = __fadd_rn(s0, t);
          pl = __fsub_rn(t, __fsub_rn(ph, s0));
        }
        df_warp_sum(ph, pl);
        if (lane == 0 && rr < rows) x[r0 + rr] = double(ph) + double(pl);
      }
      __syncthreads();
      if (tid == 0) {
        __threadfence();
        atomicAdd(flags + nblk, 1);  // blocks finish in order: this is block number t
      }
      return;
    }
  }
  // row sums of the off-diagonal part
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    double v = (sizeof(TF) == 4) ? double(ah[i]) + double(al[i]) : ad[i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sacc[warp * 8 + i] = v;
  }
  // diagonal block
  {
    TF dpre[16];
    load_tile(r0, dpre);
    store_tile(dpre);
  }
  __syncthreads();
  __shared__ double s_rdiag[kTB];
  constexpr bool unit = (MODE == 0 || MODE == 3);
  if (sizeof(TF) == 8 && !unit && tid < rows) s_rdiag[tid] = 1.0 / double(sT[tid][tid]);
  __syncthreads();
  if (sizeof(TF) == 4 && tid < 32) {
    // FP32 factors: the same column-oriented substitution in double-float arithmetic on the FP32 pipes
    // (one warp's FP64 instructions would serialise on the SM's few FP64 units)
    float v0h = 0.f, v0l = 0.f, v1h = 0.f, v1l = 0.f;
    if (tid < rows) {
      const double v = x[r0 + tid] - sacc[tid];
      v0h = float(v);
      v0l = float(v - double(v0h));
    }
    if (tid + 32 < rows) {
      const double v = x[r0 + tid + 32] - sacc[tid + 32];
      v1h = float(v);
      v1l = float(v - double(v1h));
    }
    for (int s2 = 0; s2 < rows; ++s2) {
      const int i = fwd ? s2 : rows - 1 - s2;
      const bool hi_slot = (i >> 5) != 0;
      float xh = __shfl_sync(0xffffffffu, hi_slot ? v1h : v0h, i & 31);
      float xl = __shfl_sync(0xffffffffu, hi_slot ? v1l : v0l, i & 31);
      if (!unit) df_div1(xh, xl, float(sT[i][i]), xh, xl);
      if ((i & 31) == tid) {
        if (hi_slot) { v1h = xh; v1l = xl; }
        else { v0h = xh; v0l = xl; }
      }
      const int ra = tid, rb = tid + 32;
      if (fwd ? ra > i : ra < i) df_fma(-float(sT[ra][i]), xh, xl, v0h, v0l);
      if (rb < rows && (fwd ? rb > i : rb < i)) df_fma(-float(sT[rb][i]), xh, xl, v1h, v1l);
    }
    if (tid < rows) x[r0 + tid] = double(v0h) + double(v0l);
    if (tid + 32 < rows) x[r0 + tid + 32] = double(v1h) + double(v1l);
  } else if (sizeof(TF) == 8 && tid < 32) {
    // column-oriented substitution: lane owns rows lane and lane+32; x_i is broadcast by one shuffle and
    // every unsolved row is updated right away (no global loads on the dependent chain)
    double v0 = 0.0, v1 = 0.0;
    if (tid < rows) v0 = x[r0 + tid] - sacc[tid];
    if (tid + 32 < rows) v1 = x[r0 + tid + 32] - sacc[tid + 32];
    for (int s2 = 0; s2 < rows; ++s2) {
      const int i = fwd ? s2 : rows - 1 - s2;
      double xi = __shfl_sync(0xffffffffu, (i >> 5) ? v1 : v0, i & 31);
      if (!unit) xi *= s_rdiag[i];
      if ((i & 31) == tid) {
        if (i >> 5) v1 = xi;
        else v0 = xi;
      }
      const int ra = tid, rb = tid + 32;
      if (fwd ? ra > i : ra < i) v0 -= double(sT[ra][i]) * xi;
      if (rb < rows && (fwd ? rb > i : rb < i)) v1 -= double(sT[rb][i]) * xi;
    }
    if (tid < rows) x[r0 + tid] = v0;
    if (tid + 32 < rows) x[r0 + tid + 32] = v1;
  }
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    atomicAdd(flags + nblk, 1);  // blocks finish in order: this is block number t
  }
}

}  // namespace

// (h, l) += (a, b) across the 4 lanes of an aligned group (double-float, FP32 instructions)
__device__ __forceinline__ void df_quad_sum(float& h, float& l) {
#pragma unroll
  for (int o = 1; o <= 2; o <<= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, h, o), ol = __shfl_xor_sync(0xffffffffu, l, o);
    const float s = __fadd_rn(h, oh);
    const float bb = __fsub_rn(s, h);
    float t = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(oh, bb));
    t = __fadd_rn(t, __fadd_rn(l, ol));
    h = __fadd_rn(s, t);
    l = __fsub_rn(t, __fsub_rn(h, s));
  }
}

// Triangular solve with FP32 factors and inverted diagonal blocks (the refinement's preconditioner).
// Same ticket/done-counter chain as trsv_kernel, arranged for a short critical path: four threads per row
// (16 columns each, so every reduction is two shuffles), the block's right-hand side split into
// double-float before the wait, and every solved block published twice, as FP64 x and as the double-float
// planes xh/xl that the later blocks read (no FP64 conversions on the chain).
template <int MODE>
__global__ void __launch_bounds__(256) trsv_f32_kernel(const float* __restrict__ F, int64_t ldf, int n, double* x,
                                                       float* xh_g, float* xl_g, int* ticket, int* flags,
                                                       DeviceStatus* st, const float* __restrict__ dinv) {
  __shared__ float sT[kTB][kTB + 1];
  extern __shared__ __align__(16) unsigned char tf_smem[];
  float(*sDh)[kTB + 1] = reinterpret_cast<float(*)[kTB + 1]>(tf_smem);
  float(*sDl)[kTB + 1] = sDh + kTB;
  __shared__ float sxh[kTB], sxl[kTB], srh[kTB], srl[kTB];
  __shared__ int s_blk, s_done;
  const int tid = threadIdx.x;
  const int nblk = int(ceil_div(n, kTB));
  if (tid == 0) {
    s_blk = atomicAdd(ticket, 1);
    s_done = 0;
  }
  __syncthreads();
  const int t = s_blk;
  if (t >= nblk) return;
  constexpr bool fwd = (MODE == 0 || MODE == 2);
  constexpr bool trans = (MODE >= 2);
  const int blk = fwd ? t : nblk - 1 - t;
  const int r0 = blk * kTB;
  const int rows = min(kTB, n - r0);
  const int row = tid >> 2, part = tid & 3;
  // inputs no other block writes, fetched before any wait
  float bh = 0.f, bl = 0.f;
  if (part == 0 && row < rows) {
    const double b = x[r0 + row];
    bh = float(b);
    bl = float(b - double(bh));
  }
  {
    constexpr int which = (MODE == 0 || MODE == 3) ? 0 : 1;  // 0: inv(L_bb), 1: inv(U_bb); transposed for 2, 3
    const float* Dh = dinv + (size_t(blk) * 4 + which * 2) * kTB * kTB;
    const float* Dlo = Dh + kTB * kTB;
    for (int e = tid; e < kTB * kTB; e += blockDim.x) {
      const int a = e >> 6, b = e & 63;
      const int ra = trans ? b : a, cb = trans ? a : b;
      sDh[ra][cb] = __ldg(Dh + e);
      sDl[ra][cb] = __ldg(Dlo + e);
    }
  }
  auto load_tile = [&](int c0, float (&pre)[16]) {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int e = tid + 256 * i;
      const int a = e >> 6, b = e & 63;
      float v = 0.f;
      if (!trans) {
        if (r0 + a < n && c0 + b < n) v = F[int64_t(r0 + a) * ldf + c0 + b];
      } else {
        if (c0 + a < n && r0 + b < n) v = F[int64_t(c0 + a) * ldf + r0 + b];
      }
      pre[i] = v;
    }
  };
  float pre[16];
  if (t > 0) load_tile((fwd ? 0 : nblk - 1) * kTB, pre);
  float ah = 0.f, al = 0.f;
  for (int q = 0; q < t; ++q) {
    const int jb = fwd ? q : nblk - 1 - q;
    const int c0 = jb * kTB;
    const int cols = min(kTB, n - c0);
    if (tid == 0 && s_done <= q) {
      volatile int* vc = flags + nblk;
      long long it = 0;
      int d;
      while ((d = *vc) <= q) {
        if (++it > spin_limit()) {
          status_error(st, UPDES_ERR_TIMEOUT);
          atomicCAS(&st->timeout_tag, 0, 20 + MODE);
          d = q + 1;
          break;
        }
        __nanosleep(20);
      }
      __threadfence();
      s_done = d;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int e = tid + 256 * i;
      const int a = e >> 6, b = e & 63;
      if (!trans) sT[a][b] = pre[i];
      else sT[b][a] = pre[i];
    }
    if (tid < kTB) {
      sxh[tid] = tid < cols ? __ldcg(xh_g + c0 + tid) : 0.f;
      sxl[tid] = tid < cols ? __ldcg(xl_g + c0 + tid) : 0.f;
    }
    __syncthreads();
    if (q + 1 < t) load_tile((fwd ? q + 1 : nblk - 2 - q) * kTB, pre);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const int c = part * 16 + ((k + 4 * part) & 15);  // rotated per part: fewer bank conflicts
      df_fma(sT[row][c], sxh[c], sxl[c], ah, al);
    }
    __syncthreads();
  }
  df_quad_sum(ah, al);
  if (part == 0) {
    // right-hand side of this block minus the off-diagonal part, double-float
    float rh = 0.f, rl = 0.f;
    if (row < rows) {
      const float ch = -ah, cl = -al;
      const float s0 = __fadd_rn(bh, ch);
      const float bb = __fsub_rn(s0, bh);
      float tt = __fadd_rn(__fsub_rn(bh, __fsub_rn(s0, bb)), __fsub_rn(ch, bb));
      tt = __fadd_rn(tt, __fadd_rn(bl, cl));
      rh = __fadd_rn(s0, tt);
      rl = __fsub_rn(tt, __fsub_rn(rh, s0));
    }
    srh[row] = rh;
    srl[row] = rl;
  }
  __syncthreads();
  // x_blk = D (b - off-diagonal part)
  float ph = 0.f, pl = 0.f;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const int c = part * 16 + ((k + 4 * part) & 15);
    const float dh = sDh[row][c], dl = sDl[row][c], xh = srh[c], xl = srl[c];
    const float p = __fmul_rn(dh, xh);
    const float pe = __fmaf_rn(dh, xh, -p);
    const float s0 = __fadd_rn(ph, p);
    const float bb = __fsub_rn(s0, ph);
    float tt = __fadd_rn(__fsub_rn(ph, __fsub_rn(s0, bb)), __fsub_rn(p, bb));
    tt = __fadd_rn(tt, __fadd_rn(pl, __fmaf_rn(dh, xl, __fmaf_rn(dl, xh, pe))));
    ph = __fadd_rn(s0, tt);
    pl = __fsub_rn(tt, __fsub_rn(ph, s0));
  }
  df_quad_sum(ph, pl);
  if (part == 0 && row < rows) {
    xh_g[r0 + row] = ph;
    xl_g[r0 + row] = pl;
    x[r0 + row] = double(ph) + double(pl);
  }
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    atomicAdd(flags + nblk, 1);  // blocks finish in order: this is block number t
  }
}

// (ah, al) += (bh, bl), renormalised.
__device__ __forceinline__ void df_add_to(float& ah, float& al, float bh, float bl) {
  const float s0 = __fadd_rn(ah, bh);
  const float bb = __fsub_rn(s0, ah);
  float t = __fadd_rn(__fsub_rn(ah, __fsub_rn(s0, bb)), __fsub_rn(bh, bb));
  t = __fadd_rn(t, __fadd_rn(al, bl));
  ah = __fadd_rn(s0, t);
  al = __fsub_rn(t, __fsub_rn(ah, s0));
}

// df_fma on two independent column pairs at once with the packed FP32x2 instructions of sm_100+ (one
// issue slot per pair); y - x is fma(x, -1, y), which rounds once like a subtraction.
__device__ __forceinline__ float2 sub2(float2 y, float2 x) { return __ffma2_rn(x, make_float2(-1.f, -1.f), y); }

__device__ __forceinline__ void df_fma_x2(float2 f, float2 fl, float2 xh, float2 xl, float2& sh, float2& sl) {
  const float2 p = __fmul2_rn(f, xh);
  const float2 pe = __ffma2_rn(f, xh, make_float2(-p.x, -p.y));
  const float2 s0 = __fadd2_rn(sh, p);
  const float2 bb = sub2(s0, sh);
  float2 t = __fadd2_rn(sub2(sh, sub2(s0, bb)), sub2(p, bb));
  t = __fadd2_rn(t, __fadd2_rn(sl, __ffma2_rn(f, xl, __ffma2_rn(fl, xh, pe))));
  sh = __fadd2_rn(s0, t);
  sl = sub2(t, sub2(sh, s0));
}

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// The same triangular solve in blocks of 128 rows, one CTA of 512 threads each: the chain of blocks (an L2
// hand-off per block) is half as long.  Off-diagonal 128 x 128 tiles are applied as in trsv_f32_kernel
// (four threads per row, 32 columns each, two independent accumulators); each prefetched tile is stored to
// shared memory before its block's flag is awaited, so that only the solved x and the arithmetic follow
// the flag.  The diagonal block is one matrix-vector product with its inverse (diag_inverse128).
constexpr int kTB2 = 2 * kTB;
constexpr int kT2S = kTB2 + 2;  // even row stride: column pairs load as aligned 8-byte vectors
constexpr size_t kTrsv128Smem = sizeof(float) * 3 * size_t(kTB2) * kT2S;

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// With xtag, a solved block hands its x to the blocks after it through tagged words: row i's hi and lo parts
// go to xtag[2i] and xtag[2i + 1] as (block + 1) << 32 | float bits, each one single-copy-atomic 8-byte store,
// so a reader that sees its block's tag has the value, with no flag, no fence and no second round trip.  The
// words are cleared before every call, so a tag can only come from the current call.
// VEC (untransposed modes, factors 16-byte aligned with a row stride of whole 16-byte vectors): tiles move as
// 16-byte vectors.
template <int MODE, bool VEC = false>
__global__ void __launch_bounds__(512) trsv128_f32_kernel(const float* __restrict__ F, int64_t ldf, int n, double* x,
                                                          float* xh_g, float* xl_g, int* ticket, int* flags,
                                                          DeviceStatus* st, const float* __restrict__ dinv128,
                                                          unsigned long long* xtag) {
  extern __shared__ __align__(16) unsigned char t128_smem[];
  float(*sT)[kT2S] = reinterpret_cast<float(*)[kT2S]>(t128_smem);
  float(*sDh)[kT2S] = sT + kTB2;
  float(*sDl)[kT2S] = sDh + kTB2;
  __shared__ __align__(8) float sxh[kTB2], sxl[kTB2], srh[kTB2], srl[kTB2];
  __shared__ int s_blk, s_done;
  const int tid = threadIdx.x;
  const int nblk = int(ceil_div(n, kTB2));
  if (tid == 0) {
    s_blk = atomicAdd(ticket, 1);
    s_done = 0;
  }
  __syncthreads();
  const int t = s_blk;
  if (t >= nblk) return;
  constexpr bool fwd = (MODE == 0 || MODE == 2);
  constexpr bool trans = (MODE >= 2);
  const int blk = fwd ? t : nblk - 1 - t;
  const int r0 = blk * kTB2;
  const int rows = min(kTB2, n - r0);
  const int row = tid >> 2, part = tid & 3;
  // inputs no other block writes, fetched before any wait: the right-hand side and the inverse block
  float bh = 0.f, bl = 0.f;
  if (part == 0 && row < rows) {
    const double b = x[r0 + row];
    bh = float(b);
    bl = float(b - double(bh));
  }
  {
    constexpr int which = (MODE == 0 || MODE == 3) ? 0 : 1;  // 0: inv(L_bb), 1: inv(U_bb); transposed for 2, 3
    const float* Dh = dinv128 + (size_t(blk) * 2 + which) * 2 * kTB2 * kTB2;
    const float* Dlo = Dh + kTB2 * kTB2;
    for (int e = tid; e < kTB2 * kTB2; e += blockDim.x) {
      const int a = e >> 7, b = e & 127;
      const int ra = trans ? b : a, cb = trans ? a : b;
      sDh[ra][cb] = __ldg(Dh + e);
      sDl[ra][cb] = __ldg(Dlo + e);
    }
  }
  // Untransposed tiles of 16-byte aligned factors move as 16-byte vectors: a thread's eight loads per tile
  // (rows 4 (w >> 2) + (j >> 3), columns 32 (w & 3) + 4 (j & 7) for chunk w, lane j: a warp reads four
  // 128-byte row segments) keep four times fewer requests in flight than 4-byte loads, which bounded the
  // tile stream.  Other tiles move as 4-byte loads.
  constexpr bool vec4 = VEC && !trans;
  auto load_tile = [&](int c0, float (&pre)[32]) {
    if (vec4) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int e = tid + 512 * i, w = e >> 5, j = e & 31;
        const int a = 4 * (w >> 2) + (j >> 3), b = 32 * (w & 3) + 4 * (j & 7);
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (r0 + a < n && c0 + b < n) {
          // the row holds ldf >= n entries rounded up to four: the vector stays inside it
          v = __ldg(reinterpret_cast<const float4*>(F + int64_t(r0 + a) * ldf + c0 + b));
          if (c0 + b + 1 >= n) v.y = 0.f;
          if (c0 + b + 2 >= n) v.z = 0.f;
          if (c0 + b + 3 >= n) v.w = 0.f;
        }
        pre[4 * i] = v.x;
        pre[4 * i + 1] = v.y;
        pre[4 * i + 2] = v.z;
        pre[4 * i + 3] = v.w;
      }
      return;
    }
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const int e = tid + 512 * i;
      const int a = e >> 7, b = e & 127;
      float v = 0.f;
      if (!trans) {
        if (r0 + a < n && c0 + b < n) v = F[int64_t(r0 + a) * ldf + c0 + b];
      } else {
        if (c0 + a < n && r0 + b < n) v = F[int64_t(c0 + a) * ldf + r0 + b];
      }
      pre[i] = v;
    }
  };
  auto store_tile = [&](const float (&pre)[32]) {
    if (vec4) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int e = tid + 512 * i, w = e >> 5, j = e & 31;
        const int a = 4 * (w >> 2) + (j >> 3), b = 32 * (w & 3) + 4 * (j & 7);
#pragma unroll
        for (int k = 0; k < 4; ++k) sT[a][b + k] = pre[4 * i + k];
      }
      return;
    }
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const int e = tid + 512 * i;
      const int a = e >> 7, b = e & 127;
      if (!trans) sT[a][b] = pre[i];
      else sT[b][a] = pre[i];
    }
  };
  auto tile_cols = [&](int q) { return (fwd ? q : nblk - 1 - q) * kTB2; };
  float pre[32];
  if (t > 0) {
    load_tile(tile_cols(0), pre);
    store_tile(pre);
    if (t > 1) load_tile(tile_cols(1), pre);
  }
  // two accumulators (even and odd columns of a pair) on packed pairs: half the dependent chain and half the
  // instructions
  float2 acc_h = make_float2(0.f, 0.f), acc_l = make_float2(0.f, 0.f);
  // with xtag, thread tid < 256 reads word tid of each solved block's x two tiles ahead of its use, so that
  // the blocks solved long before cost no L2 round trip on the way to the last one
  auto x_word = [&](int q) -> const unsigned long long* {
    const int c0 = tile_cols(q), rr = tid >> 1;
    return (tid < 2 * kTB2 && rr < min(kTB2, n - c0)) ? xtag + 2ll * (c0 + rr) + (tid & 1) : nullptr;
  };
  unsigned long long wpre[2] = {0ull, 0ull};
  if (xtag) {
#pragma unroll
    for (int d = 0; d < 2; ++d)
      if (d < t)
        if (const unsigned long long* p = x_word(d)) wpre[d] = ld_relaxed_u64(p);
  }
  for (int q = 0; q < t; ++q) {
    const int c0 = tile_cols(q);
    const int cols = min(kTB2, n - c0);
    if (xtag) {
      // tile q is in sT (stored in the previous round, before the barrier that ended it); each of 256
      // threads takes one word of block q's x, read ahead, and waits (bounded) only if it was not yet there
      unsigned long long w0 = wpre[0];
      wpre[0] = wpre[1];
      if (q + 2 < t)
        if (const unsigned long long* p = x_word(q + 2)) wpre[1] = ld_relaxed_u64(p);
      if (tid < 2 * kTB2) {
        const int rr = tid >> 1;
        float v = 0.f;
        if (rr < cols) {
          const unsigned want = unsigned(c0 / kTB2 + 1);
          const unsigned long long* p = xtag + 2ll * (c0 + rr) + (tid & 1);
          unsigned long long w = w0;
          long long it = 0;
          while (unsigned(w >> 32) != want) {
            if (++it > spin_limit()) {
              status_error(st, UPDES_ERR_TIMEOUT);
              atomicCAS(&st->timeout_tag, 0, 40 + MODE);
              break;
            }
            if (it > 32) __nanosleep(20);
            w = ld_relaxed_u64(p);
          }
          v = __uint_as_float(unsigned(w));
        }
        ((tid & 1) ? sxl : sxh)[rr] = v;
      }
      __syncthreads();
    } else {
      if (tid == 0 && s_done <= q) {
        // acquire loads of the count of finished blocks: they synchronise with each block's fence and increment,
        // and the CTA barrier below carries that order to the threads that then read x
        const int* vc = flags + nblk;
        long long it = 0;
        int d;
        while ((d = ld_acquire_gpu(vc)) <= q) {
          if (++it > spin_limit()) {
            status_error(st, UPDES_ERR_TIMEOUT);
            atomicCAS(&st->timeout_tag, 0, 30 + MODE);
            d = q + 1;
            break;
          }
          __nanosleep(20);
        }
        s_done = d;
      }
      __syncthreads();  // tile q is in sT (stored in the previous round); block q is solved
      if (tid < kTB2) {
        sxh[tid] = tid < cols ? __ldcg(xh_g + c0 + tid) : 0.f;
        sxl[tid] = tid < cols ? __ldcg(xl_g + c0 + tid) : 0.f;
      }
      __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const int c = part * 32 + 2 * ((k + 4 * part) & 15);  // column pair, rotated per part
      const float2 f = *reinterpret_cast<const float2*>(&sT[row][c]);
      df_fma_x2(f, make_float2(0.f, 0.f), *reinterpret_cast<const float2*>(&sxh[c]),
                *reinterpret_cast<const float2*>(&sxl[c]), acc_h, acc_l);
    }
    __syncthreads();  // every thread is done with sT and sx
    if (q + 1 < t) {
      store_tile(pre);  // tile q + 1, before its block's flag is awaited
      if (q + 2 < t) load_tile(tile_cols(q + 2), pre);
    }
  }
  float ah = acc_h.x, al = acc_l.x;
  df_add_to(ah, al, acc_h.y, acc_l.y);
  df_quad_sum(ah, al);
  if (part == 0) {
    // right-hand side of this block minus the off-diagonal part, double-float
    float rh = 0.f, rl = 0.f;
    if (row < rows) {
      rh = bh;
      rl = bl;
      df_add_to(rh, rl, -ah, -al);
    }
    srh[row] = rh;
    srl[row] = rl;
  }
  __syncthreads();
  // x_blk = inv(D) (b - off-diagonal part)
  float2 dh2 = make_float2(0.f, 0.f), dl2 = make_float2(0.f, 0.f);
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const int c = part * 32 + 2 * ((k + 4 * part) & 15);
    df_fma_x2(*reinterpret_cast<const float2*>(&sDh[row][c]), *reinterpret_cast<const float2*>(&sDl[row][c]),
              *reinterpret_cast<const float2*>(&srh[c]), *reinterpret_cast<const float2*>(&srl[c]), dh2, dl2);
  }
  float ph = dh2.x, pl = dl2.x;
  df_add_to(ph, pl, dh2.y, dl2.y);
  df_quad_sum(ph, pl);
  if (part == 0 && row < rows) {
    if (xtag) {
      const unsigned long long tag = (unsigned long long)(unsigned)(blk + 1) << 32;
      xtag[2ll * (r0 + row)] = tag | __float_as_uint(ph);
      xtag[2ll * (r0 + row) + 1] = tag | __float_as_uint(pl);
    } else {
      xh_g[r0 + row] = ph;
      xl_g[r0 + row] = pl;
    }
    x[r0 + row] = double(ph) + double(pl);
  }
  if (xtag) return;
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    atomicAdd(flags + nblk, 1);  // blocks finish in order: this is block number t
  }
}

template <typename TF>
int trsv_impl(int n, const TF* F, int64_t ldf, double* x, int mode, int* sync_ws, DeviceStatus* st, cudaStream_t s,
              const float* dinv, float* xh, float* xl, const float* dinv128, unsigned long long* xtag) {
  const int nblk = int(ceil_div(n, kTB));
  StatScope sc(kStatTrsv, s, double(n) * n, double(n) * n * 0.5 * sizeof(TF));
  UPDES_CUDA_TRY(cudaMemsetAsync(sync_ws, 0, sizeof(int) * (nblk + 2), s));
  int* ticket = sync_ws;
  int* flags = sync_ws + 1;
  if (sizeof(TF) != 4) dinv = nullptr;
  if constexpr (sizeof(TF) == 4) {
    if (dinv && xh && xl) {
      // UPDES_TRSV_BLOCK=64 selects the 64-row kernel
      static const bool rows128 = [] {
        const char* v = std::getenv("UPDES_TRSV_BLOCK");
        return !(v && std::atoi(v) == 64);
      }();
      if (rows128 && dinv128) {
        static std::atomic<unsigned long long> attr128[6] = {};
        int e;
        if ((e = smem_opt_in((const void*)trsv128_f32_kernel<0>, int(kTrsv128Smem), attr128[0])) ||
            (e = smem_opt_in((const void*)trsv128_f32_kernel<1>, int(kTrsv128Smem), attr128[1])) ||
            (e = smem_opt_in((const void*)trsv128_f32_kernel<2>, int(kTrsv128Smem), attr128[2])) ||
            (e = smem_opt_in((const void*)trsv128_f32_kernel<3>, int(kTrsv128Smem), attr128[3])) ||
            (e = smem_opt_in((const void*)trsv128_f32_kernel<0, true>, int(kTrsv128Smem), attr128[4])) ||
            (e = smem_opt_in((const void*)trsv128_f32_kernel<1, true>, int(kTrsv128Smem), attr128[5])))
          return e;
        const bool vec = (ldf & 3) == 0 && (reinterpret_cast<uintptr_t>(F) & 15) == 0;
        const unsigned g = unsigned(ceil_div(n, kTB2));
        // UPDES_TRSV_TAGS=0 hands solved blocks over by the finished-block count instead of tagged words
        static const bool tags_on = [] {
          const char* v = std::getenv("UPDES_TRSV_TAGS");
          return !(v && v[0] == '0');
        }();
        unsigned long long* tg = tags_on ? xtag : nullptr;
        if (tg) UPDES_CUDA_TRY(cudaMemsetAsync(tg, 0, 2 * size_t(n) * sizeof(unsigned long long), s));
        switch (mode) {
          case 0:
            if (vec) trsv128_f32_kernel<0, true><<<g, 512, kTrsv128Smem, s>>>(F, ldf, n, x, xh, xl, ticket, flags, st, dinv128, tg);
            else trsv128_f32_kernel<0><<<g, 512, kTrsv128Smem, s>>>(F, ldf, n, x, xh, xl, ticket, flags, st, dinv128, tg);
            break;
          case 1:
            if (vec) trsv128_f32_kernel<1, true><<<g, 512, kTrsv128Smem, s>>>(F, ldf, n, x, xh, xl, ticket, flags, st, dinv128, tg);
            else trsv128_f32_kernel<1><<<g, 512, kTrsv128Smem, s>>>(F, ldf, n, x, xh, xl, ticket, flags, st, dinv128, tg);
            break;
          case 2: trsv128_f32_kernel<2><<<g, 512, kTrsv128Smem, s>>>(F, ldf, n, x, xh, xl, ticket, flags, st, dinv128, tg); break;
          default: trsv128_f32_kernel<3><<<g, 512, kTrsv128Smem, s>>>(F, ldf, n, x, xh, xl, ticket, flags, st, dinv128, tg); break;
        }
        UPDES_LAUNCH_CHECK();
        return UPDES_OK;
      }
      const size_t smem = 2 * sizeof(float) * kTB * (kTB + 1);
      static std::atomic<unsigned long long> attr[4] = {};
      int e;
      if ((e = smem_opt_in((const void*)trsv_f32_kernel<0>, int(smem), attr[0])) ||
          (e = smem_opt_in((const void*)trsv_f32_kernel<1>, int(smem), attr[1])) ||
          (e = smem_opt_in((const void*)trsv_f32_kernel<2>, int(smem), attr[2])) ||
          (e = smem_opt_in((const void*)trsv_f32_kernel<3>, int(smem), attr[3])))
        return e;
      switch (mode) {
        case 0: trsv_f32_kernel<0><<<nblk, 256, smem, s>>>(F, ldf, n, x, xh, xl, ticket, flags, st, dinv); break;
        case 1: trsv_f32_kernel<1><<<nblk, 256, smem, s>>>(F, ldf, n, x, xh, xl, ticket, flags, st, dinv); break;
        case 2: trsv_f32_kernel<2><<<nblk, 256, smem, s>>>(F, ldf, n, x, xh, xl, ticket, flags, st, dinv); break;
        default: trsv_f32_kernel<3><<<nblk, 256, smem, s>>>(F, ldf, n, x, xh, xl, ticket, flags, st, dinv); break;
      }
      UPDES_LAUNCH_CHECK();
      return UPDES_OK;
    }
  }
  const size_t smem =
      sizeof(TF) * kTB * (kTB + 1) + kTB * (8 + 4 + 4 + 8) + (dinv ? 2 * sizeof(float) * kTB * (kTB + 1) : 0);
  {
    const int big = int(sizeof(TF) * kTB * (kTB + 1) + kTB * 24 + 2 * sizeof(float) * kTB * (kTB + 1));
    static std::atomic<unsigned long long> attr[4] = {};
    int e;
    if ((e = smem_opt_in((const void*)trsv_kernel<TF, 0>, big, attr[0])) ||
        (e = smem_opt_in((const void*)trsv_kernel<TF, 1>, big, attr[1])) ||
        (e = smem_opt_in((const void*)trsv_kernel<TF, 2>, big, attr[2])) ||
        (e = smem_opt_in((const void*)trsv_kernel<TF, 3>, big, attr[3])))
      return e;
  }
  switch (mode) {
    case 0: trsv_kernel<TF, 0><<<nblk, 256, smem, s>>>(F, ldf, n, x, ticket, flags, st, dinv); break;
    case 1: trsv_kernel<TF, 1><<<nblk, 256, smem, s>>>(F, ldf, n, x, ticket, flags, st, dinv); break;
    case 2: trsv_kernel<TF, 2><<<nblk, 256, smem, s>>>(F, ldf, n, x, ticket, flags, st, dinv); break;
    default: trsv_kernel<TF, 3><<<nblk, 256, smem, s>>>(F, ldf, n, x, ticket, flags, st, dinv); break;
  }
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

template int trsv_impl<double>(int, const double*, int64_t, double*, int, int*, DeviceStatus*, cudaStream_t,
                               const float*, float*, float*, const float*, unsigned long long*);
template int trsv_impl<float>(int, const float*, int64_t, double*, int, int*, DeviceStatus*, cudaStream_t,
                              const float*, float*, float*, const float*, unsigned long long*);

namespace {

// Inverses of the 64 x 64 diagonal blocks of FP32 factors (unit lower L_bb and upper U_bb), formed in FP64
// and stored as double-float planes: dinv[blk] = {inv(L) hi, inv(L) lo, inv(U) hi, inv(U) lo}, each 64 x 64
// row-major.  Rows past n (last block) are completed by the identity.  Threads 0-63 form the columns of
// inv(L), threads 64-127 those of inv(U), each by substitution against a unit vector.
__global__ void __launch_bounds__(128) diag_inverse_kernel(const float* __restrict__ F, int64_t ldf, int n,
                                                           float* __restrict__ dinv) {
  extern __shared__ double di_smem[];
  double(*B)[kTB + 1] = reinterpret_cast<double(*)[kTB + 1]>(di_smem);          // the diagonal block
  double(*X)[kTB + 1] = reinterpret_cast<double(*)[kTB + 1]>(di_smem + kTB * (kTB + 1));      // inv(L)
  double(*Y)[kTB + 1] = reinterpret_cast<double(*)[kTB + 1]>(di_smem + 2 * kTB * (kTB + 1));  // inv(U)
  const int blk = blockIdx.x, r0 = blk * kTB, rows = min(kTB, n - r0);
  for (int e = threadIdx.x; e < kTB * kTB; e += blockDim.x) {
    const int i = e >> 6, j = e & 63;
    double v = (i == j) ? 1.0 : 0.0;
    if (i < rows && j < rows) v = double(F[int64_t(r0 + i) * ldf + r0 + j]);
    B[i][j] = v;
  }
  __syncthreads();
  const int j = threadIdx.x & 63;
  if (threadIdx.x < 64) {
    // L X = I: column j, forward (unit diagonal)
    for (int i = 0; i < kTB; ++i) {
      double v = (i == j) ? 1.0 : 0.0;
      for (int k = j; k < i; ++k) v -= B[i][k] * X[k][j];
      X[i][j] = (i < j) ? 0.0 : v;
    }
  } else {
    // U Y = I: column j, backward
    for (int i = kTB - 1; i >= 0; --i) {
      double v = (i == j) ? 1.0 : 0.0;
      for (int k = i + 1; k <= j; ++k) v -= B[i][k] * Y[k][j];
      Y[i][j] = (i > j) ? 0.0 : v / B[i][i];
    }
  }
  __syncthreads();
  float* out = dinv + size_t(blk) * 4 * kTB * kTB;
  for (int e = threadIdx.x; e < kTB * kTB; e += blockDim.x) {
    const int i = e >> 6, c = e & 63;
    const double l = X[i][c], u = Y[i][c];
    const float lh = float(l), uh = float(u);
    out[e] = lh;
    out[kTB * kTB + e] = float(l - double(lh));
    out[2 * kTB * kTB + e] = uh;
    out[3 * kTB * kTB + e] = float(u - double(uh));
  }
}

}  // namespace

size_t diag_inverse_bytes(int n) { return size_t(ceil_div(n, kTB)) * 4 * kTB * kTB * sizeof(float); }

namespace {

// Inverses of the 128 x 128 diagonal blocks, composed in FP64 from the two 64 x 64 inverses of
// diag_inverse_kernel (read back from their double-float planes) and the coupling tile T of the factors:
//   unit lower:  inv [[A, 0], [T, B]] = [[inv A, 0], [-inv B T inv A, inv B]]
//   upper:       inv [[A, T], [0, B]] = [[inv A, -inv A T inv B], [0, inv B]]
// blockIdx.y = 0 for L, 1 for U; out: per (block, factor) the hi and lo planes of the 128 x 128 inverse.
__global__ void __launch_bounds__(256) diag_inverse128_kernel(const float* __restrict__ F, int64_t ldf, int n,
                                                              const float* __restrict__ dinv64,
                                                              float* __restrict__ dinv128) {
  extern __shared__ double d128_smem[];
  double(*Xa)[kTB + 1] = reinterpret_cast<double(*)[kTB + 1]>(d128_smem);
  double(*Xb)[kTB + 1] = Xa + kTB;
  double(*T)[kTB + 1] = Xb + kTB;
  double(*P)[kTB + 1] = T + kTB;
  const int blk = blockIdx.x, which = blockIdx.y, tid = threadIdx.x;
  const int r0 = blk * 2 * kTB, rows = min(2 * kTB, n - r0);
  const bool two = rows > kTB;
  const int rb = rows - kTB;  // rows of the second half
  for (int e = tid; e < kTB * kTB; e += blockDim.x) {
    const int i = e >> 6, j = e & 63;
    const float* a = dinv64 + (size_t(2 * blk) * 4 + which * 2) * kTB * kTB;
    Xa[i][j] = double(a[e]) + double(a[kTB * kTB + e]);
    double xb = 0.0, tv = 0.0;
    if (two) {
      const float* b = dinv64 + (size_t(2 * blk + 1) * 4 + which * 2) * kTB * kTB;
      xb = double(b[e]) + double(b[kTB * kTB + e]);
      if (which == 0) {
        if (i < rb) tv = double(F[int64_t(r0 + kTB + i) * ldf + r0 + j]);
      } else {
        if (j < rb) tv = double(F[int64_t(r0 + i) * ldf + r0 + kTB + j]);
      }
    }
    Xb[i][j] = xb;
    T[i][j] = tv;
  }
  __syncthreads();
  if (two) {
    // P = T inv A (lower) or T inv B (upper); then the off-diagonal block -inv B P or -inv A P into T
    for (int e = tid; e < kTB * kTB; e += blockDim.x) {
      const int i = e >> 6, j = e & 63;
      double acc = 0.0;
      for (int k = 0; k < kTB; ++k) acc = fma(T[i][k], which == 0 ? Xa[k][j] : Xb[k][j], acc);
      P[i][j] = acc;
    }
    __syncthreads();
    for (int e = tid; e < kTB * kTB; e += blockDim.x) {
      const int i = e >> 6, j = e & 63;
      double acc = 0.0;
      for (int k = 0; k < kTB; ++k) acc = fma(which == 0 ? Xb[i][k] : Xa[i][k], P[k][j], acc);
      T[i][j] = -acc;
    }
    __syncthreads();
  }
  float* hi = dinv128 + (size_t(blk) * 2 + which) * 2 * (2 * kTB) * (2 * kTB);
  float* lo = hi + (2 * kTB) * (2 * kTB);
  for (int e = tid; e < 4 * kTB * kTB; e += blockDim.x) {
    const int i = e >> 7, j = e & 127;
    const int qi = i >> 6, qj = j >> 6, ii = i & 63, jj = j & 63;
    double v = 0.0;
    if (qi == 0 && qj == 0) v = Xa[ii][jj];
    else if (qi == 1 && qj == 1) v = two ? Xb[ii][jj] : 0.0;
    else if (two && which == 0 && qi == 1 && qj == 0) v = T[ii][jj];
    else if (two && which == 1 && qi == 0 && qj == 1) v = T[ii][jj];
    const float h = float(v);
    hi[e] = h;
    lo[e] = float(v - double(h));
  }
}

}  // namespace

size_t diag_inverse128_bytes(int n) { return size_t(ceil_div(n, 2 * kTB)) * 4 * (2 * kTB) * (2 * kTB) * sizeof(float); }

int diag_inverse128(int n, const float* F, int64_t ldf, const float* dinv64, float* dinv128, cudaStream_t s) {
  const size_t smem = 4 * kTB * (kTB + 1) * sizeof(double);
  static std::atomic<unsigned long long> attr{0};
  if (int e = smem_opt_in((const void*)diag_inverse128_kernel, int(smem), attr)) return e;
  StatScope sc(kStatOther, s, 4.0 * kTB * kTB * kTB * ceil_div(n, 2 * kTB), diag_inverse128_bytes(n));
  diag_inverse128_kernel<<<dim3(unsigned(ceil_div(n, 2 * kTB)), 2), 256, smem, s>>>(F, ldf, n, dinv64, dinv128);
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

int diag_inverse(int n, const float* F, int64_t ldf, float* dinv, cudaStream_t s) {
  const size_t smem = 3 * kTB * (kTB + 1) * sizeof(double);
  static std::atomic<unsigned long long> attr{0};
  if (int e = smem_opt_in((const void*)diag_inverse_kernel, int(smem), attr)) return e;
  StatScope sc(kStatOther, s, 2.0 * kTB * kTB * kTB / 3.0 * ceil_div(n, kTB), diag_inverse_bytes(n));
  diag_inverse_kernel<<<unsigned(ceil_div(n, kTB)), 128, smem, s>>>(F, ldf, n, dinv);
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

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
#include <vector>

#include "common.cuh"
#include "lu.cuh"
#include "stats.cuh"
#include "gemm_tc.cuh"

namespace {

constexpr int kPanelThreads = 256;

struct Cand {
  double absval;
  int idx;
  int pad;
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
  extern __shared__ double smem[];
  double* tile = smem;                                   // rows_per_cta x nb
  double* prow = tile + int64_t(rows_per_cta) * nb;      // nb
  double* drow = prow + nb;                              // nb
  __shared__ double red_v[kPanelThreads / 32];
  __shared__ int red_i[kPanelThreads / 32];
  __shared__ int s_best_local, s_gw, s_p;
  __shared__ double s_pivval;

  const int G = gridDim.x, g = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int rbase = k + g * rows_per_cta;
  const int rcount = max(0, min(rows_per_cta, n - rbase));

  for (int64_t e = tid; e < int64_t(rcount) * nb; e += blockDim.x) {
    const int l = int(e / nb), c = int(e % nb);
    const int64_t idx = int64_t(rbase + l) * ldw + k + c;
    if constexpr (DF_IN) tile[e] = double(static_cast<const float*>(W)[idx]) + double(Wlo[idx]);
    else tile[e] = static_cast<const double*>(W)[idx];
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
      const double v = fabs(tile[int64_t(l) * nb + j]);
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
      Cand c;
      c.absval = bv;
      c.idx = bi;
      c.pad = 0;
      __stcg(reinterpret_cast<double2*>(cand + par * G + g), *reinterpret_cast<double2*>(&c));
      s_best_local = (bi == 0x7fffffff) ? -1 : bi - rbase;
    }
    __syncthreads();
    if (s_best_local >= 0)
      for (int c = tid; c < nb; c += blockDim.x)
        __stcg(cand_row + (int64_t(par) * G + g) * nb + c, tile[int64_t(s_best_local) * nb + c]);
    if (diag >= rbase && diag < rbase + rcount)
      for (int c = tid; c < nb; c += blockDim.x) __stcg(diag_row + par * nb + c, tile[int64_t(diag - rbase) * nb + c]);
    if (!grid_barrier(bar, G, st, 1)) return;
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
      prow[c] = __ldcg(cand_row + (int64_t(par) * G + gw) * nb + c);
      drow[c] = __ldcg(diag_row + par * nb + c);
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
      const double rinv = 1.0 / pv;
      const int l0 = max(0, diag + 1 - rbase);
      for (int l = l0 + tid; l < rcount; l += blockDim.x) tile[int64_t(l) * nb + j] *= rinv;
      __syncthreads();
      const int w = nb - j - 1;
      if (w > 0) {
        const int64_t tot = int64_t(rcount - l0) * w;
        for (int64_t e = tid; e < tot; e += blockDim.x) {
          const int l = l0 + int(e / w), c = j + 1 + int(e % w);
          tile[int64_t(l) * nb + c] -= tile[int64_t(l) * nb + j] * prow[c];
        }
      }
    }
    __syncthreads();
  }
  for (int64_t e = tid; e < int64_t(rcount) * nb; e += blockDim.x) {
    const int l = int(e / nb), c = int(e % nb);
    F[int64_t(rbase + l) * ldf + k + c] = TF(tile[e]);
  }
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

// Row interchanges as a gather/scatter through a scratch buffer, for up to 3 (plane, column range) jobs.
struct SwapJobs {
  float* plane[3];
  int64_t c0[3], c1[3];
  int njobs;
};

__global__ void swap_gather_kernel(SwapJobs jobs, int64_t ld, const int32_t* __restrict__ map, float* scratch,
                                   int64_t scratch_ld) {
  const int q = blockIdx.y, j = blockIdx.z;
  if (j >= jobs.njobs || q >= map[0]) return;
  const int64_t c = jobs.c0[j] + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (c >= jobs.c1[j]) return;
  scratch[(int64_t(j) * 128 + q) * scratch_ld + (c - jobs.c0[j])] = jobs.plane[j][int64_t(map[129 + q]) * ld + c];
}

__global__ void swap_scatter_kernel(SwapJobs jobs, int64_t ld, const int32_t* __restrict__ map, const float* scratch,
                                    int64_t scratch_ld) {
  const int q = blockIdx.y, j = blockIdx.z;
  if (j >= jobs.njobs || q >= map[0]) return;
  const int64_t c = jobs.c0[j] + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (c >= jobs.c1[j]) return;
  jobs.plane[j][int64_t(map[1 + q]) * ld + c] = scratch[(int64_t(j) * 128 + q) * scratch_ld + (c - jobs.c0[j])];
}

// U = L^-1 W on rows [k, k+nb), columns [c0, c1): L unit lower from F (FP32), W double-float, FP64 arithmetic,
// result rounded into F.
__global__ void __launch_bounds__(64) trsm_df_kernel(float* Whi, const float* Wlo, int64_t ld, int k, int nb,
                                                     int64_t c0, int64_t c1) {
  __shared__ double sL[64 * 64];
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    sL[e] = (j < i) ? double(Whi[int64_t(k + i) * ld + k + j]) : 0.0;
  }
  __syncthreads();
  const int64_t c = c0 + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (c >= c1) return;
  double x[64];
  for (int i = 0; i < nb; ++i) {
    const int64_t idx = int64_t(k + i) * ld + c;
    double v = double(Whi[idx]) + double(Wlo[idx]);
    for (int j = 0; j < i; ++j) v -= sL[i * nb + j] * x[j];
    x[i] = v;
  }
  for (int i = 0; i < nb; ++i) Whi[int64_t(k + i) * ld + c] = float(x[i]);
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

int g_num_sms = 0;

int num_sms() {
  if (!g_num_sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 1;
  }
  return g_num_sms;
}

}  // namespace

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
  int G = std::min(sms, int(ceil_div(m, 32)));
  int rows = int(ceil_div(m, G));
  size_t smem = (size_t(rows) * w + 2 * w) * sizeof(double);
  while (smem > 200 * 1024 && G < 2 * sms) {
    ++G;
    rows = int(ceil_div(m, G));
    smem = (size_t(rows) * w + 2 * w) * sizeof(double);
  }
  if (smem > 200 * 1024) return UPDES_ERR_UNSUPPORTED;
  auto kern = panel_kernel<TF, DF_IN>;
  UPDES_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
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

size_t lu_df_workspace_bytes(int n) {
  // panel scratch (rounded up to 256 B), 2 KB swap map, 3 x 128 rows of swap scratch
  return ((lu_panel_workspace_bytes(kLuNb) + 255) & ~size_t(255)) + 2048 + 3ull * 128 * (size_t(n) + 64) * sizeof(float);
}

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
  int32_t* swap_map = reinterpret_cast<int32_t*>(after);
  float* scratch = reinterpret_cast<float*>(after + 2048);
  const int64_t scratch_ld = int64_t(n) + 64;
  UPDES_CUDA_TRY(cudaMemsetAsync(bar, 0, 256, s));
  constexpr int kOuter = 4 * kLuNb;  // 256: width of the exact trailing updates
  auto swaps = [&](int k, int w) -> int {
    SwapJobs j{};
    int nj = 0;
    int64_t maxc = 0;
    if (k + w < n) {
      j.plane[nj] = Whi; j.c0[nj] = k + w; j.c1[nj] = n; ++nj;
      j.plane[nj] = Wlo; j.c0[nj] = k + w; j.c1[nj] = n; ++nj;
      maxc = n - k - w;
    }
    if (k > 0) {
      j.plane[nj] = Whi; j.c0[nj] = 0; j.c1[nj] = k; ++nj;
      maxc = std::max<int64_t>(maxc, k);
    }
    j.njobs = nj;
    if (!nj) return UPDES_OK;
    dim3 grid(unsigned(ceil_div(maxc, 256)), 128, nj);
    StatScope sc(kStatOther, s, 0.0, 2.0 * 2 * w * maxc * 4.0 * nj);
    swap_gather_kernel<<<grid, 256, 0, s>>>(j, ld, swap_map, scratch, scratch_ld);
    UPDES_LAUNCH_CHECK();
    swap_scatter_kernel<<<grid, 256, 0, s>>>(j, ld, swap_map, scratch, scratch_ld);
    UPDES_LAUNCH_CHECK();
    return UPDES_OK;
  };
  auto trsm = [&](int k, int w, int64_t c0, int64_t c1) -> int {
    if (c1 <= c0) return UPDES_OK;
    StatScope sc(kStatTrsm, s, double(w) * w * (c1 - c0), double(w) * (c1 - c0) * 12.0);
    trsm_df_kernel<<<unsigned(ceil_div(c1 - c0, 64)), 64, 0, s>>>(Whi, Wlo, ld, k, w, c0, c1);
    UPDES_LAUNCH_CHECK();
    return UPDES_OK;
  };
  auto upd = [&](int r0, int r1, int c0, int c1, int kk0, int kk1) -> int {
    // W[r0:r1, c0:c1] -= F[r0:r1, kk0:kk1] * F[kk0:kk1, c0:c1]
    return ozaki_update(Whi + int64_t(r0) * ld + c0, Wlo + int64_t(r0) * ld + c0, ld, Whi + int64_t(r0) * ld + kk0,
                        ld, Whi + int64_t(kk0) * ld + c0, ld, r1 - r0, c1 - c0, kk1 - kk0, st, s);
  };
  int e;
  for (int K0 = 0; K0 < n; K0 += kOuter) {
    const int KE = std::min(K0 + kOuter, n);
    for (int k = K0; k < KE; k += nb) {
      const int w = std::min(nb, KE - k);
      if ((e = launch_panel<float, true>(Whi, Wlo, ld, Whi, ld, n, k, w, piv, bar, cand, cand_row, diag_row,
                                         swap_map, st, s)))
        return e;
      if ((e = swaps(k, w))) return e;
      if (k + w < KE) {
        if ((e = trsm(k, w, k + w, KE))) return e;
        if ((e = upd(k + w, n, k + w, KE, k, k + w))) return e;
      }
    }
    if (KE < n) {
      for (int b = K0; b < KE; b += nb) {
        const int w = std::min(nb, KE - b);
        if ((e = trsm(b, w, KE, n))) return e;
        if (b + w < KE && (e = upd(b + w, KE, KE, n, b, b + w))) return e;
      }
      if ((e = upd(KE, n, KE, n, K0, KE))) return e;
    }
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
  UPDES_CUDA_TRY(cudaMemsetAsync(bar, 0, 256, s));
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
  const float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  sh = s;
  sl = __fadd_rn(sl, __fadd_rn(t, __fmaf_rn(f, xl, e)));
}

template <typename TF, int MODE>
__global__ void __launch_bounds__(256) trsv_kernel(const TF* __restrict__ F, int64_t ldf, int n, double* x,
                                                   int* ticket, int* flags, DeviceStatus* st) {
  extern __shared__ __align__(16) unsigned char trsv_smem[];
  TF(*sT)[kTB + 1] = reinterpret_cast<TF(*)[kTB + 1]>(trsv_smem);
  double* sxd = reinterpret_cast<double*>(trsv_smem + sizeof(TF) * kTB * (kTB + 1));  // 64
  float* sxh = reinterpret_cast<float*>(sxd + kTB);                                    // 64
  float* sxl = sxh + kTB;                                                              // 64
  double* sacc = reinterpret_cast<double*>(sxl + kTB);                                 // 64
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
  for (int q = 0; q < t; ++q) {
    const int jb = fwd ? q : nblk - 1 - q;
    const int c0 = jb * kTB;
    const int cols = min(kTB, n - c0);
    if (tid == 0) {
      volatile int* vf = flags + jb;
      long long it = 0;
      while (*vf == 0) {
        if (++it > kSpinLimit) {
          status_error(st, UPDES_ERR_TIMEOUT);
          atomicCAS(&st->timeout_tag, 0, 10 + MODE);
          break;
        }
        __nanosleep(32);
      }
      __threadfence();
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
  if (tid < 32) {
    double xi_lane[2] = {0.0, 0.0};
    for (int s2 = 0; s2 < rows; ++s2) {
      const int i = fwd ? s2 : rows - 1 - s2;
      double part_sum = 0.0;
      for (int j = tid; j < rows; j += 32) {
        const bool dep = fwd ? (j < i) : (j > i);
        if (dep) part_sum += double(sT[i][j]) * xi_lane[j >> 5];
      }
      for (int o = 16; o > 0; o >>= 1) part_sum += __shfl_xor_sync(0xffffffffu, part_sum, o);
      double v = x[r0 + i] - sacc[i] - part_sum;
      constexpr bool unit = (MODE == 0 || MODE == 3);
      if (!unit) v = v / double(sT[i][i]);
      if ((i & 31) == tid) xi_lane[i >> 5] = v;
    }
    for (int i = tid; i < rows; i += 32) x[r0 + i] = xi_lane[i >> 5];
  }
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    atomicExch(flags + blk, 1);
  }
}

}  // namespace

template <typename TF>
int trsv_impl(int n, const TF* F, int64_t ldf, double* x, int mode, int* sync_ws, DeviceStatus* st, cudaStream_t s) {
  const int nblk = int(ceil_div(n, kTB));
  StatScope sc(kStatTrsv, s, double(n) * n, double(n) * n * 0.5 * sizeof(TF));
  UPDES_CUDA_TRY(cudaMemsetAsync(sync_ws, 0, sizeof(int) * (nblk + 1), s));
  int* ticket = sync_ws;
  int* flags = sync_ws + 1;
  const size_t smem = sizeof(TF) * kTB * (kTB + 1) + kTB * (8 + 4 + 4 + 8);
  switch (mode) {
    case 0: trsv_kernel<TF, 0><<<nblk, 256, smem, s>>>(F, ldf, n, x, ticket, flags, st); break;
    case 1: trsv_kernel<TF, 1><<<nblk, 256, smem, s>>>(F, ldf, n, x, ticket, flags, st); break;
    case 2: trsv_kernel<TF, 2><<<nblk, 256, smem, s>>>(F, ldf, n, x, ticket, flags, st); break;
    default: trsv_kernel<TF, 3><<<nblk, 256, smem, s>>>(F, ldf, n, x, ticket, flags, st); break;
  }
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

template int trsv_impl<double>(int, const double*, int64_t, double*, int, int*, DeviceStatus*, cudaStream_t);
template int trsv_impl<float>(int, const float*, int64_t, double*, int, int*, DeviceStatus*, cudaStream_t);

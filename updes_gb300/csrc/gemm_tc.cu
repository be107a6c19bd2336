// Tensor-core trailing update of the mixed-precision LU (sm_103a, tcgen05).
//
//   C  <-  C - A * B        C: FP32 hi/lo pairs ("double-float", ~48 bits)
//                           A: m x K FP32 (L factor block), B: K x nc FP32 (U factor block)
//
// Every FP32 operand is written as D bf16 integer digits (D = UPDES_OZAKI_DIGITS,
// 3 by default) under a power-of-two scale shared by a row of A (a column of
// B) over each 64-wide k-block:
//   a = 2^(eA-8) * (d1 + 2^-9 d2 + 2^-18 d3 + ...),   |d_i| <= 256 (exact in bf16),
// exact for entries within 2^(9D-25) of the row maximum and otherwise cut at
// 2^-(9D-1) of it.  Digit products are <= 2^16, a 64-term sum is <= 2^22 and a
// group of at most D products of equal weight 2^-9g stays <= 2^24, so each of
// the 2D-1 FP32 TMEM accumulators holds an exact integer: the tensor cores add
// no rounding (FP32-accumulated updates lose the Schur complements of these
// ill-conditioned matrices).  The epilogue folds the groups into a
// double-float value and subtracts it from C with error-free transformations
// (FP32 ALU only; FP64 throughput is low on GB300).
// Each CTA owns a 128 x 64 tile of C; one thread issues tcgen05.mma
// (kind::f16, bf16 operands from 128B-swizzled K-major shared memory, FP32
// accumulators in tensor memory); every wait is bounded.
#include <cuda_bf16.h>

#include <atomic>

#include "gemm_tc.cuh"
#include "stats.cuh"

#ifndef UPDES_OZAKI_DIGITS
#define UPDES_OZAKI_DIGITS 3
#endif

namespace {

constexpr int TM = 128, TN = 64, TK = 64;
constexpr int kThreads = 256;
constexpr uint32_t kTmemCols = 512;  // kGroups x 64 columns, rounded to a power of two
constexpr int kDigits = UPDES_OZAKI_DIGITS, kGroups = 2 * kDigits - 1;
static_assert(kGroups * TN <= int(kTmemCols), "accumulators must fit in tensor memory");
constexpr int kATile = TM * TK * 2;  // 16 KB per digit plane
constexpr int kBTile = TN * TK * 2;  //  8 KB per digit plane
constexpr int kSmemOperands = kDigits * (kATile + kBTile);
// two operand buffers + scales + partial maxima; more than half of an SM's shared memory, so one CTA per
// SM (it owns 512 TMEM columns)
constexpr int kSmemBytes = 2 * kSmemOperands + 1024 /*align*/ + 2 * (TM + TN) * 4 + 16 * TN * 4 + 64;
static_assert(kSmemBytes > 116 * 1024 && kSmemBytes <= 227 * 1024, "shared memory layout");

// instruction descriptor: D = F32, A = B = BF16, both K-major, N = 64, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(TN >> 3) << 17) | (uint32_t(TM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor: K-major, 128B swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  uint64_t d = uint64_t((saddr & 0x3FFFFu) >> 4);
  d |= uint64_t(1) << 16;             // leading byte offset (unused with 128B swizzle, K-major)
  d |= uint64_t(1024 >> 4) << 32;     // stride byte offset
  d |= uint64_t(1) << 46;             // descriptor version
  d |= uint64_t(2) << 61;             // SWIZZLE_128B
  return d;
}

// byte offset of element (row, k) of a K-major, 128B-swizzled bf16 tile (64 k per row)
__device__ __forceinline__ uint32_t sw128(int row, int k) {
  return uint32_t((row >> 3) * 1024 + (row & 7) * 128 + ((((k >> 3) ^ row) & 7) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ float pow2f(int e) {  // 2^e for e in [-126, 127]
  return __int_as_float((e + 127) << 23);
}

// exponent e with max < 2^e (frexp convention), clamped so that scalings stay in range
__device__ __forceinline__ int exp_of(float mx) {
  const int E = (__float_as_int(mx) >> 23) & 0xFF;
  if (E == 0) return -100;  // zero or subnormal: digits round to zero
  return max(E - 126, -100);
}

// a * scale = d[0] + 2^-9 d[1] + 2^-18 d[2] + ... (+ a remainder below the last digit), |d[i]| <= 256
__device__ __forceinline__ void digits(float a, float scale, float (&d)[kDigits]) {
  float r = __fmul_rn(a, scale);  // exact: power-of-two scaling, |r| <= 256
#pragma unroll
  for (int i = 0; i < kDigits; ++i) {
    d[i] = rintf(r);
    r = __fmul_rn(__fsub_rn(r, d[i]), 512.f);  // exact: |r - d| <= 1/2
  }
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase) {
  for (long long it = 0; it < kTcSpinLimit; ++it) {
    if (mbar_try_wait(bar, phase)) return true;
    __nanosleep(32);
  }
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

template <bool ACC>
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "n"(ACC ? 1 : 0)
      : "memory");
}

// Digit product (A, B) over the four k-steps of a block into group A + B.  The descriptors are built once
// per buffer and every operand offset is a compile-time constant (descriptor units of 16 bytes), so the
// issuing thread keeps pace with the tensor pipe.
template <int A, int B>
__device__ __forceinline__ void mma_product(uint32_t tmem, uint64_t a0, uint64_t b0) {
  constexpr int g = A + B;
  constexpr bool first = (A == (g >= kDigits ? g - kDigits + 1 : 0));  // the group's first product
  const uint32_t d = tmem + uint32_t(g * TN);
#pragma unroll
  for (int kk = 0; kk < TK / 16; ++kk) {
    const uint64_t ad = a0 + uint64_t(A * (kATile >> 4) + kk * 2), bd = b0 + uint64_t(B * (kBTile >> 4) + kk * 2);
    if (first && kk == 0) mma_bf16<false>(d, ad, bd);
    else mma_bf16<true>(d, ad, bd);
  }
}

// all D x D products, a-major (so each group's first product is issued first)
template <int A, int B>
__device__ __forceinline__ void mma_all(uint32_t tmem, uint64_t a0, uint64_t b0) {
  if constexpr (A < kDigits) {
    mma_product<A, B>(tmem, a0, b0);
    if constexpr (B + 1 < kDigits) mma_all<A, B + 1>(tmem, a0, b0);
    else mma_all<A + 1, 0>(tmem, a0, b0);
  }
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Global -> register staging of one 64-wide k block: A rows (4 x 8 values per thread) and B (16 values).
struct Stage {
  float4 a[4][2];
  float4 b[4];
};

__device__ __forceinline__ void stage_load(Stage& st, const float* __restrict__ A, int64_t lda,
                                           const float* __restrict__ B, int64_t ldb, int r0, int c0, int m, int nc,
                                           int K, int kb, int tid, bool vec_ok) {
#pragma unroll
  for (int it = 0; it < 4; ++it) {
    const int chunk = tid + it * kThreads;  // 1024 chunks of 8 k values: row = chunk / 8
    const int row = chunk >> 3, kc = chunk & 7;
    const int gr = r0 + row, k0 = kb + kc * 8;
    if (vec_ok && gr < m && k0 + 7 < K) {
      const float4* p = reinterpret_cast<const float4*>(A + int64_t(gr) * lda + k0);
      st.a[it][0] = __ldg(p);
      st.a[it][1] = __ldg(p + 1);
    } else {
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = (gr < m && k0 + u < K) ? A[int64_t(gr) * lda + k0 + u] : 0.f;
      st.a[it][0] = make_float4(v[0], v[1], v[2], v[3]);
      st.a[it][1] = make_float4(v[4], v[5], v[6], v[7]);
    }
  }
  // B: thread owns 4 consecutive columns j4..j4+3 and 4 consecutive k rows kq*4..kq*4+3
  const int j4 = (tid & 15) * 4, kq = tid >> 4;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int k = kb + kq * 4 + u, gc = c0 + j4;
    if (vec_ok && k < K && gc + 3 < nc) {
      st.b[u] = __ldg(reinterpret_cast<const float4*>(B + int64_t(k) * ldb + gc));
    } else {
      float v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = (k < K && gc + q < nc) ? B[int64_t(k) * ldb + gc + q] : 0.f;
      st.b[u] = make_float4(v[0], v[1], v[2], v[3]);
    }
  }
}

__device__ __forceinline__ float f4(const float4& v, int i) { return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w; }

// Digits of a staged block into one shared-memory buffer (A: row scales, B: column scales).
__device__ __forceinline__ void stage_digits(const Stage& st, uint8_t* sA, uint8_t* sB, float* sSA, float* sSB,
                                             float* sBmax, int tid) {
#pragma unroll
  for (int it = 0; it < 4; ++it) {
    const int chunk = tid + it * kThreads;
    const int row = chunk >> 3, kc = chunk & 7;
    float v[8];
#pragma unroll
    for (int u = 0; u < 4; ++u) { v[u] = f4(st.a[it][0], u); v[4 + u] = f4(st.a[it][1], u); }
    float mx = 0.f;
#pragma unroll
    for (int u = 0; u < 8; ++u) mx = fmaxf(mx, fabsf(v[u]));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 2));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 4));
    const int e = exp_of(mx);
    if (kc == 0) sSA[row] = pow2f(e - 8);
    const float scale = pow2f(8 - e);
    __align__(16) __nv_bfloat16 d[kDigits][8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      float dd[kDigits];
      digits(v[u], scale, dd);
#pragma unroll
      for (int p = 0; p < kDigits; ++p) d[p][u] = __float2bfloat16_rn(dd[p]);
    }
    const uint32_t off = sw128(row, kc * 8);
#pragma unroll
    for (int p = 0; p < kDigits; ++p) *reinterpret_cast<uint4*>(sA + p * kATile + off) = *reinterpret_cast<uint4*>(d[p]);
  }
  const int j4 = (tid & 15) * 4, kq = tid >> 4;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    float mx = 0.f;
#pragma unroll
    for (int u = 0; u < 4; ++u) mx = fmaxf(mx, fabsf(f4(st.b[u], q)));
    sBmax[kq * TN + j4 + q] = mx;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int j = j4 + q;
    float mx = 0.f;
    for (int w = 0; w < 16; ++w) mx = fmaxf(mx, sBmax[w * TN + j]);
    const int e = exp_of(mx);
    if (kq == 0) sSB[j] = pow2f(e - 8);
    const float scale = pow2f(8 - e);
    __align__(8) __nv_bfloat16 d[kDigits][4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      float dd[kDigits];
      digits(f4(st.b[u], q), scale, dd);
#pragma unroll
      for (int p = 0; p < kDigits; ++p) d[p][u] = __float2bfloat16_rn(dd[p]);
    }
    const uint32_t off = sw128(j, kq * 4);
#pragma unroll
    for (int p = 0; p < kDigits; ++p) *reinterpret_cast<uint2*>(sB + p * kBTile + off) = *reinterpret_cast<uint2*>(d[p]);
  }
}

__global__ void __launch_bounds__(kThreads, 1)
    ozaki_update_kernel(float* __restrict__ Chi, float* __restrict__ Clo, int64_t ldc, const float* __restrict__ A,
                        int64_t lda, const float* __restrict__ B, int64_t ldb, int m, int nc, int K,
                        DeviceStatus* st) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  // two buffers of digit planes: [buf][A planes | B planes]
  uint8_t* sOps[2] = {smem, smem + kSmemOperands};
  float* sScale = reinterpret_cast<float*>(smem + 2 * kSmemOperands);  // [buf][128 row + 64 col]
  float* sBmax = sScale + 2 * (TM + TN);                                 // 16 x 64 partial column maxima
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r0 = blockIdx.y * TM, c0 = blockIdx.x * TN;
  const bool vec_ok = ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15) == 0 &&
                      (lda & 3) == 0 && (ldb & 3) == 0;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(&mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_fail = 0;
  }
  Stage stg;
  stage_load(stg, A, lda, B, ldb, r0, c0, m, nc, K, 0, tid, vec_ok);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  stage_digits(stg, sOps[0], sOps[0] + kDigits * kATile, sScale, sScale + TM, sBmax, tid);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();

  // this thread's row and 32 columns of the result, accumulated in double-float over all k blocks
  const int row = (warp & 3) * 32 + lane;
  const int colbase = (warp >> 2) * 32;
  const uint32_t lane_base = uint32_t((warp & 3) * 32) << 16;
  float acc_h[32], acc_l[32];
#pragma unroll
  for (int u = 0; u < 32; ++u) { acc_h[u] = 0.f; acc_l[u] = 0.f; }

  uint32_t phase = 0, failed_phase = 0;
  const int nsub = int(ceil_div(K, TK));
  for (int sb = 0; sb < nsub; ++sb) {
    const int buf = sb & 1;
    uint8_t* sA = sOps[buf];
    uint8_t* sB = sOps[buf] + kDigits * kATile;
    // ---- issue kDigits^2 digit products x 4 k-steps into kGroups accumulators ----
    if (tid == 0) {
      tc_fence_after();
      // products in order of a; the first product of group g = a + b is (max(0, g - D + 1), ...)
      mma_all<0, 0>(tmem, make_desc(smem_u32(sA)), make_desc(smem_u32(sB)));
      mma_commit(&mbar);
    }
    __syncwarp();
    // ---- meanwhile: stage and digitise the next k block into the other buffer ----
    if (sb + 1 < nsub) {
      stage_load(stg, A, lda, B, ldb, r0, c0, m, nc, K, (sb + 1) * TK, tid, vec_ok);
      uint8_t* nA = sOps[buf ^ 1];
      float* nS = sScale + (buf ^ 1) * (TM + TN);
      stage_digits(stg, nA, nA + kDigits * kATile, nS, nS + TM, sBmax, tid);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    // ---- wait for the accumulators ----
    if (!mbar_wait_bounded(&mbar, phase)) {
      s_fail = 1;
      failed_phase = phase;
    }
    phase ^= 1u;
    tc_fence_after();
    __syncthreads();
    if (s_fail) break;
    // ---- fold the exact group sums into this thread's double-float accumulators ----
    {
      const float* sSA = sScale + buf * (TM + TN);
      const float* sSB = sSA + TM;
      const float sa = sSA[row];
#pragma unroll
      for (int ch = 0; ch < 2; ++ch) {
        const int col = colbase + ch * 16;
        float gacc[kGroups][16];
#pragma unroll
        for (int g = 0; g < kGroups; ++g) tmem_ld16(tmem + lane_base + uint32_t(g * TN + col), gacc[g]);
        tmem_wait_ld();
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          float h, l, e;
          two_sum(gacc[0][u], __fmul_rn(gacc[1][u], 1.953125e-3f), h, l);
          two_sum(h, __fmul_rn(gacc[2][u], 3.814697265625e-06f), h, e);
          l = __fadd_rn(l, e);
          float w = 3.814697265625e-06f;
#pragma unroll
          for (int g = 3; g < kGroups; ++g) {
            w = __fmul_rn(w, 1.953125e-3f);
            l = __fadd_rn(l, __fmul_rn(gacc[g][u], w));
          }
          const float sc = __fmul_rn(sa, sSB[col + u]);
          h = __fmul_rn(h, sc);
          l = __fmul_rn(l, sc);
          float s1, t1;
          two_sum(acc_h[ch * 16 + u], h, s1, t1);
          t1 = __fadd_rn(t1, __fadd_rn(acc_l[ch * 16 + u], l));
          fast_two_sum(s1, t1, acc_h[ch * 16 + u], acc_l[ch * 16 + u]);
        }
      }
    }
    tc_fence_before();
    __syncthreads();
  }
  // ---- C -= accumulated product, once ----
  if (!s_fail) {
    const int gr = r0 + row;
    if (gr < m) {
      float* ph = Chi + int64_t(gr) * ldc + c0 + colbase;
      float* pl = Clo + int64_t(gr) * ldc + c0 + colbase;
      const bool vec_c = (((reinterpret_cast<uintptr_t>(ph) | reinterpret_cast<uintptr_t>(pl)) & 15) == 0) &&
                         c0 + colbase + 31 < nc;
      if (vec_c) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          float4 hv = reinterpret_cast<float4*>(ph)[q], lv = reinterpret_cast<float4*>(pl)[q];
          float hh[4] = {hv.x, hv.y, hv.z, hv.w}, ll[4] = {lv.x, lv.y, lv.z, lv.w};
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            float sx, tx;
            two_sum(hh[u], -acc_h[q * 4 + u], sx, tx);
            tx = __fadd_rn(tx, __fsub_rn(ll[u], acc_l[q * 4 + u]));
            fast_two_sum(sx, tx, hh[u], ll[u]);
          }
          reinterpret_cast<float4*>(ph)[q] = make_float4(hh[0], hh[1], hh[2], hh[3]);
          reinterpret_cast<float4*>(pl)[q] = make_float4(ll[0], ll[1], ll[2], ll[3]);
        }
      } else {
#pragma unroll
        for (int u = 0; u < 32; ++u) {
          if (c0 + colbase + u < nc) {
            float sx, tx;
            two_sum(ph[u], -acc_h[u], sx, tx);
            tx = __fadd_rn(tx, __fsub_rn(pl[u], acc_l[u]));
            fast_two_sum(sx, tx, ph[u], pl[u]);
          }
        }
      }
    }
  }
  if (s_fail && tid == 0) {
    status_error(st, UPDES_ERR_TIMEOUT);
    atomicCAS(&st->timeout_tag, 0, 40);
    // give in-flight MMAs a bounded chance to finish before the tensor memory is released
    mbar_wait_bounded(&mbar, failed_phase);
  }
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

}  // namespace


int ozaki_update(float* Chi, float* Clo, int64_t ldc, const float* A, int64_t lda, const float* B, int64_t ldb,
                 int m, int nc, int K, DeviceStatus* st, cudaStream_t s) {
  if (m <= 0 || nc <= 0 || K <= 0) return UPDES_OK;
  static std::atomic<unsigned long long> attr{0};
  if (int e = smem_opt_in((const void*)ozaki_update_kernel, kSmemBytes, attr)) return e;
  dim3 grid(unsigned(ceil_div(nc, TN)), unsigned(ceil_div(m, TM)));
  StatScope sc(kStatGemm, s, 2.0 * m * double(nc) * K, double(m) * nc * 16.0 + (double(m) + nc) * K * 4.0);
  ozaki_update_kernel<<<grid, kThreads, kSmemBytes, s>>>(Chi, Clo, ldc, A, lda, B, ldb, m, nc, K, st);
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

// Tensor-core trailing update of the mixed-precision LU, persistent and warp-specialised (sm_103a).
//
//   C  <-  C - A * B        C: FP32 hi/lo pairs ("double-float", ~48 bits)
//                           A: m x K FP32 (L factor block), B: K x nc FP32 (U factor block)
//
// Numerics.  Every FP32 operand is written as 3 bf16 integer digits under a power-of-two scale shared by a
// row of A (a column of B) over each 64-wide k block:
//   a = 2^(e-8) * (d0 + 2^-9 d1 + 2^-18 d2),   |d_i| <= 256 (exact in bf16),
// exact for entries within a factor 4 of the block's row maximum and cut at 2^-26 of it otherwise.  Digit
// products are <= 2^16 and a 64-term sum is <= 2^22; the products of equal weight 2^-9g (g = a + b) are
// summed in one FP32 tensor-memory accumulator, at most 3 of them, so every accumulator holds an exact
// integer below 2^24 and the tensor cores add no rounding.  The product d2 * e2 (weight 2^-36) lies ten
// bits below the digit cut and is left out: 8 products, 4 accumulators.  The epilogue folds the four
// exact group sums of each k block into per-thread double-float accumulators with error-free
// transformations (FP32 ALU: GB300's FP64 rate is low), and subtracts the result from C once per tile.
//
// Structure.  A pre-pass writes the digits once per update (A as [3][m][Kp] bf16, B transposed as
// [3][nc][Kp] bf16, Kp = K rounded up to 64, zero padded) and the scales.  The main kernel is persistent
// (one CTA per SM, tiles of 128 x 64 taken round robin) with three roles:
//   warp 0      TMA producer: the 3 + 3 digit tiles of a k block into a 2-stage ring (128B swizzle, 72 KB
//               a stage, the most that fits beside the C tile);
//   warp 1      MMA issuer: 8 products x 4 k-steps of tcgen05.mma (kind::f16, M=128, N=64) into one of
//               two accumulator sets (4 groups x 64 columns each, 512 TMEM columns in all);
//   warps 2-17  epilogue: tcgen05.ld of the 4 groups, fold, and at the end of a tile C -= acc on the C tile
//               in shared memory; one of its threads stores the tile by TMA and, once the store has read
//               the buffer, loads the next tile's C into it.
// The fold of one k block runs while the tensor cores work on the next, the C read-modify-write of a tile
// overlaps the MMAs of the following tile, and the operand stream never waits for the C buffer.  Every mbarrier wait is bounded; a timeout sets the status
// word and an abort flag that every role checks, and tensor memory is freed on every path.
#include <atomic>

#include <cuda.h>
#include <cuda_bf16.h>

#include "gemm_tc.cuh"
#include "stats.cuh"

namespace {

constexpr int TM = 128, TN = 64, TK = 64;
constexpr int kDigits = 3, kGroups = 4;  // 8 digit products
constexpr int kStages = 2;  // equal to the number of accumulator sets (one barrier serves both)
// epilogue: kEpiWarps warps, four per lane quarter of the tile (the warps a TMEM lane quarter allows), each
// with kEpiCols columns
constexpr int kEpiWarps = 16, kEpiCols = TN / (kEpiWarps / 4);
constexpr int kWarps = 2 + kEpiWarps, kThreads = kWarps * 32;
constexpr uint32_t kTmemCols = 512;  // 2 sets x 4 groups x 64 columns
constexpr int kATile = TM * TK * 2;  // 16 KB per digit plane
constexpr int kBTile = TN * TK * 2;  //  8 KB per digit plane
constexpr int kStageBytes = kDigits * (kATile + kBTile);  // 72 KB
constexpr int kCHalf = TM * 32 * 4;                         // 16 KB: 128 rows x 32 FP32 (one 128-B swizzled box)
constexpr int kCBytes = 4 * kCHalf;                         // C tile: {hi, lo} x {columns 0-31, 32-63}
constexpr int kSmemBytes = kStages * kStageBytes + kCBytes + 1024;
static_assert(kSmemBytes <= 227 * 1024, "shared memory");

// instruction descriptor: D = F32, A = B = BF16, both K-major, N = 64, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(TN >> 3) << 17) | (uint32_t(TM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor: K-major, 128B swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  uint64_t d = uint64_t((saddr & 0x3FFFFu) >> 4);
  d |= uint64_t(1) << 16;
  d |= uint64_t(1024 >> 4) << 32;
  d |= uint64_t(1) << 46;
  d |= uint64_t(2) << 61;
  return d;
}

__device__ __forceinline__ float pow2f(int e) { return __int_as_float((e + 127) << 23); }

__device__ __forceinline__ int exp_of(float mx) {
  const int E = (__float_as_int(mx) >> 23) & 0xFF;
  if (E == 0) return -100;
  return max(E - 126, -100);
}

// Error-free sum (Knuth's TwoSum) and Dekker's Fast2Sum on column pairs, with the packed FP32x2 instructions
// of sm_100+ (one issue slot per pair).  y - x is formed as fma(x, -1, y): the product is exact, so it rounds once like a subtraction.
__device__ __forceinline__ float2 sub2(float2 y, float2 x) { return __ffma2_rn(x, make_float2(-1.f, -1.f), y); }

__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = __fadd2_rn(a, b);
  const float2 bb = sub2(s, a);
  e = __fadd2_rn(sub2(a, sub2(s, bb)), sub2(b, bb));
}

__device__ __forceinline__ void fast_two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = __fadd2_rn(a, b);
  e = sub2(b, sub2(s, a));
}

// ---- mbarrier / tcgen05 / TMA primitives -------------------------------------------------------------
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

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Bounded wait; gives up when the abort flag is raised by another role.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase, volatile int* abort_flag) {
  for (long long it = 0; it < kTcSpinLimit; ++it) {
    if (mbar_try_wait(bar, phase)) return true;
    if ((it & 63) == 63 && *abort_flag) return false;
    if (it > 256) __nanosleep(32);
  }
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D (+)= A * B with both operands from shared-memory descriptors; ACC = false overwrites D.
template <bool ACC>
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "n"(ACC ? 1 : 0)
      : "memory");
}

// The 32 MMAs of one k block: digit products (a, b) with a + b <= 3 (d2 * e2 is below the digit cut), four
// k-steps of 16 each, into accumulator group a + b.  Descriptors are built once; every operand offset is a
// compile-time constant added to them (descriptor address units are 16 bytes: a digit plane of A is 1024
// units, of B 512, a k-step 2), so the issuing thread keeps pace with the tensor pipe.
template <int A, int B>
__device__ __forceinline__ void mma_product(uint32_t tset, uint64_t a0, uint64_t b0) {
  constexpr int g = A + B;
  constexpr bool first = (A == (g > 2 ? g - 2 : 0));  // the group's first product overwrites it
  const uint32_t d = tset + uint32_t(g * TN);
#pragma unroll
  for (int kk = 0; kk < TK / 16; ++kk) {
    const uint64_t ad = a0 + uint64_t(A * (kATile >> 4) + kk * 2), bd = b0 + uint64_t(B * (kBTile >> 4) + kk * 2);
    if (first && kk == 0) mma_bf16<false>(d, ad, bd);
    else mma_bf16<true>(d, ad, bd);
  }
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float* v) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr)
               : "memory");
#pragma unroll
  for (int i = 0; i < 4; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// L2 eviction policies for the copies below: the digit tiles of L and U are reused by every tile of their
// row band / column across the whole launch, while each C tile is read and written once; marking C
// evict-first and the digits evict-last keeps the streamed C planes (gigabytes per launch at n = 22,506) from
// pushing the digit tiles out of L2 between their uses.
__device__ __forceinline__ uint64_t l2_policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}

// 3-D tiled TMA load (x = k offset, y = row, z = digit plane) completing on an mbarrier, with an L2 policy.
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar,
                                            uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1, {%2, %3, %4}], [%5], %6;" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}

// 2-D tiled TMA load (x = column, y = row) completing on an mbarrier, and the matching bulk-group store, with
// an L2 policy.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint64_t* bar,
                                            uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}

__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, uint32_t src, uint64_t policy) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group.L2::cache_hint [%0, {%1, %2}], [%3], %4;" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(src), "l"(policy)
               : "memory");
}

// ---- digit pre-pass ------------------------------------------------------------------------------------
// A (m x K, lda) -> Ad[p][r][k] (bf16, p < 3, k < Kp) and As[r][kb] = 2^(e-8), one warp per (row, k block);
// bx is the block's index among the row part's blocks.
__device__ __forceinline__ void digits_rows(int bx, const float* __restrict__ A, int64_t lda, int m, int K, int Kp,
                                            __nv_bfloat16* __restrict__ Ad, float* __restrict__ As) {
  const int64_t w = (int64_t(bx) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nkb = Kp / TK;
  if (w >= int64_t(m) * nkb) return;
  const int r = int(w / nkb), kb = int(w % nkb);
  float v[2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int k = kb * TK + lane + 32 * u;
    v[u] = k < K ? A[int64_t(r) * lda + k] : 0.f;
  }
  float mx = fmaxf(fabsf(v[0]), fabsf(v[1]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  const int e = exp_of(mx);
  if (lane == 0) As[int64_t(r) * nkb + kb] = pow2f(e - 8);
  const float scale = pow2f(8 - e);
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    float x = __fmul_rn(v[u], scale);  // exact, |x| <= 256
    const int64_t base = int64_t(r) * Kp + kb * TK + lane + 32 * u;
#pragma unroll
    for (int p = 0; p < kDigits; ++p) {
      const float d = rintf(x);
      Ad[int64_t(p) * m * Kp + base] = __float2bfloat16_rn(d);
      x = __fmul_rn(__fsub_rn(x, d), 512.f);  // exact
    }
  }
}

// B (K x nc, ldb) -> Bd[p][c][k] (bf16, transposed) and Bs[kb][c] (row stride ncp = nc rounded up to TN, the
// padding columns 0); a CTA per (64 k, 64 columns) tile: column tile bx, k block kb.
__device__ __forceinline__ void digits_cols(int bx, int kb, const float* __restrict__ B, int64_t ldb, int nc, int K,
                                            int Kp, __nv_bfloat16* __restrict__ Bd, float* __restrict__ Bs) {
  __shared__ float t[TK][TN + 1];
  const int c0 = bx * TN;
  for (int e = threadIdx.x; e < TK * TN; e += blockDim.x) {
    const int k = e / TN, c = e % TN;
    const int gk = kb * TK + k, gc = c0 + c;
    t[k][c] = (gk < K && gc < nc) ? B[int64_t(gk) * ldb + gc] : 0.f;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ncp = ceil_div(nc, TN) * TN;
  for (int c = warp; c < TN; c += blockDim.x / 32) {
    const int gc = c0 + c;
    if (gc >= nc) {
      if (lane == 0) Bs[kb * ncp + gc] = 0.f;
      continue;
    }
    float v[2] = {t[lane][c], t[lane + 32][c]};
    float mx = fmaxf(fabsf(v[0]), fabsf(v[1]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const int e = exp_of(mx);
    if (lane == 0) Bs[kb * ncp + gc] = pow2f(e - 8);
    const float scale = pow2f(8 - e);
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      float x = __fmul_rn(v[u], scale);
      const int64_t base = int64_t(gc) * Kp + kb * TK + lane + 32 * u;
#pragma unroll
      for (int p = 0; p < kDigits; ++p) {
        const float d = rintf(x);
        Bd[int64_t(p) * nc * Kp + base] = __float2bfloat16_rn(d);
        x = __fmul_rn(__fsub_rn(x, d), 512.f);
      }
    }
  }
}

// Both digit passes of one update in a single launch: blocks [0, row_blocks) take the rows of A, the next
// col_tiles x nkb blocks the (column tile, k block) tiles of B.
__global__ void __launch_bounds__(256) digits_kernel(const float* __restrict__ A, int64_t lda, int m,
                                                     const float* __restrict__ B, int64_t ldb, int nc, int K, int Kp,
                                                     int row_blocks, int col_tiles, __nv_bfloat16* __restrict__ Ad,
                                                     float* __restrict__ As, __nv_bfloat16* __restrict__ Bd,
                                                     float* __restrict__ Bs) {
  const int b = int(blockIdx.x);
  if (b < row_blocks) {
    digits_rows(b, A, lda, m, K, Kp, Ad, As);
  } else {
    const int q = b - row_blocks;
    digits_cols(q % col_tiles, q / col_tiles, B, ldb, nc, K, Kp, Bd, Bs);
  }
}

// ---- main kernel ---------------------------------------------------------------------------------------
struct Ctrl {
  // With two stages and two accumulator sets, k block j uses stage j % 2 and set j % 2: the one commit of its
  // MMAs (tfull[j % 2]) both hands the set to the epilogue and frees the stage for the producer.
  uint64_t full[kStages], tfull[2], tempty[2], cfull, cready;
  uint32_t tmem;
  int abort_flag;
};

// 18 warps: a sub-partition holds up to 5 of them in its 16,384 registers, so at most 96 registers a thread
__global__ void __launch_bounds__(kThreads, 1)
    ozaki3_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                  const __grid_constant__ CUtensorMap tmCh, const __grid_constant__ CUtensorMap tmCl,
                  const float* __restrict__ As, const float* __restrict__ Bs, int m, int nc, int Kp,
                  DeviceStatus* st) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sC = smem + kStages * kStageBytes;  // C tile, 128B-swizzled boxes: hi[0:32], hi[32:64], lo[0:32], lo[32:64]
  __shared__ Ctrl ctl;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tiles_n = int(ceil_div(nc, TN)), tiles_m = int(ceil_div(m, TM));
  const int ntiles = tiles_n * tiles_m;
  const int64_t ncp = int64_t(tiles_n) * TN;  // row stride of the column scales
  const int nkb = Kp / TK;
  volatile int* abort_flag = &ctl.abort_flag;
  const uint64_t pol_keep = l2_policy_evict_last(), pol_stream = l2_policy_evict_first();

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&ctl.full[s], 1);
    }
    for (int s = 0; s < 2; ++s) {
      mbar_init(&ctl.tfull[s], 1);
      mbar_init(&ctl.tempty[s], kEpiWarps);
    }
    mbar_init(&ctl.cfull, 1);
    mbar_init(&ctl.cready, kEpiWarps);
    ctl.abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&ctl.tmem)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = ctl.tmem;
  int last_commit = -1;  // MMA issuer: index of the last committed k block

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmCh)) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmCl)) : "memory");
      int j = 0;
      for (int t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x) {
        const int r0 = (t / tiles_n) * TM, c0 = (t % tiles_n) * TN;
        for (int kb = 0; kb < nkb; ++kb, ++j) {
          const int s = j % kStages;
          const uint32_t ph = uint32_t(j / kStages) & 1u;
          if (!mbar_wait(&ctl.tfull[s], ph ^ 1u, abort_flag)) {  // k block j - 2's MMAs are done
            if (!*abort_flag) { status_error(st, UPDES_ERR_TIMEOUT); atomicCAS(&st->timeout_tag, 0, 41); }
            *abort_flag = 1;
            break;
          }
          uint8_t* sA = smem + s * kStageBytes;
          uint8_t* sB = sA + kDigits * kATile;
          mbar_expect_tx(&ctl.full[s], uint32_t(kStageBytes));
#pragma unroll
          for (int p = 0; p < kDigits; ++p) {
            tma_load_3d(smem_u32(sA + p * kATile), &tmA, kb * TK, r0, p, &ctl.full[s], pol_keep);
            tma_load_3d(smem_u32(sB + p * kBTile), &tmB, kb * TK, c0, p, &ctl.full[s], pol_keep);
          }
        }
      }
      if (*abort_flag) {
        // copies still in flight must land before the CTA's shared memory goes away (bounded)
        for (int jj = (j > kStages ? j - kStages : 0); jj < j; ++jj) {
          for (long long it = 0; it < (1 << 22); ++it) {
            if (mbar_try_wait(&ctl.full[jj % kStages], uint32_t(jj / kStages) & 1u)) break;
            __nanosleep(64);
          }
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int j = 0;
      for (int t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x) {
        for (int kb = 0; kb < nkb; ++kb, ++j) {
          const int s = j % kStages, set = j & 1;
          const uint32_t ph = uint32_t(j / kStages) & 1u, tph = uint32_t(j >> 1) & 1u;
          if (!mbar_wait(&ctl.full[s], ph, abort_flag) || !mbar_wait(&ctl.tempty[set], tph ^ 1u, abort_flag)) {
            if (!*abort_flag) { status_error(st, UPDES_ERR_TIMEOUT); atomicCAS(&st->timeout_tag, 0, 42); }
            *abort_flag = 1;
            break;
          }
          tc_fence_after();
          const uint8_t* sA = smem + s * kStageBytes;
          const uint64_t a0 = make_desc(smem_u32(sA)), b0 = make_desc(smem_u32(sA + kDigits * kATile));
          const uint32_t tset = tmem + uint32_t(set * kGroups * TN);
          mma_product<0, 0>(tset, a0, b0);
          mma_product<0, 1>(tset, a0, b0);
          mma_product<1, 0>(tset, a0, b0);
          mma_product<0, 2>(tset, a0, b0);
          mma_product<1, 1>(tset, a0, b0);
          mma_product<2, 0>(tset, a0, b0);
          mma_product<1, 2>(tset, a0, b0);
          mma_product<2, 1>(tset, a0, b0);
          mma_commit(&ctl.tfull[set]);
          last_commit = j;
        }
      }
    }
  } else {
    // ---------------- epilogue: lane quarter q = warp % 4, column group h ----------------
    const int q = warp & 3, h = (warp - 2) >> 2;
    const int row_in_tile = q * 32 + lane;
    const int colbase = h * kEpiCols;
    const uint32_t lane_base = uint32_t(q * 32) << 16;
    int j = 0, tl = 0;
    // the storer stores each tile's C and, as soon as the store has read the buffer, loads the next tile's C
    // into it, so that the operand stream of the producer never waits on the C buffer
    const bool storer = (warp == 2 && lane == 0);
    int c_pending = -1;  // storer: local index of the tile whose C load is in flight and not yet waited for
    auto load_c = [&](int t_next, int tl_next) {
      const int r0n = (t_next / tiles_n) * TM, c0n = (t_next % tiles_n) * TN;
      mbar_expect_tx(&ctl.cfull, uint32_t(kCBytes));
      tma_load_2d(smem_u32(sC), &tmCh, c0n, r0n, &ctl.cfull, pol_stream);
      tma_load_2d(smem_u32(sC + kCHalf), &tmCh, c0n + 32, r0n, &ctl.cfull, pol_stream);
      tma_load_2d(smem_u32(sC + 2 * kCHalf), &tmCl, c0n, r0n, &ctl.cfull, pol_stream);
      tma_load_2d(smem_u32(sC + 3 * kCHalf), &tmCl, c0n + 32, r0n, &ctl.cfull, pol_stream);
      c_pending = tl_next;
    };
    if (storer && blockIdx.x < ntiles) load_c(blockIdx.x, 0);
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++tl) {
      const int r0 = (t / tiles_n) * TM, c0 = (t % tiles_n) * TN;
      const int gr = r0 + row_in_tile;
      // accumulators of the thread's row over its kEpiCols columns, as column pairs
      float2 acc_h[kEpiCols / 2], acc_l[kEpiCols / 2];
#pragma unroll
      for (int u = 0; u < kEpiCols / 2; ++u) { acc_h[u] = make_float2(0.f, 0.f); acc_l[u] = make_float2(0.f, 0.f); }
      bool ok = true;
      for (int kb = 0; kb < nkb; ++kb, ++j) {
        const int set = j & 1;
        const uint32_t tph = uint32_t(j >> 1) & 1u;
        // scales of this k block: the row's (loaded before the wait) and, per chunk of four columns, the
        // columns' (the same 16-byte vector for every lane: one broadcast load)
        const float sa = gr < m ? __ldg(As + int64_t(gr) * nkb + kb) : 0.f;
        const float4* sbp = reinterpret_cast<const float4*>(Bs + int64_t(kb) * ncp + c0 + colbase);
        // every wait ends in a warp vote, so a warp always leaves together (tcgen05.ld needs all 32 lanes)
        if (!__all_sync(0xffffffffu, mbar_wait(&ctl.tfull[set], tph, abort_flag))) {
          if (lane == 0 && !*abort_flag) { status_error(st, UPDES_ERR_TIMEOUT); atomicCAS(&st->timeout_tag, 0, 43); }
          *abort_flag = 1;
          ok = false;
          break;
        }
        tc_fence_after();
#pragma unroll
        for (int ch = 0; ch < kEpiCols / 4; ++ch) {
          const int col = colbase + ch * 4;
          const float4 s4 = __ldg(sbp + ch);
          float g[kGroups][4];
#pragma unroll
          for (int gi = 0; gi < kGroups; ++gi)
            tmem_ld4(tmem + lane_base + uint32_t(set * kGroups * TN + gi * TN + col), g[gi]);
          tmem_wait_ld();
          if (ch == kEpiCols / 4 - 1) {
            // every chunk has been read: release the accumulator set to the MMA issuer
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&ctl.tempty[set]);
          }
          const float2 c9 = make_float2(1.953125e-3f, 1.953125e-3f);          // 2^-9
          const float2 c18 = make_float2(3.814697265625e-06f, 3.814697265625e-06f);  // 2^-18
          const float2 sa2 = make_float2(sa, sa);
#pragma unroll
          for (int u = 0; u < 4; u += 2) {
            const int cu = ch * 4 + u;  // the pair's first column among the thread's kEpiCols
            const float2 sb2 = u ? make_float2(s4.z, s4.w) : make_float2(s4.x, s4.y);
            // k-block value = g0 + 2^-9 g1 + 2^-18 (g2 + 2^-9 g3): g0 + 2^-9 g1 exactly as (hh, ll); the two
            // small groups merged in one rounding (about 2^-40 of the block's scale, far below the digit cut)
            float2 hh, ll;
            two_sum2(make_float2(g[0][u], g[0][u + 1]), __fmul2_rn(make_float2(g[1][u], g[1][u + 1]), c9), hh, ll);
            const float2 g23 = __ffma2_rn(make_float2(g[3][u], g[3][u + 1]), c9, make_float2(g[2][u], g[2][u + 1]));
            ll = __ffma2_rn(g23, c18, ll);
            const float2 sc = __fmul2_rn(sa2, sb2);  // powers of two: exact
            hh = __fmul2_rn(hh, sc);
            ll = __fmul2_rn(ll, sc);
            // acc += (hh, ll); the low word is renormalised by the final update of C (K <= 1024: at most 16 blocks)
            float2 s1, t1;
            two_sum2(acc_h[cu >> 1], hh, s1, t1);
            acc_h[cu >> 1] = s1;
            acc_l[cu >> 1] = __fadd2_rn(acc_l[cu >> 1], __fadd2_rn(t1, ll));
          }
        }
      }
      if (!ok) break;
      // ---- C -= acc in shared memory (the tile arrived by TMA), then one thread stores it back ----
      if (!__all_sync(0xffffffffu, mbar_wait(&ctl.cfull, uint32_t(tl) & 1u, abort_flag))) {
        if (lane == 0 && !*abort_flag) { status_error(st, UPDES_ERR_TIMEOUT); atomicCAS(&st->timeout_tag, 0, 45); }
        *abort_flag = 1;
        break;
      }
      if (storer) c_pending = -1;
      {
        // this thread's row in the 128B-swizzled boxes: 16-byte chunk q of row r sits at chunk q ^ (r & 7)
        const int r = row_in_tile;
        const int half = colbase >> 5, qbase = (colbase & 31) >> 2;  // box and first 16-byte chunk
        uint8_t* hrow = sC + half * kCHalf + (r >> 3) * 1024 + (r & 7) * 128;
        uint8_t* lrow = hrow + 2 * kCHalf;
#pragma unroll
        for (int qq = 0; qq < kEpiCols / 4; ++qq) {
          const int off = (((qbase + qq) ^ (r & 7)) << 4);
          const float4 hv = *reinterpret_cast<float4*>(hrow + off), lv = *reinterpret_cast<float4*>(lrow + off);
          float2 hx[2] = {make_float2(hv.x, hv.y), make_float2(hv.z, hv.w)};
          float2 lx[2] = {make_float2(lv.x, lv.y), make_float2(lv.z, lv.w)};
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            float2 sx, tx;
            two_sum2(hx[u], make_float2(-acc_h[qq * 2 + u].x, -acc_h[qq * 2 + u].y), sx, tx);
            tx = __fadd2_rn(tx, sub2(lx[u], acc_l[qq * 2 + u]));
            fast_two_sum2(sx, tx, hx[u], lx[u]);
          }
          *reinterpret_cast<float4*>(hrow + off) = make_float4(hx[0].x, hx[0].y, hx[1].x, hx[1].y);
          *reinterpret_cast<float4*>(lrow + off) = make_float4(lx[0].x, lx[0].y, lx[1].x, lx[1].y);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic writes -> visible to TMA
      __syncwarp();
      if (lane == 0) mbar_arrive(&ctl.cready);
      bool stop = false;
      if (storer) {
        if (!mbar_wait(&ctl.cready, uint32_t(tl) & 1u, abort_flag)) {
          if (!*abort_flag) { status_error(st, UPDES_ERR_TIMEOUT); atomicCAS(&st->timeout_tag, 0, 46); }
          *abort_flag = 1;
          stop = true;
        }
      }
      if (storer && !stop) {
        // rows >= m and columns >= nc are outside the tensor and are not written
        tma_store_2d(&tmCh, c0, r0, smem_u32(sC), pol_stream);
        tma_store_2d(&tmCh, c0 + 32, r0, smem_u32(sC + kCHalf), pol_stream);
        tma_store_2d(&tmCl, c0, r0, smem_u32(sC + 2 * kCHalf), pol_stream);
        tma_store_2d(&tmCl, c0 + 32, r0, smem_u32(sC + 3 * kCHalf), pol_stream);
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // the buffer has been read
        if (t + int(gridDim.x) < ntiles && !*abort_flag) load_c(t + int(gridDim.x), tl + 1);
      }
      if (__any_sync(0xffffffffu, stop)) break;  // the whole warp leaves together
    }
    if (storer) {
      asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");  // stores complete before exit
      if (c_pending >= 0) {
        // a C load still in flight (only after an abort) must land before shared memory goes away (bounded)
        for (long long it = 0; it < (1 << 22); ++it) {
          if (mbar_try_wait(&ctl.cfull, uint32_t(c_pending) & 1u)) break;
          __nanosleep(64);
        }
      }
    }
  }

  // ---- teardown: all roles done; make sure no MMA is in flight before tensor memory is freed ----
  __syncthreads();
  if (warp == 1) {
    if (ctl.abort_flag && lane == 0 && last_commit >= 0) {
      // MMAs complete in order: once the last commit has arrived nothing reads tensor memory (bounded)
      for (long long it = 0; it < (1 << 22); ++it) {
        if (mbar_try_wait(&ctl.tfull[last_commit & 1], uint32_t(last_commit >> 1) & 1u)) break;
        __nanosleep(64);
      }
    }
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

// cuTensorMapEncodeTiled, resolved at run time through the runtime's entry-point query, so the library
// does not link against the driver library and still loads on hosts without a GPU driver.
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// 3-D map over digit planes [3][rows][Kp] bf16, box 64 (k) x box_rows x 1, 128B swizzle
int make_map(CUtensorMap* map, void* base, int rows, int Kp, int box_rows) {
  cuuint64_t dims[3] = {cuuint64_t(Kp), cuuint64_t(rows), cuuint64_t(kDigits)};
  cuuint64_t strides[2] = {cuuint64_t(Kp) * 2, cuuint64_t(rows) * Kp * 2};
  cuuint32_t box[3] = {cuuint32_t(TK), cuuint32_t(box_rows), 1};
  cuuint32_t estr[3] = {1, 1, 1};
  const EncodeTiledFn fn = encode_tiled();
  if (!fn) return UPDES_ERR_CUDA;
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? UPDES_OK : UPDES_ERR_CUDA;
}

// 2-D map over an FP32 plane (rows x cols, row stride ld elements), box 32 columns x 128 rows, 128B swizzle
int make_map_c(CUtensorMap* map, float* base, int rows, int cols, int64_t ld) {
  const EncodeTiledFn fn = encode_tiled();
  if (!fn) return UPDES_ERR_CUDA;
  cuuint64_t dims[2] = {cuuint64_t(cols), cuuint64_t(rows)};
  cuuint64_t strides[1] = {cuuint64_t(ld) * 4};
  cuuint32_t box[2] = {32, cuuint32_t(TM)};
  cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? UPDES_OK : UPDES_ERR_CUDA;
}

int num_sms_cached() {
  static std::atomic<int> sms{0};
  if (!sms.load()) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    sms.store(v > 0 ? v : 1);
  }
  return sms.load();
}

}  // namespace

size_t ozaki3_scratch_bytes(int mmax, int ncmax, int Kmax) {
  const size_t Kp = size_t(ceil_div(Kmax, TK)) * TK;
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  return al(kDigits * size_t(mmax) * Kp * 2) + al(kDigits * size_t(ncmax) * Kp * 2) + al(size_t(mmax) * (Kp / TK) * 4) +
         al(size_t(ceil_div(ncmax, TN)) * TN * (Kp / TK) * 4) + 256;
}

int ozaki3_update(float* Chi, float* Clo, int64_t ldc, const float* A, int64_t lda, const float* B, int64_t ldb,
                  int m, int nc, int K, void* scratch, size_t scratch_bytes, DeviceStatus* st, cudaStream_t s,
                  int max_ctas, bool a_digits_ready) {
  if (m <= 0 || nc <= 0 || K <= 0) return UPDES_OK;
  // the tile accumulator's low word is left unnormalised across k blocks: a few blocks only
  if (K > 1024) return UPDES_ERR_UNSUPPORTED;
  if (!scratch || scratch_bytes < ozaki3_scratch_bytes(m, nc, K)) return UPDES_ERR_WORKSPACE;
  if ((reinterpret_cast<uintptr_t>(scratch) & 255) != 0) return UPDES_ERR_INVALID;
  // C goes through TMA: 16-byte aligned planes and row stride (else the caller uses the other kernel)
  if (((reinterpret_cast<uintptr_t>(Chi) | reinterpret_cast<uintptr_t>(Clo)) & 15) != 0 || (ldc & 3) != 0)
    return UPDES_ERR_UNSUPPORTED;
  const int Kp = int(ceil_div(K, TK)) * TK, nkb = Kp / TK;
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  // A's digits and scales first: their place depends only on m and K, so an update with the same A can reuse them
  char* p = static_cast<char*>(scratch);
  __nv_bfloat16* Ad = reinterpret_cast<__nv_bfloat16*>(p);
  p += al(kDigits * size_t(m) * Kp * 2);
  float* As = reinterpret_cast<float*>(p);
  p += al(size_t(m) * nkb * 4);
  __nv_bfloat16* Bd = reinterpret_cast<__nv_bfloat16*>(p);
  p += al(kDigits * size_t(nc) * Kp * 2);
  float* Bs = reinterpret_cast<float*>(p);

  static std::atomic<unsigned long long> attr{0};
  if (int e = smem_opt_in((const void*)ozaki3_kernel, kSmemBytes, attr)) return e;
  CUtensorMap mapA, mapB, mapCh, mapCl;
  int e = make_map(&mapA, Ad, m, Kp, TM);
  if (e) return e;
  if ((e = make_map(&mapB, Bd, nc, Kp, TN))) return e;
  if ((e = make_map_c(&mapCh, Chi, m, nc, ldc))) return e;
  if ((e = make_map_c(&mapCl, Clo, m, nc, ldc))) return e;

  StatScope sc(kStatGemm, s, 2.0 * m * double(nc) * K, double(m) * nc * 16.0 + (double(m) + nc) * K * 4.0);
  {
    const int64_t warps = int64_t(m) * nkb;
    const int row_blocks = a_digits_ready ? 0 : int(ceil_div(warps * 32, 256)), col_tiles = int(ceil_div(nc, TN));
    digits_kernel<<<unsigned(row_blocks + col_tiles * nkb), 256, 0, s>>>(A, lda, m, B, ldb, nc, K, Kp, row_blocks,
                                                                      col_tiles, Ad, As, Bd, Bs);
    UPDES_LAUNCH_CHECK();
  }
  const int ntiles = int(ceil_div(m, TM) * ceil_div(nc, TN));
  const int grid = std::min(ntiles, max_ctas > 0 ? std::min(max_ctas, num_sms_cached()) : num_sms_cached());
  ozaki3_kernel<<<grid, kThreads, kSmemBytes, s>>>(mapA, mapB, mapCh, mapCl, As, Bs, m, nc, Kp, st);
  UPDES_LAUNCH_CHECK();
  return UPDES_OK;
}

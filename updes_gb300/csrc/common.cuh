// Shared helpers for the updes_gb300 CUDA sources (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "../../include/updes_gb300.h"

#define UPDES_CUDA_TRY(expr)                                   \
  do {                                                         \
    cudaError_t _e = (expr);                                   \
    if (_e != cudaSuccess) {                                   \
      updes_set_last_cuda_error(_e, #expr, __FILE__, __LINE__); \
      return UPDES_ERR_CUDA;                                   \
    }                                                          \
  } while (0)

void stats_count_launch(int n);
#define UPDES_LAUNCH_CHECK()          \
  do {                                \
    stats_count_launch(1);            \
    UPDES_CUDA_TRY(cudaGetLastError()); \
  } while (0)

// Records the last CUDA error (text retrievable through updes_last_error()) and clears the calling
// thread's pending runtime error, so that a failure reported once is not reported again by the next
// launch check of an unrelated call on the same thread.
void updes_set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line);

// Raises a kernel's dynamic shared-memory limit to `bytes` on the current device, once per device
// (`done` holds one bit per device ordinal).  The limit belongs to the function on the device and is
// shared by every host thread, so it is set to the kernel's largest need and never changed per call: a
// per-call value set by one thread could undercut a launch that another thread is about to make.
inline int smem_opt_in(const void* func, int bytes, std::atomic<unsigned long long>& done) {
  int dev = 0;
  UPDES_CUDA_TRY(cudaGetDevice(&dev));
  const unsigned long long bit = 1ull << (dev & 63);
  if (done.load() & bit) return UPDES_OK;
  UPDES_CUDA_TRY(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  done.fetch_or(bit);
  return UPDES_OK;
}

// Device-side status word layout (written by kernels, read by the host after a sync).
// word 0: first error code (UPDES_ERR_*) raised by any kernel, 0 if none
// word 1: LU info (1 + first step with a zero / non-finite pivot), 0 if none
// word 2: where a bounded wait gave up (kernel-specific tag)
struct DeviceStatus {
  int32_t error;
  int32_t lu_info;
  int32_t timeout_tag;
  int32_t pad;
};

__device__ __forceinline__ void status_error(DeviceStatus* st, int code) {
  atomicCAS(&st->error, 0, code);
}

__host__ __device__ __forceinline__ int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Iteration cap of the spin-waits between CTAs (grid barriers, panel records, triangular-solve flags; each
// iteration also sleeps 20-64 ns): a few seconds at most by default.  updes_set_spin_limit changes it at run
// time on the current device.  Without relocatable device code every translation unit holds its own copy
// of the variable, so each unit registers a setter for its copy (below) and that call runs all of them.
constexpr long long kDefaultSpinLimit = 1ll << 26;
static __device__ long long g_spin_limit = kDefaultSpinLimit;
__device__ __forceinline__ long long spin_limit() { return g_spin_limit; }

// Iteration cap of the tensor-core update's mbarrier waits.  It stays a constant: when such a wait gives up,
// the kernel still waits for its own copies in flight before it leaves, and that wait must be long enough
// for the copies to land whatever limit a caller sets for the waits between CTAs.
constexpr long long kTcSpinLimit = kDefaultSpinLimit;

int register_spin_limit_setter(int (*setter)(long long));
namespace {
inline int set_unit_spin_limit(long long v) { return int(cudaMemcpyToSymbol(g_spin_limit, &v, sizeof(v))); }
const int g_spin_setter_registered = register_spin_limit_setter(&set_unit_spin_limit);
}  // namespace

// Grid-wide barrier for a cooperative launch (all CTAs co-resident).
// `bar` points at two words: arrival count and generation.  Returns false if
// the wait gave up (the caller must then stop and report UPDES_ERR_TIMEOUT).
__device__ __forceinline__ bool grid_barrier(unsigned int* bar, unsigned int nblocks, DeviceStatus* st,
                                             int tag) {
  __syncthreads();
  __shared__ int ok;
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned int* vgen = bar + 1;
    unsigned int gen = *vgen;
    __threadfence();
    unsigned int ticket = atomicAdd(bar, 1u);
    if (ticket == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const long long lim = spin_limit();
      long long it = 0;
      while (*vgen == gen) {
        if (++it > lim) {
          ok = 0;
          status_error(st, UPDES_ERR_TIMEOUT);
          atomicCAS(&st->timeout_tag, 0, tag);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

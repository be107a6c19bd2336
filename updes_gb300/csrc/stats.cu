#include <atomic>
#include <mutex>
#include <vector>

#include "stats.cuh"

namespace {
std::atomic<long long> g_launches{0};
std::atomic<int> g_timing{0};
std::mutex g_mu;
struct Rec {
  int cat;
  cudaEvent_t a, b;
  double flops, bytes;
};
std::vector<Rec> g_recs;
double g_ms[kStatCount], g_flops[kStatCount], g_bytes[kStatCount];
long long g_count[kStatCount];

void resolve_locked() {
  for (auto& r : g_recs) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      g_ms[r.cat] += ms;
      g_flops[r.cat] += r.flops;
      g_bytes[r.cat] += r.bytes;
      g_count[r.cat] += 1;
    }
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  g_recs.clear();
}
}  // namespace

void stats_count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
bool stats_timing() { return g_timing.load(std::memory_order_relaxed) != 0; }

StatScope::StatScope(int c, cudaStream_t st, double fl, double by) : cat(c), s(st), ev0(nullptr), flops(fl), bytes(by) {
  if (!stats_timing()) return;
  // no timing of work recorded into a CUDA graph (its events would never complete on their own)
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
  cudaEvent_t a;
  if (cudaEventCreate(&a) == cudaSuccess) {
    cudaEventRecord(a, s);
    ev0 = a;
  }
}

StatScope::~StatScope() {
  if (!ev0) return;
  cudaEvent_t b;
  if (cudaEventCreate(&b) != cudaSuccess) {
    cudaEventDestroy(static_cast<cudaEvent_t>(ev0));
    return;
  }
  cudaEventRecord(b, s);
  std::lock_guard<std::mutex> lk(g_mu);
  g_recs.push_back(Rec{cat, static_cast<cudaEvent_t>(ev0), b, flops, bytes});
}

extern "C" void updes_stats_reset(int32_t enable_timing) {
  std::lock_guard<std::mutex> lk(g_mu);
  resolve_locked();
  for (int i = 0; i < kStatCount; ++i) g_ms[i] = g_flops[i] = g_bytes[i] = 0.0, g_count[i] = 0;
  g_launches.store(0);
  g_timing.store(enable_timing ? 1 : 0);
}

extern "C" void updes_stats_read(updes_stats* out) {
  if (!out) return;
  std::lock_guard<std::mutex> lk(g_mu);
  resolve_locked();
  out->launches = g_launches.load();
  for (int i = 0; i < kStatCount; ++i) {
    out->count[i] = g_count[i];
    out->ms[i] = g_ms[i];
    out->flops[i] = g_flops[i];
    out->bytes[i] = g_bytes[i];
  }
}

// ---- run-time limit of the spin-waits between CTAs ------------------------------------------------------

namespace {
std::mutex g_spin_mu;
std::vector<int (*)(long long)>& spin_setters() {
  static std::vector<int (*)(long long)> v;  // constructed on first use: registration runs at load time
  return v;
}
}  // namespace

int register_spin_limit_setter(int (*setter)(long long)) {
  std::lock_guard<std::mutex> lk(g_spin_mu);
  spin_setters().push_back(setter);
  return 0;
}

extern "C" int updes_set_spin_limit(int64_t iterations) {
  if (iterations < 0) return UPDES_ERR_INVALID;
  const long long v = iterations == 0 ? kDefaultSpinLimit : (long long)iterations;
  std::lock_guard<std::mutex> lk(g_spin_mu);
  for (auto fn : spin_setters()) {
    const cudaError_t e = cudaError_t(fn(v));
    if (e != cudaSuccess) {
      updes_set_last_cuda_error(e, "cudaMemcpyToSymbol(g_spin_limit)", __FILE__, __LINE__);
      return UPDES_ERR_CUDA;
    }
  }
  return UPDES_OK;
}

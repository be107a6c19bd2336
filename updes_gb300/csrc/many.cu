// Many independent collocation systems in one call (clouds of different sizes, kernels and boundary
// conditions, as in a parameter sweep).  The reference solves each with its own pde_solver call
// (updes/operators.py:559-618), one after the other.  Here `streams` host threads each drive one CUDA
// stream with its own slice of the workspace and take the next unsolved system (largest first, so the
// long solves start early) until none is left; every solve is updes_solve's assemble -> mixed LU ->
// refinement -> values.  Small systems leave most of the GPU idle on their own, so the streams overlap
// their factorisations and refinements.
#include <algorithm>
#include <atomic>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"

void updes_set_last_error_text(const std::string& text);
std::string updes_last_error_text();

namespace {

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

int max_slice_bytes(const updes_problem* problems, int32_t count, const updes_solve_opts* opts, size_t* out) {
  size_t mx = 0;
  for (int32_t i = 0; i < count; ++i) {
    size_t b = 0;
    const int e = updes_solve_workspace(&problems[i], opts, &b);
    if (e) return e;
    mx = std::max(mx, b);
  }
  *out = align256(mx);
  return UPDES_OK;
}

}  // namespace

extern "C" int updes_solve_many_workspace(const updes_problem* problems, int32_t count,
                                          const updes_solve_opts* opts, int32_t streams, size_t* bytes) {
  if (!problems || count <= 0 || streams <= 0 || streams > 64 || !bytes) return UPDES_ERR_INVALID;
  size_t slice = 0;
  const int e = max_slice_bytes(problems, count, opts, &slice);
  if (e) return e;
  *bytes = slice * size_t(std::min<int32_t>(streams, count)) + 256;
  return UPDES_OK;
}

extern "C" int updes_solve_many(const updes_problem* problems, int32_t count, const double* const* q,
                                double* const* coeffs, double* const* vals, const updes_solve_opts* opts,
                                updes_solve_info* infos, void* workspace, size_t workspace_bytes, int32_t streams) {
  if (!problems || count <= 0 || !q || !coeffs || streams <= 0 || streams > 64 || !workspace)
    return UPDES_ERR_INVALID;
  size_t slice = 0;
  int e = max_slice_bytes(problems, count, opts, &slice);
  if (e) return e;
  const int nstreams = std::min<int32_t>(streams, count);
  if (workspace_bytes < slice * size_t(nstreams) + 256) return UPDES_ERR_WORKSPACE;
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));

  // largest systems first
  std::vector<int32_t> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
    return problems[a].N + problems[a].M > problems[b].N + problems[b].M;
  });

  int dev = 0;
  UPDES_CUDA_TRY(cudaGetDevice(&dev));
  std::vector<cudaStream_t> ss(nstreams, nullptr);
  for (int t = 0; t < nstreams; ++t) {
    if (cudaStreamCreateWithFlags(&ss[t], cudaStreamNonBlocking) != cudaSuccess) {
      for (int u = 0; u < t; ++u) cudaStreamDestroy(ss[u]);
      return UPDES_ERR_CUDA;
    }
  }
  std::atomic<int32_t> next{0};
  std::atomic<int> first_error{UPDES_OK};
  std::string first_text;  // written once, by the thread whose failure is reported
  auto solve_one = [&](int t, int32_t k) {
    const int32_t i = order[k];
    updes_solve_info local;
    updes_solve_info* info = infos ? &infos[i] : &local;
    const int st = updes_solve(&problems[i], q[i], coeffs[i], vals ? vals[i] : nullptr, opts, info,
                               base + slice * size_t(t), slice, ss[t]);
    if (st) {
      int expected = UPDES_OK;
      if (first_error.compare_exchange_strong(expected, st))
        first_text = "system " + std::to_string(i) + (st == UPDES_ERR_CUDA ? ": " + updes_last_error_text() : "");
    }
  };
  // The first (largest) system on the calling thread: it also performs the library's one-time kernel
  // set-up before any worker starts.
  solve_one(0, next.fetch_add(1));
  auto worker = [&](int t) {
    cudaSetDevice(dev);
    for (;;) {
      const int32_t k = next.fetch_add(1);
      if (k >= count) break;
      solve_one(t, k);
    }
  };
  std::vector<std::thread> threads;
  for (int t = 1; t < nstreams; ++t) threads.emplace_back(worker, t);
  worker(0);
  for (auto& th : threads) th.join();
  for (int t = 0; t < nstreams; ++t) {
    cudaStreamSynchronize(ss[t]);
    cudaStreamDestroy(ss[t]);
  }
  const int e0 = first_error.load();
  if (e0) updes_set_last_error_text(first_text);
  return e0;
}

// Launch counting and optional per-category CUDA-event timing (for the bench's
// live roofline: launches, device time and algorithmic work of each kernel class).
#pragma once

#include "common.cuh"

enum StatCat { kStatGemm = 0, kStatPanel, kStatTrsm, kStatTrsv, kStatGemv, kStatAssemble, kStatOther, kStatCount };


bool stats_timing();
// Record an event pair around launches of one category on stream s (no-op unless timing is on).
struct StatScope {
  int cat;
  cudaStream_t s;
  void* ev0;
  double flops, bytes;
  StatScope(int c, cudaStream_t st, double fl = 0.0, double by = 0.0);
  ~StatScope();
};

// Tensor-core trailing update of the mixed-precision LU (see gemm_tc.cu).
#pragma once

#include "common.cuh"

struct GemmTcCtx {
  void* ws;
  size_t ws_bytes;
};

bool gemm_tc_enabled();
size_t gemm_tc_workspace_bytes(int n);
int gemm_tc_update(void* ctx, int n, int k, int nb, double* W, int64_t ldw, const void* F, int64_t ldf,
                   cudaStream_t s);

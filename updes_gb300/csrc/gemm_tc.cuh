// Tensor-core trailing update of the mixed-precision LU (see gemm_tc.cu).
#pragma once

#include "common.cuh"


// C (double-float planes hi/lo, ldc) -= A (m x K FP32, lda) * B (K x nc FP32, ldb), products exact.
int ozaki_update(float* Chi, float* Clo, int64_t ldc, const float* A, int64_t lda, const float* B, int64_t ldb,
                 int m, int nc, int K, DeviceStatus* st, cudaStream_t s);

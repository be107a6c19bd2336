// Tensor-core trailing update of the mixed-precision LU (see gemm_tc.cu).
#pragma once

#include "common.cuh"


// C (double-float planes hi/lo, ldc) -= A (m x K FP32, lda) * B (K x nc FP32, ldb), products exact.
int ozaki_update(float* Chi, float* Clo, int64_t ldc, const float* A, int64_t lda, const float* B, int64_t ldb,
                 int m, int nc, int K, DeviceStatus* st, cudaStream_t s);

// The persistent, warp-specialised version (gemm_tc3.cu): digits written once per update into `scratch`
// (ozaki3_scratch_bytes(m, nc, K) bytes, 256-byte aligned), 8 digit products, TMA-fed.  The kernel keeps one
// CTA per SM; `max_ctas` > 0 caps its grid so that work on another stream keeps the remaining SMs.
size_t ozaki3_scratch_bytes(int mmax, int ncmax, int Kmax);
// a_digits_ready: the previous update on `scratch` had the same A (same m, K and values), whose digits and
// scales are still there; only B's are written.
int ozaki3_update(float* Chi, float* Clo, int64_t ldc, const float* A, int64_t lda, const float* B, int64_t ldb,
                  int m, int nc, int K, void* scratch, size_t scratch_bytes, DeviceStatus* st, cudaStream_t s,
                  int max_ctas = 0, bool a_digits_ready = false);

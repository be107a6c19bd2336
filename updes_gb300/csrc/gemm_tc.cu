// Tensor-core trailing update of the mixed-precision LU (not yet enabled:
// the SIMT FP64-accumulating update in lu.cu runs instead).
#include "gemm_tc.cuh"

bool gemm_tc_enabled() { return false; }
size_t gemm_tc_workspace_bytes(int n) { (void)n; return 0; }
int gemm_tc_update(void*, int, int, int, double*, int64_t, const void*, int64_t, cudaStream_t) {
  return UPDES_ERR_UNSUPPORTED;
}

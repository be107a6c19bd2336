// Internal interface of the LU and triangular-solve kernels.
#pragma once

#include "common.cuh"

constexpr int kLuNb = 64;  // panel width

// Optional replacement of the trailing update W[k+nb:, k+nb:] -= F21 * F12.
struct LuHooks {
  void* ctx;
  int (*gemm)(void* ctx, int n, int k, int nb, double* W, int64_t ldw, const void* F, int64_t ldf, cudaStream_t s);
};

size_t lu_panel_workspace_bytes(int nb);

template <typename TF>
int lu_factor_impl(int n, double* W, int64_t ldw, TF* F, int64_t ldf, int32_t* piv, void* ws, size_t ws_bytes,
                   DeviceStatus* st, cudaStream_t s, const LuHooks* hooks);

// mode: 0 = L, 1 = U, 2 = U^T, 3 = L^T (x overwritten in place); sync_ws: ceil(n/64)+1 ints.
// dinv (FP32 factors only, may be null): inverted diagonal blocks from diag_inverse, applied as matvecs
// instead of the substitution inside each block.
// xh, xl (n FP32 each, may be null): scratch planes that carry solved blocks in double-float between CTAs
// (used together with dinv).
// dinv128 (with dinv, xh, xl): inverted 128 x 128 diagonal blocks from diag_inverse128, for the 128-row solve.
// xtag (with dinv128, may be null): 2n 8-byte words through which the 128-row solve hands each solved block
// to the blocks after it, the double-float value and the block's tag in one word (no flag, no fence).
template <typename TF>
int trsv_impl(int n, const TF* F, int64_t ldf, double* x, int mode, int* sync_ws, DeviceStatus* st, cudaStream_t s,
              const float* dinv = nullptr, float* xh = nullptr, float* xl = nullptr, const float* dinv128 = nullptr,
              unsigned long long* xtag = nullptr);

// Inverses of the 64 x 64 diagonal blocks of FP32 LU factors, as double-float planes (diag_inverse_bytes).
size_t diag_inverse_bytes(int n);
int diag_inverse(int n, const float* F, int64_t ldf, float* dinv, cudaStream_t s);
// Inverses of the 128 x 128 diagonal blocks, composed from those of diag_inverse (diag_inverse128_bytes).
size_t diag_inverse128_bytes(int n);
int diag_inverse128(int n, const float* F, int64_t ldf, const float* dinv64, float* dinv128, cudaStream_t s);

// Mixed LU on a double-float working matrix (Whi, Wlo FP32 planes): factors in FP32 (overwriting Whi),
// every trailing update formed exactly on the tensor cores and accumulated in double-float.
size_t lu_df_workspace_bytes(int n);
int lu_factor_df(int n, float* Whi, float* Wlo, int64_t ld, int32_t* piv, void* ws, size_t ws_bytes, DeviceStatus* st,
                 cudaStream_t s);

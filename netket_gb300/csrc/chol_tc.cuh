// Tensor-core blocked Cholesky (chol_tc.cu): the factor of the refined solve.
#pragma once

#include <cuda_fp16.h>

#include "common.cuh"

namespace vmck {

// Rows of a block row of the factorisation (the K of the trailing update, and
// the K stride of the split panel): chol_block_rows(n) is CHOL_BLOCK below
// n = CHOL_BIG_N / 2, 1024 up to 1.5 CHOL_BIG_N and 2048 above (each block step
// reads and writes the trailing matrix once, so at large n a taller block cuts
// that traffic while the leaf chain no longer bounds the time), unless
// VMCK_CHOL_BLOCK (128 ... 4096, powers of two; read once per process) forces
// one.
constexpr int CHOL_BLOCK = 512;
constexpr int64_t CHOL_BIG_N = 32768;
int chol_block_rows(int64_t n);

// An operand of tc_gemm: FP16 hi / lo rows of a split FP32 matrix, K contiguous
// (element (row, k) at hi[row * ld + k]); TMA sees kdim x rows and fills zeros
// beyond.  ld must be a multiple of 8 and the bases 16-byte aligned.
struct SplitOperand {
  const __half *hi, *lo;
  int64_t ld;
  int64_t kdim;
  int64_t rows;
};

// Power-of-two s with bound * s < 2^13 (exponent clamped); 1 for a bound that is
// zero, negative or not finite.
__device__ __forceinline__ float split_scale(float bound) {
  if (!(bound > 0.0f) || !(bound <= 3.0e38f)) return 1.0f;
  int e = 0;
  frexpf(bound, &e);  // bound = f 2^e, f in [0.5, 1)
  e = max(-100, min(100, e));
  return ldexpf(1.0f, 13 - e);
}

// v s = hi + lo, both FP16 (22 significant bits together).
__device__ __forceinline__ void split_f16(float v, float s, __half &hi, __half &lo) {
  const float t = v * s;
  hi = __float2half_rn(t);
  lo = __float2half_rn(t - __half2float(hi));
}

// C[m + nn ldc] = alpha (A_op B_op^T)(m, nn) / (sa sb) + beta C (tri: m <= nn
// only) on the tensor cores (chol_tc.cu); optional split output of the result.
// Products hi hi + hi lo + lo hi, and lo lo with lolo.  Split K (kchunk > 0, a
// multiple of 64, below K): the K range [z kchunk, +kchunk) of every output
// tile goes to C + z zstride (partial sums, beta 0, no tri / split output).
int tc_gemm(cudaStream_t st, const SplitOperand &a, int a_row0, const SplitOperand &b,
            int b_row0, int k_off, int M, int N, int K, float *C, int64_t ldc, float alpha,
            float beta, const float *sa, const float *sb, int tri, __half *oh, __half *ol,
            int64_t ldo, int o_rows, int o_col0, const float *so, int32_t *status, int max_ctas,
            int lolo = 0, int kchunk = 0, int64_t zstride = 0);

// Device workspace (bytes) of chol_tc_factor for an n x n matrix.
int64_t chol_tc_workspace_bytes(int64_t n);

// Streams and events of the look-ahead factorisation (owned by the caller):
// chain (high priority) runs the latency-bound panel chain, side the bulk of the
// trailing updates, chain2 (high priority, optional) the rest of each panel's
// block-row update; events: chol_events_needed(n).
struct CholStreams {
  cudaStream_t chain, side;
  cudaEvent_t *events;
  int n_events;
  // (optional, high priority) the part of a panel's block-row update below the
  // next panel's rows, off the chain
  cudaStream_t chain2 = nullptr;
};
int chol_events_needed(int64_t n);

// In-place upper Cholesky A = U^T U of the column-major FP32 matrix A (n x n,
// upper triangle valid, ld n).  ws: chol_tc_workspace_bytes(n) bytes.  On
// return *yinv (inside ws) holds, per 128-row diagonal block K, Y_K = U_KK^-T as
// a zero-padded column-major 128 x 128 matrix.  Failed pivots / non-finite
// diagonals are OR-ed into *status.  With ls the trailing updates overlap the
// panel chain on two streams (the caller's stream waits for both at the end);
// without it everything runs on st.
int chol_tc_factor(cudaStream_t st, float *A, int64_t n, void *ws, int32_t *status,
                   float **yinv, const CholStreams *ls = nullptr);

}  // namespace vmck

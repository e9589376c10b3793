// Tensor-core (tcgen05) form of the structured Gram contraction; implemented in
// gram_tc.cu.
#pragma once

#include "common.cuh"

namespace vmck {

int64_t gram_tc_workspace_doubles(int M, int64_t n);

// c: shifted, rounded tanh(theta); h, w, s0sq: double-float epilogue terms
// (see gram.cu); T64 nullable.
int gram_tc_launch(vmck_ctx *ctx, cudaStream_t st, const float *c, const uint32_t *bits,
                   int words, int N, int M, int64_t n, const float2 *h, const float2 *w,
                   const float2 *s0sq, double inv_n, double diag_shift, double *T64, float *T32,
                   double *ws, int split, int32_t *status);

}  // namespace vmck

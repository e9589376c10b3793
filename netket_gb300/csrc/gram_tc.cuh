// Tensor-core (tcgen05) form of the structured Gram contraction; implemented in
// gram_tc.cu.
#pragma once

#include "common.cuh"

namespace vmck {

int64_t gram_tc_workspace_doubles(int M, int64_t n);

int gram_tc_launch(vmck_ctx *ctx, cudaStream_t st, const float *tanh_theta, const uint32_t *bits,
                   int words, int N, int M, int64_t n, const double *g, const double *cptr,
                   double inv_n, double diag_shift, double *T64, float *T32, double *ws);

}  // namespace vmck

// Structured minSR matrix for the RBM, T = O_L O_L^T + diag_shift I, formed
// without the (n, P) Jacobian.
//
// For the RBM, O(s) = [t_s | x_s (x) t_s | x_s] with t = tanh(theta), so
//   O(s).O(s') = (t_s.t_s') (1 + x_s.x_s') + x_s.x_s'
// and centring (O_c = O - 1 obar^T) gives
//   T = (G - g 1^T - 1 g^T + c 1 1^T) / n + diag_shift I,   g = O obar, c = |obar|^2.
// The dominant work is the (n x n x M) contraction t t^T; x.x' is exact integer
// arithmetic (popcount of XOR-ed sign bitmasks).  Only the lower triangle
// (row >= col, row-major) is produced, which is all the Cholesky reads.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "gram_tc.cuh"

namespace vmck {

// ---------------------------------------------------------------- helpers
__global__ void sign_bits_kernel(const int8_t *__restrict__ x, int64_t n, int N, int words,
                                 uint32_t *__restrict__ bits) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= n * words) return;
  int64_t s = e / words;
  int w = (int)(e % words);
  uint32_t v = 0;
  for (int q = 0; q < 32; ++q) {
    int i = w * 32 + q;
    if (i < N && x[s * N + i] < 0) v |= 1u << q;
  }
  bits[e] = v;
}

// g_s = t_s . (tbar + x_s^T Kbar) + x_s . xbar  (FP64); 16 samples per CTA,
// their configurations staged once in shared memory (N <= 288).
constexpr int G_SPB = 16, G_NMAX = 288;

template <typename T>
__global__ void __launch_bounds__(256) g_vector_kernel(const T *__restrict__ t,
                                                       const int8_t *__restrict__ x, int N, int M,
                                                       int64_t n, const double *__restrict__ obar,
                                                       double *__restrict__ g) {
  __shared__ int8_t xs[G_SPB][G_NMAX];
  __shared__ double part[G_SPB][8];
  const int64_t s0 = (int64_t)blockIdx.x * G_SPB;
  const double *tbar = obar, *Kbar = obar + M, *xbar = obar + M + (int64_t)N * M;
  const int ns = (int)std::min<int64_t>(G_SPB, n - s0);
  for (int e = threadIdx.x; e < G_SPB * N; e += blockDim.x) {
    int q = e / N, i = e % N;
    xs[q][i] = (q < ns) ? x[(s0 + q) * N + i] : int8_t(0);
  }
  __syncthreads();
  double gp[G_SPB];
#pragma unroll
  for (int q = 0; q < G_SPB; ++q) gp[q] = 0;
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    double y[G_SPB];
    const double tb = tbar[j];
#pragma unroll
    for (int q = 0; q < G_SPB; ++q) y[q] = tb;
    for (int i = 0; i < N; ++i) {
      const double kb = Kbar[(int64_t)i * M + j];
#pragma unroll
      for (int q = 0; q < G_SPB; ++q) y[q] += xs[q][i] > 0 ? kb : -kb;
    }
#pragma unroll
    for (int q = 0; q < G_SPB; ++q)
      if (q < ns) gp[q] += (double)t[(s0 + q) * M + j] * y[q];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < G_SPB; ++q) {
    double v = warp_sum(gp[q]);
    if (lane == 0) part[q][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < ns) {
    const int q = threadIdx.x;
    double v = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += part[q][w];
    for (int i = 0; i < N; ++i) v += xs[q][i] > 0 ? xbar[i] : -xbar[i];
    g[s0 + q] = v;
  }
}

__global__ void sumsq_kernel(const double *__restrict__ v, int64_t P, double *out) {
  __shared__ double red[32];
  double s = 0;
  for (int64_t p = threadIdx.x; p < P; p += blockDim.x) s += v[p] * v[p];
  s = block_sum(s, red);
  if (threadIdx.x == 0) *out = s;
}

// ---------------------------------------------------------------- SIMT Gram
constexpr int GT = 64, GK = 16;

__device__ inline void tri_tile(int64_t bid, int64_t &I, int64_t &J) {
  int64_t i = (int64_t)((sqrt(8.0 * (double)bid + 1.0) - 1.0) * 0.5);
  while (i * (i + 1) / 2 > bid) --i;
  while ((i + 1) * (i + 2) / 2 <= bid) ++i;
  I = i;
  J = bid - i * (i + 1) / 2;
}

template <typename T>
__global__ void __launch_bounds__(256) gram_simt_kernel(
    const T *__restrict__ t, const uint32_t *__restrict__ bits, int words, int N, int M, int64_t n,
    const double *__restrict__ g, const double *__restrict__ cptr, double inv_n,
    double diag_shift, double *__restrict__ T64, float *__restrict__ T32) {
  __shared__ T ta[GK][GT];
  __shared__ T tb[GK][GT];
  __shared__ uint32_t ba[GT][9];
  __shared__ uint32_t bb[GT][9];
  int64_t I, J;
  tri_tile(blockIdx.x, I, J);
  const int64_t r0 = I * GT, c0 = J * GT;
  const int tid = threadIdx.x, tr = tid >> 4, tc = tid & 15;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0;
  for (int k0 = 0; k0 < M; k0 += GK) {
    for (int e = tid; e < GT * GK; e += 256) {
      int r = e / GK, k = e % GK;
      int64_t ra = r0 + r, rb = c0 + r;
      int kk = k0 + k;
      ta[k][r] = (ra < n && kk < M) ? t[ra * M + kk] : T(0);
      tb[k][r] = (rb < n && kk < M) ? t[rb * M + kk] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < GK; ++k) {
      T a4[4], b4[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a4[i] = ta[k][tr * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b4[j] = tb[k][tc * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += a4[i] * b4[j];
    }
    __syncthreads();
  }
  for (int e = tid; e < GT * words; e += 256) {
    int r = e / words, w = e % words;
    ba[r][w] = (r0 + r < n) ? bits[(r0 + r) * words + w] : 0u;
    bb[r][w] = (c0 + r < n) ? bits[(c0 + r) * words + w] : 0u;
  }
  __syncthreads();
  const double c = *cptr;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t s = r0 + tr * 4 + i;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t sp = c0 + tc * 4 + j;
      if (s < n && sp <= s) {
        int diff = 0;
        for (int w = 0; w < words; ++w) diff += __popc(ba[tr * 4 + i][w] ^ bb[tc * 4 + j][w]);
        const double B = (double)(N - 2 * diff);
        const double A = (double)acc[i][j];
        double v = (A * (1.0 + B) + B - g[s] - g[sp] + c) * inv_n;
        if (s == sp) v += diag_shift;
        T64[s * n + sp] = v;
        if (T32) T32[s * n + sp] = (float)v;
      }
    }
  }
}

}  // namespace vmck

using namespace vmck;

static int64_t gram_words(int N) { return (N + 31) / 32; }

extern "C" int64_t vmck_gram_workspace_size(int32_t N, int32_t M, int64_t n) {
  (void)M;
  int64_t words = gram_words(N);
  return n /*g*/ + 2 /*c*/ + (n * words + 1) / 2 /*bits*/ + vmck::gram_tc_workspace_doubles(M, n) + 8;
}

extern "C" int vmck_rbm_gram(vmck_ctx *ctx, vmck_stream s, int32_t mode, int32_t dtype,
                             const void *tanh_theta, const int8_t *x, int32_t N, int32_t M,
                             int64_t n, const double *obar, double diag_shift, double *T64,
                             float *T32, double *workspace, int64_t workspace_len) {
  VMCK_REQUIRE(tanh_theta && x && obar && T64 && workspace && N > 0 && M > 0 && n > 0,
               "rbm_gram arguments");
  VMCK_REQUIRE(N <= 288, "rbm_gram supports N <= 288");
  VMCK_REQUIRE(workspace_len >= vmck_gram_workspace_size(N, M, n), "rbm_gram workspace too small");
  VMCK_REQUIRE((mode == 0 && dtype == VMCK_F64) || (mode == 1 && dtype == VMCK_F32) ||
                   (mode == 2 && dtype == VMCK_F32),
               "rbm_gram: mode/dtype combination (0:F64, 1:F32, 2:F32 tanh input)");
  cudaStream_t st = as_stream(s);
  const int words = (int)gram_words(N);
  double *g = workspace;
  double *cptr = workspace + n;
  uint32_t *bits = reinterpret_cast<uint32_t *>(workspace + n + 2);
  double *tc_ws = workspace + n + 2 + (n * words + 1) / 2;
  const int64_t P = (int64_t)M + (int64_t)N * M + N;
  sign_bits_kernel<<<ceil_div(n * words, 256), 256, 0, st>>>(x, n, N, words, bits);
  int rc = check_launch("gram sign bits");
  if (rc) return rc;
  const unsigned gblocks = (unsigned)((n + 15) / 16);
  if (dtype == VMCK_F64)
    g_vector_kernel<double><<<gblocks, 256, 0, st>>>(static_cast<const double *>(tanh_theta), x, N,
                                                     M, n, obar, g);
  else
    g_vector_kernel<float><<<gblocks, 256, 0, st>>>(static_cast<const float *>(tanh_theta), x, N,
                                                    M, n, obar, g);
  rc = check_launch("gram g vector");
  if (rc) return rc;
  sumsq_kernel<<<1, 1024, 0, st>>>(obar, P, cptr);
  rc = check_launch("gram |obar|^2");
  if (rc) return rc;
  const double inv_n = 1.0 / (double)n;
  if (mode == 2)
    return gram_tc_launch(ctx, st, static_cast<const float *>(tanh_theta), bits, words, N, M, n, g,
                          cptr, inv_n, diag_shift, T64, T32, tc_ws);
  const int64_t nt = (n + GT - 1) / GT;
  const int64_t tiles = nt * (nt + 1) / 2;
  VMCK_REQUIRE(tiles < (1ll << 31), "too many tiles");
  if (dtype == VMCK_F64)
    gram_simt_kernel<double><<<(unsigned)tiles, 256, 0, st>>>(
        static_cast<const double *>(tanh_theta), bits, words, N, M, n, g, cptr, inv_n, diag_shift,
        T64, T32);
  else
    gram_simt_kernel<float><<<(unsigned)tiles, 256, 0, st>>>(
        static_cast<const float *>(tanh_theta), bits, words, N, M, n, g, cptr, inv_n, diag_shift,
        T64, T32);
  return check_launch("gram simt");
}

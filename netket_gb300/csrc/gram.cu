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

#include <cuda_bf16.h>

#include "common.cuh"
#include "chol_tc.cuh"
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

// Double-float form for FP32 tanh(theta): the ~6.5e8 accumulations per call
// would otherwise run on the FP64 pipe.  t enters as c + s0 (the shifted,
// rounded values of gram_shift_kernel plus the shift), exactly as the
// contraction sees it; obar_df holds (hi, lo) pairs of obar.
__global__ void __launch_bounds__(256) g_vector_df_kernel(const float *__restrict__ c,
                                                          const float *__restrict__ s0,
                                                          const int8_t *__restrict__ x, int N,
                                                          int M, int64_t n,
                                                          const float2 *__restrict__ obar_df,
                                                          const double *__restrict__ obar,
                                                          double *__restrict__ g) {
  __shared__ int8_t xs[G_SPB][G_NMAX];
  __shared__ double part[G_SPB][8];
  const int64_t s0i = (int64_t)blockIdx.x * G_SPB;
  const float2 *Kbar = obar_df + M;
  const double *xbar = obar + M + (int64_t)N * M;
  const int ns = (int)std::min<int64_t>(G_SPB, n - s0i);
  for (int e = threadIdx.x; e < G_SPB * N; e += blockDim.x) {
    int q = e / N, i = e % N;
    xs[q][i] = (q < ns) ? x[(s0i + q) * N + i] : int8_t(0);
  }
  __syncthreads();
  df32 gp[G_SPB];
#pragma unroll
  for (int q = 0; q < G_SPB; ++q) gp[q] = {0.0f, 0.0f};
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    df32 y[G_SPB];
    const float2 tb = obar_df[j];
    const float sj = s0[j];
#pragma unroll
    for (int q = 0; q < G_SPB; ++q) y[q] = {tb.x, tb.y};
    for (int i = 0; i < N; ++i) {
      const float2 kb = Kbar[(int64_t)i * M + j];
      const df32 kp = {kb.x, kb.y}, km = {-kb.x, -kb.y};
#pragma unroll
      for (int q = 0; q < G_SPB; ++q) y[q] = df_add(y[q], xs[q][i] > 0 ? kp : km);
    }
#pragma unroll
    for (int q = 0; q < G_SPB; ++q)
      if (q < ns) gp[q] = df_add(gp[q], df_mul(y[q], df_two_sum(c[(s0i + q) * M + j], sj)));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < G_SPB; ++q) {
    double v = warp_sum(df_to_double(gp[q]));
    if (lane == 0) part[q][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < ns) {
    const int q = threadIdx.x;
    double v = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += part[q][w];
    for (int i = 0; i < N; ++i) v += xs[q][i] > 0 ? xbar[i] : -xbar[i];
    g[s0i + q] = v;
  }
}

// Shift of the FP32 contraction: s0 = fp32(mean of t) from obar, and
// c = round(t - s0) with terms = 0 (FP32), 1 (one BF16), 2 (hi + lo BF16) or
// 3 (a multiple of 2^-19, the fixed-point grid of mode 4's split); c is exactly
// what the contraction multiplies.  A = t t^T is then
// c c^T + w 1^T + 1 w^T + |s0|^2 with w_s = c_s . s0, and only c c^T is
// accumulated in FP32 -- its entries are small where hidden units are biased,
// which keeps the centred T free of catastrophic cancellation.
__global__ void gram_shift_kernel(const float *__restrict__ t, const double *__restrict__ obar,
                                  int64_t n, int M, int terms, float *__restrict__ c,
                                  float *__restrict__ s0) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e < M) s0[e] = __double2float_rn(obar[e]);
  if (e >= n * M) return;
  const int j = (int)(e % M);
  const float v = __fsub_rn(t[e], __double2float_rn(obar[j]));
  if (terms == 0) {
    c[e] = v;
  } else if (terms == 3) {
    c[e] = rintf(v * 524288.0f) * (1.0f / 524288.0f);  // |v| < 2: exact scalings
  } else {
    const float hi = __bfloat162float(__float2bfloat16(v));
    c[e] = (terms == 1) ? hi : __fadd_rn(hi, __bfloat162float(__float2bfloat16(__fsub_rn(v, hi))));
  }
}

// w_s = c_s . s0 (one warp per sample, FP64) and |s0|^2, as double-float pairs
__global__ void gram_shift_dot_kernel(const float *__restrict__ c, const float *__restrict__ s0,
                                      int64_t n, int M, float2 *__restrict__ w,
                                      float2 *__restrict__ s0sq) {
  const int64_t s = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (s < n) {
    double acc = 0.0;
    for (int j = lane; j < M; j += 32) acc += (double)c[s * M + j] * (double)s0[j];
    acc = warp_sum(acc);
    if (lane == 0) {
      const df32 d = df_from(acc);
      w[s] = make_float2(d.hi, d.lo);
    }
  }
  if (blockIdx.x == 0 && (threadIdx.x >> 5) == 0) {
    double q = 0.0;
    for (int j = lane; j < M; j += 32) q += (double)s0[j] * (double)s0[j];
    q = warp_sum(q);
    if (lane == 0) {
      const df32 d = df_from(q);
      *s0sq = make_float2(d.hi, d.lo);
    }
  }
}

__global__ void to_df_kernel(const double *__restrict__ v, int64_t P, float2 *__restrict__ out) {
  int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= P) return;
  const df32 d = df_from(v[p]);
  out[p] = make_float2(d.hi, d.lo);
}

__global__ void sumsq_kernel(const double *__restrict__ v, int64_t P, double *out) {
  __shared__ double red[32];
  double s = 0;
  for (int64_t p = threadIdx.x; p < P; p += blockDim.x) s += v[p] * v[p];
  s = block_sum(s, red);
  if (threadIdx.x == 0) *out = s;
}

// h_s = g_s - c / 2 as a double-float pair, so that T = (G - h_s - h_s') / n
__global__ void h_df_kernel(const double *__restrict__ g, const double *__restrict__ cptr,
                            int64_t n, float2 *__restrict__ h) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const df32 d = df_from(g[s] - 0.5 * (*cptr));
  h[s] = make_float2(d.hi, d.lo);
}

// Gram epilogue value in double-float arithmetic: Ac = c_s.c_s' from the FP32
// contraction, the shift terms w, |s0|^2, B = x.x' exact, h = g - |obar|^2 / 2.
// Returns (((Ac + w_s + w_s' + |s0|^2)(1 + B) + B) - h_s - h_s') / n (+ shift).
__device__ __forceinline__ df32 gram_value_df(float Ac, float2 ws, float2 wc, df32 s0sq, int B,
                                              float2 hs, float2 hc, float inv_n, bool diag,
                                              df32 shift) {
  df32 a = df_add(df32{ws.x, ws.y}, df32{wc.x, wc.y});
  a = df_add(a, s0sq);
  a = df_add(a, Ac);
  df32 v = df_mul(a, (float)(1 + B));
  v = df_add(v, (float)B);
  v = df_add(v, df32{-hs.x, -hs.y});
  v = df_add(v, df32{-hc.x, -hc.y});
  v = df_mul(v, inv_n);
  if (diag) v = df_add(v, shift);
  return v;
}

// ---------------------------------------------------------------- fixed-point split (mode 4)
// c (|c| < 2) -> hi + lo with u = c 2^8: hi = rint(u), an integer of at most
// 512 in magnitude, and lo = rint((u - hi) 2^11) 2^-11, so c = (hi + lo) 2^-8 to
// 2^-20 (exactly: the shift kernel has put c on the 2^-19 grid, so that the
// shift terms w and g see the same c as the contraction).  Both are exact in FP16.  Every hi * hi product is an integer below
// 2^18 and a 64-wide slab of them sums to an integer of at most 2^24: the
// tensor core forms each slab's large part exactly, whatever its rounding, and
// the only rounding of it is the round-to-nearest FP32 sum over slabs in
// registers.  (A floating split leaves the tensor core's truncating alignment
// in the slab sums, an error of ~2^-22 of the sum that is biased toward zero;
// amplified by T's centring it pushed the smallest eigenvalue of T below
// diag_shift 1e-4 at n = 65,536, M = 2048.)  The scale 2^8 goes to *scale.
__global__ void gram_split_fixed_kernel(const float *__restrict__ c, int64_t n, int M, int ldk,
                                        __half *__restrict__ hi, __half *__restrict__ lo,
                                        float *scale) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e == 0) *scale = 256.0f;
  if (e >= n * ldk) return;
  const int64_t r = e / ldk;
  const int k = (int)(e - r * ldk);
  float h = 0.0f, l = 0.0f;
  if (k < M) {
    const float u = c[r * M + k] * 256.0f;  // exact: a power-of-two scaling
    h = rintf(u);
    l = rintf((u - h) * 2048.0f) * (1.0f / 2048.0f);  // u - h is exact (Sterbenz)
  }
  hi[e] = __float2half_rn(h);
  lo[e] = __float2half_rn(l);
}

// ---------------------------------------------------------------- assembly (mode 4)
// T from Ac = c c^T (FP32, already in T32's lower triangle, written by the
// tensor-core GEMM): the same double-float epilogue as the SIMT Gram.  Block
// (x, y) covers columns [256 x, +256) of rows [64 y, +64), lower triangle only;
// a thread keeps its column's sign bits and pairs in registers, the row's are
// warp-uniform loads.
constexpr int GA_ROWS = 64;
__global__ void __launch_bounds__(256) gram_assemble_kernel(
    const uint32_t *__restrict__ bits, int words, int N, int64_t n,
    const float2 *__restrict__ hdf, const float2 *__restrict__ wdf,
    const float2 *__restrict__ s0sq_p, float inv_n, df32 shift, double *__restrict__ T64,
    float *__restrict__ T32) {
  const int64_t c0 = (int64_t)blockIdx.x * 256;
  const int64_t r0 = (int64_t)blockIdx.y * GA_ROWS;
  const int64_t r1 = r0 + GA_ROWS < n ? r0 + GA_ROWS : n;
  if (r1 <= c0) return;  // the whole block lies above the diagonal
  const int64_t c = c0 + threadIdx.x;
  if (c >= n) return;
  uint32_t cb[9];
#pragma unroll
  for (int w = 0; w < 9; ++w) cb[w] = w < words ? bits[c * words + w] : 0u;
  const float2 wc = wdf[c], hc = hdf[c], q = *s0sq_p;
  for (int64_t r = r0 > c ? r0 : c; r < r1; ++r) {
    int diff = 0;
#pragma unroll
    for (int w = 0; w < 9; ++w)
      if (w < words) diff += __popc(cb[w] ^ __ldg(bits + r * words + w));
    const int64_t e = r * n + c;
    const df32 v = gram_value_df(T32[e], wdf[r], wc, df32{q.x, q.y}, N - 2 * diff, hdf[r], hc,
                                 inv_n, r == c, shift);
    T32[e] = v.hi + v.lo;
    if (T64) T64[e] = df_to_double(v);
  }
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
    const double *__restrict__ g, const double *__restrict__ cptr, const float2 *__restrict__ hdf,
    const float2 *__restrict__ wdf, const float2 *__restrict__ s0sq_p, double inv_n,
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
  const df32 shift_df = {(float)diag_shift, (float)(diag_shift - (double)(float)diag_shift)};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t s = r0 + tr * 4 + i;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t sp = c0 + tc * 4 + j;
      if (s < n && sp <= s) {
        int diff = 0;
        for (int w = 0; w < words; ++w) diff += __popc(ba[tr * 4 + i][w] ^ bb[tc * 4 + j][w]);
        const int B = N - 2 * diff;
        if (sizeof(T) == 8) {
          const double A = (double)acc[i][j];
          double v = (A * (1.0 + B) + B - g[s] - g[sp] + c) * inv_n;
          if (s == sp) v += diag_shift;
          if (T64) T64[s * n + sp] = v;
          if (T32) T32[s * n + sp] = (float)v;
        } else {
          const float2 q = *s0sq_p;
          const df32 v = gram_value_df((float)acc[i][j], wdf[s], wdf[sp], df32{q.x, q.y}, B,
                                       hdf[s], hdf[sp], (float)inv_n, s == sp, shift_df);
          if (T64) T64[s * n + sp] = df_to_double(v);
          if (T32) T32[s * n + sp] = v.hi + v.lo;
        }
      }
    }
  }
}

}  // namespace vmck

using namespace vmck;

static int64_t gram_words(int N) { return (N + 31) / 32; }

struct GramWs {
  double *g, *cptr;
  uint32_t *bits;
  float2 *obar_df, *hdf, *wdf, *s0sq;
  float *c, *s0;
  double *tc;
};

static GramWs gram_ws_layout(double *ws, int N, int M, int64_t n) {
  const int64_t words = gram_words(N);
  const int64_t P = (int64_t)M + (int64_t)N * M + N;
  GramWs w;
  w.g = ws;
  w.cptr = ws + n;
  w.bits = reinterpret_cast<uint32_t *>(ws + n + 2);
  double *p = ws + n + 2 + (n * words + 1) / 2;
  w.obar_df = reinterpret_cast<float2 *>(p);
  p += P;
  w.hdf = reinterpret_cast<float2 *>(p);
  p += n;
  w.wdf = reinterpret_cast<float2 *>(p);
  p += n;
  w.s0sq = reinterpret_cast<float2 *>(p);
  p += 2;
  w.s0 = reinterpret_cast<float *>(p);
  p += (M + 1) / 2 + 2;
  w.c = reinterpret_cast<float *>(p);
  p += (n * (int64_t)M + 1) / 2 + 2;
  w.tc = p;
  return w;
}

extern "C" int64_t vmck_gram_workspace_size(int32_t N, int32_t M, int64_t n) {
  const int64_t words = gram_words(N);
  const int64_t P = (int64_t)M + (int64_t)N * M + N;
  // the tail: the tensor-core Gram's panels, or the split rows of mode 4
  const int64_t split = ((n * ((M + 7) & ~7) + 511) & ~int64_t(511)) * 2 * 2 / 8 + (1024 + 16) / 8;
  return n + 2 + (n * words + 1) / 2 + P + n + n + 2 + (M + 1) / 2 + 2 + (n * (int64_t)M + 1) / 2 +
         2 + std::max(vmck::gram_tc_workspace_doubles(M, n), split) + 8;
}

extern "C" int vmck_rbm_gram(vmck_ctx *ctx, vmck_stream s, int32_t mode, int32_t dtype,
                             const void *tanh_theta, const int8_t *x, int32_t N, int32_t M,
                             int64_t n, const double *obar, double diag_shift, double *T64,
                             float *T32, double *workspace, int64_t workspace_len,
                             int32_t *status) {
  VMCK_REQUIRE(tanh_theta && x && obar && (T64 || T32) && workspace && N > 0 && M > 0 && n > 0,
               "rbm_gram arguments");
  VMCK_REQUIRE(N <= 288, "rbm_gram supports N <= 288");
  VMCK_REQUIRE(workspace_len >= vmck_gram_workspace_size(N, M, n), "rbm_gram workspace too small");
  VMCK_REQUIRE((mode == 0 && dtype == VMCK_F64) || (mode >= 1 && mode <= 4 && dtype == VMCK_F32),
               "rbm_gram: mode/dtype combination (0: F64, 1-4: F32 tanh input)");
  VMCK_REQUIRE(mode < 2 || T32, "rbm_gram: tensor-core modes write T32");
  cudaStream_t st = as_stream(s);
  const int words = (int)gram_words(N);
  GramWs w = gram_ws_layout(workspace, N, M, n);
  const int64_t P = (int64_t)M + (int64_t)N * M + N;
  sign_bits_kernel<<<ceil_div(n * words, 256), 256, 0, st>>>(x, n, N, words, w.bits);
  int rc = check_launch("gram sign bits");
  if (rc) return rc;
  const unsigned gblocks = (unsigned)((n + G_SPB - 1) / G_SPB);
  if (dtype == VMCK_F64) {
    g_vector_kernel<double><<<gblocks, 256, 0, st>>>(static_cast<const double *>(tanh_theta), x,
                                                     N, M, n, obar, w.g);
  } else {
    const int terms = mode == 2 ? 2 : (mode == 3 ? 1 : (mode == 4 ? 3 : 0));
    gram_shift_kernel<<<ceil_div(n * (int64_t)M, 256), 256, 0, st>>>(
        static_cast<const float *>(tanh_theta), obar, n, M, terms, w.c, w.s0);
    if ((rc = check_launch("gram shift"))) return rc;
    gram_shift_dot_kernel<<<ceil_div(n, 8), 256, 0, st>>>(w.c, w.s0, n, M, w.wdf, w.s0sq);
    if ((rc = check_launch("gram shift dot"))) return rc;
    to_df_kernel<<<ceil_div(P, 256), 256, 0, st>>>(obar, P, w.obar_df);
    if ((rc = check_launch("gram obar pairs"))) return rc;
    g_vector_df_kernel<<<gblocks, 256, 0, st>>>(w.c, w.s0, x, N, M, n, w.obar_df, obar, w.g);
  }
  if ((rc = check_launch("gram g vector"))) return rc;
  sumsq_kernel<<<1, 1024, 0, st>>>(obar, P, w.cptr);
  if ((rc = check_launch("gram |obar|^2"))) return rc;
  h_df_kernel<<<ceil_div(n, 256), 256, 0, st>>>(w.g, w.cptr, n, w.hdf);
  if ((rc = check_launch("gram h pairs"))) return rc;
  const double inv_n = 1.0 / (double)n;
  if (mode == 4) {
    VMCK_REQUIRE(n < (int64_t)INT32_MAX && (n + GA_ROWS - 1) / GA_ROWS <= 65535,
                 "rbm_gram mode 4: too many samples");
    // c c^T on the tensor cores: c = t - s0 (|c| < 2) split into fixed-point
    // FP16 hi / lo, the triangular split GEMM (all four products: the Gram
    // matrix of hi + lo) into T32, then the double-float assembly
    const int ldk = (M + 7) & ~7;
    __half *hi = reinterpret_cast<__half *>(
        (reinterpret_cast<uintptr_t>(w.tc) + 1023) & ~uintptr_t(1023));
    __half *lo = hi + ((n * ldk + 511) & ~int64_t(511));
    float *scale = reinterpret_cast<float *>(lo + ((n * ldk + 511) & ~int64_t(511)));
    gram_split_fixed_kernel<<<ceil_div(n * ldk, 256), 256, 0, st>>>(w.c, n, M, ldk, hi, lo,
                                                                     scale);
    if ((rc = check_launch("gram split"))) return rc;
    const SplitOperand op{hi, lo, ldk, M, n};
    if ((rc = tc_gemm(st, op, 0, op, 0, 0, (int)n, (int)n, M, T32, n, 1.0f, 0.0f, scale, scale,
                      1, nullptr, nullptr, 0, 0, 0, nullptr, status, 0, 1)))
      return rc;
    const df32 shift = {(float)diag_shift, (float)(diag_shift - (double)(float)diag_shift)};
    gram_assemble_kernel<<<dim3((unsigned)((n + 255) / 256),
                                (unsigned)((n + GA_ROWS - 1) / GA_ROWS)),
                           256, 0, st>>>(w.bits, words, N, n, w.hdf, w.wdf, w.s0sq,
                                         (float)inv_n, shift, T64, T32);
    return check_launch("gram assemble");
  }
  if (mode >= 2)
    return gram_tc_launch(ctx, st, w.c, w.bits, words, N, M, n, w.hdf, w.wdf, w.s0sq, inv_n,
                          diag_shift, T64, T32, w.tc, mode == 2 ? 1 : 0, status);
  const int64_t nt = (n + GT - 1) / GT;
  const int64_t tiles = nt * (nt + 1) / 2;
  VMCK_REQUIRE(tiles < (1ll << 31), "too many tiles");
  if (dtype == VMCK_F64)
    gram_simt_kernel<double><<<(unsigned)tiles, 256, 0, st>>>(
        static_cast<const double *>(tanh_theta), w.bits, words, N, M, n, w.g, w.cptr, w.hdf,
        w.wdf, w.s0sq, inv_n, diag_shift, T64, T32);
  else
    gram_simt_kernel<float><<<(unsigned)tiles, 256, 0, st>>>(
        w.c, w.bits, words, N, M, n, w.g, w.cptr, w.hdf, w.wdf, w.s0sq, inv_n, diag_shift, T64,
        T32);
  return check_launch("gram simt");
}

// Shared device helpers for libvmck: status handling, Philox4x32-10,
// log_cosh, warp/block reductions.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "../../include/vmck.h"

namespace vmck {

// ----------------------------------------------------------------- host status
void set_last_error(const char *fmt, ...);

void count_launch();

// Wall-time limit (ns) of the device-side waits for work (vmck_set_wait_limit_ns).
unsigned long long wait_limit_ns();

// Every kernel launch of the library is followed by check_launch, which also
// counts it (vmck_launch_count).
inline int check_launch(const char *what) {
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error("%s: %s", what, cudaGetErrorString(e));
    return VMCK_ERR_CUDA;
  }
  return VMCK_OK;
}

#define VMCK_CUDA(call)                                                        \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      ::vmck::set_last_error("%s:%d %s: %s", __FILE__, __LINE__, #call,        \
                             cudaGetErrorString(e_));                          \
      return VMCK_ERR_CUDA;                                                    \
    }                                                                          \
  } while (0)

#define VMCK_REQUIRE(cond, msg)                                                \
  do {                                                                         \
    if (!(cond)) {                                                             \
      ::vmck::set_last_error("argument check failed: %s", msg);                \
      return VMCK_ERR_ARG;                                                     \
    }                                                                          \
  } while (0)

inline cudaStream_t as_stream(vmck_stream s) { return reinterpret_cast<cudaStream_t>(s); }

inline int ceil_div(int64_t a, int64_t b) { return static_cast<int>((a + b - 1) / b); }

// ----------------------------------------------------------------- Philox4x32-10
// Counter-based generator of Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3" (SC'11): ten rounds of two 32x32->64 multiplies
// with the paper's multipliers and Weyl key increments.
struct u32x4 {
  uint32_t x, y, z, w;
};

__device__ __forceinline__ u32x4 philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = u32x4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// uniform in [0, 1) with 24 random bits
__device__ __forceinline__ float u01f(uint32_t v) { return (v >> 8) * (1.0f / 16777216.0f); }
// uniform in [0, 1) with 53 random bits
__device__ __forceinline__ double u01d(uint32_t a, uint32_t b) {
  uint64_t v = (static_cast<uint64_t>(a) << 21) ^ static_cast<uint64_t>(b >> 11);
  return static_cast<double>(v & ((1ull << 53) - 1)) * (1.0 / 9007199254740992.0);
}
// integer in [0, n) by multiply-shift
__device__ __forceinline__ uint32_t below(uint32_t v, uint32_t n) { return __umulhi(v, n); }

// ----------------------------------------------------------------- log_cosh
// log(cosh(x)) = |x| + log1p(exp(-2|x|)) - log(2), the stable form of
// netket/nn/activation.py:78-84.
__device__ __forceinline__ double log_cosh(double x) {
  x = fabs(x);
  return x + log1p(exp(-2.0 * x)) - 0.69314718055994530942;
}
__device__ __forceinline__ float log_cosh(float x) {
  x = fabsf(x);
  return x + log1pf(expf(-2.0f * x)) - 0.693147180559945309f;
}
// Same formula with one special-function op: e = exp(-2|x|) on the MUFU unit
// (__expf), log1p(e) for e in (0, 1] as a degree-9 polynomial in e on the FMA
// pipe (a Chebyshev fit of log1p on [0, 1] made for this library, converted to
// the monomial basis; error 5e-9 in exact arithmetic, ~1e-7 after FP32 Horner
// rounding).  The sampler and local-energy kernels evaluate hundreds of
// log_cosh per proposal / connected element, and the MUFU unit (a quarter of
// the FMA rate) bounds them.  Absolute error of the result ~5e-7 at |x| ~ 20
// (half an ulp of the result), ~1e-7 for |x| < 4; used by the FP32 paths,
// whose results carry a 1e-4 relative bound.
__device__ __forceinline__ float log_cosh_fast(float x) {
  x = fabsf(x);
  const float e = __expf(-2.0f * x);
  float p = 0.003752624150365591f;
  p = __fmaf_rn(p, e, -0.02303827926516533f);
  p = __fmaf_rn(p, e, 0.06651248037815094f);
  p = __fmaf_rn(p, e, -0.12526661157608032f);
  p = __fmaf_rn(p, e, 0.1846884787082672f);
  p = __fmaf_rn(p, e, -0.24635660648345947f);
  p = __fmaf_rn(p, e, 0.3328184187412262f);
  p = __fmaf_rn(p, e, -0.4999622404575348f);
  p = __fmaf_rn(p, e, 0.999998927116394f);
  p = __fmaf_rn(p, e, 5.239402245393876e-09f);
  return x + p - 0.693147180559945309f;
}
__device__ __forceinline__ double log_cosh_fast(double x) { return log_cosh(x); }

// exp of a log-amplitude ratio in a local-energy sum: in FP32 (one accurate
// expf) when the ratio cannot overflow, else in double.  GB300's FP64 pipe is
// narrow enough that a double exp per connected element dominated the FP32
// local-energy kernels.
__device__ __forceinline__ double exp_ratio(float x) {
  return x < 80.0f ? (double)expf(x) : exp((double)x);
}
__device__ __forceinline__ double exp_ratio(double x) { return exp(x); }

// ----------------------------------------------------------------- double-float
// Pairs (hi, lo) of FP32 values carrying ~48 significant bits, with the
// error-free transformations of Knuth (TwoSum) and Dekker (TwoProduct via FMA).
// Used where GB300's FP64 pipe would be the bottleneck (it issues roughly two
// FP64 FMAs per clock per SM) but FP32 accuracy is not enough.
struct df32 {
  float hi, lo;
};
__device__ __forceinline__ df32 df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ df32 df_quick_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df32 df_two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ df32 df_add(df32 a, df32 b) {
  const df32 s = df_two_sum(a.hi, b.hi);
  return df_quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df32 df_add(df32 a, float b) {
  const df32 s = df_two_sum(a.hi, b);
  return df_quick_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}
__device__ __forceinline__ df32 df_neg(df32 a) { return {-a.hi, -a.lo}; }
// a * b for a float b (error of the lo * b product is below the pair's precision)
__device__ __forceinline__ df32 df_mul(df32 a, float b) {
  const df32 p = df_two_prod(a.hi, b);
  return df_quick_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}
__device__ __forceinline__ df32 df_mul(df32 a, df32 b) {
  const df32 p = df_two_prod(a.hi, b.hi);
  return df_quick_two_sum(p.hi, __fadd_rn(p.lo, __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi))));
}
__device__ __forceinline__ df32 df_from(double d) {
  const float h = __double2float_rn(d);
  return {h, __double2float_rn(d - (double)h)};
}
// (double)(hi + lo) assembled from the bit fields with integer operations: for a
// normalised pair (|lo| <= ulp(hi) / 2) lo lands in the 29 low mantissa bits a
// double has below hi's, so the result is exact (a subtraction that borrows
// from hi's leading bit renormalises by one place).  GB300 issues roughly one
// FP64 instruction per clock per SM, so two conversions and an add per element
// would bound the Gram epilogues; zero / subnormal / non-finite hi and
// non-normalised pairs take the FP64 route.
__device__ __forceinline__ double df_to_double(df32 a) {
  const uint32_t hb = __float_as_uint(a.hi), lb = __float_as_uint(a.lo);
  const int he = (int)((hb >> 23) & 0xFFu), le = (int)((lb >> 23) & 0xFFu);
  const int sh = (le > 0 ? le : 1) - he + 29;  // lo in units of hi's last double bit
  if (he == 0 || he == 0xFF || le == 0xFF || sh > 5) return (double)a.hi + (double)a.lo;
  long long X = (long long)((hb & 0x7FFFFFu) | 0x800000u) << 29;
  const unsigned long long ml = (lb & 0x7FFFFFu) | (le ? 0x800000u : 0u);
  const long long li = (long long)(sh >= 0 ? (ml << sh) : (sh > -40 ? (ml >> -sh) : 0ull));
  X = ((hb ^ lb) >> 31) ? X - li : X + li;
  int e = he - 127 + 1023;
  if (X < (1ll << 52)) {
    X <<= 1;
    --e;
  }
  return __longlong_as_double((long long)(((unsigned long long)(hb >> 31) << 63) |
                                          ((unsigned long long)e << 52) |
                                          ((unsigned long long)X & ((1ull << 52) - 1))));
}

// ----------------------------------------------------------------- reductions
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum; every thread receives the result.  `red` must hold
// blockDim.x/32 elements of T.  Deterministic (fixed tree).
template <typename T>
__device__ __forceinline__ T block_sum(T v, T *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  T t = (lane < nw) ? red[lane] : T(0);
  t = warp_sum(t);
  return t;
}

template <typename T>
struct Real;
template <>
struct Real<double> {
  static constexpr int code = VMCK_F64;
};
template <>
struct Real<float> {
  static constexpr int code = VMCK_F32;
};

}  // namespace vmck

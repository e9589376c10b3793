// The RBM's dense contractions on the tensor cores (FP32 parameters):
//
//   theta = x W + b        (RBM.__call__'s nn.Dense, netket/models/rbm.py:58-60)
//   O^T v                  (the VJP of expect_forces.py:98-104 and O_L^T aux of
//                           _src/ngd/srt.py:83-84 for the RBM Jacobian
//                           O(s) = [t_s, x_s (x) t_s, x_s], t = tanh theta)
//
// Both run tc_gemm_kernel (chol_tc.cu: tcgen05 kind::f16 on operands split into
// FP16 hi + lo, 22 significant bits, FP32 accumulation drained from tensor
// memory every 64-wide K slab).  The spins x_s = +-1 are exact in FP16 (lo = 0).
//
// theta: A_op = W^T split (M rows, K = N), B_op = x (n rows), C = x W (n x M
// row-major); one epilogue pass adds b, writes theta / tanh theta and the row
// sums of log_cosh theta + a.x.
//
// O^T v: A_op = v (.) [t, 1] split (M + 1 rows, K = n samples), B_op = [x, 1]
// (N + 1 rows); C[j + i (M + 1)] = sum_s v_s t_sj x_si holds the kernel part
// (i < N, j < M), the hidden bias part (i = N) and the visible bias part
// (j = M) at once.  K = n is long, so it is split into kz chunks (partial C per
// chunk, summed in FP64 in a fixed order by the scatter kernel).
#include <algorithm>

#include <cuda_fp16.h>

#include "chol_tc.cuh"
#include "common.cuh"

namespace vmck {

namespace {

constexpr int64_t align_up(int64_t v, int64_t a) { return (v + a - 1) / a * a; }

struct LogpsiTcWs {
  __half *wt_hi, *wt_lo, *x_hi, *x_lo;
  float *theta, *scale;
  int64_t bytes;
};

// Workspace layout of the theta GEMM (bytes; theta only when the caller has no
// theta buffer).
LogpsiTcWs logpsi_tc_layout(char *base, int N, int M, int64_t n, bool own_theta) {
  const int64_t np = align_up(N, 8);
  LogpsiTcWs w{};
  int64_t o = 0;
  auto take = [&](int64_t bytes) {
    const int64_t at = o;
    o = align_up(o + bytes, 1024);
    return base ? base + at : nullptr;
  };
  w.wt_hi = reinterpret_cast<__half *>(take((int64_t)M * np * 2));
  w.wt_lo = reinterpret_cast<__half *>(take((int64_t)M * np * 2));
  w.x_hi = reinterpret_cast<__half *>(take(n * np * 2));
  w.x_lo = reinterpret_cast<__half *>(take(n * np * 2));
  w.theta = reinterpret_cast<float *>(take(own_theta ? n * M * 4 : 0));
  w.scale = reinterpret_cast<float *>(take(16));
  w.bytes = o + 1024;
  return w;
}

struct OtvTcWs {
  __half *a_hi, *a_lo, *b_hi, *b_lo;
  float *part, *scale;
  int64_t ldk, kchunk;
  int kz;
  int64_t bytes;
};

// Split of K = n: about four waves of (M + 1) x (N + 1) output tiles over the
// SMs, chunks a multiple of the 64-wide slab.
void otv_split(int N, int M, int64_t n, int sms, int64_t &kchunk, int &kz) {
  const int64_t tiles = ((M + 1 + 127) / 128) * ((N + 1 + 255) / 256);
  int64_t want = std::max<int64_t>(1, (4 * (int64_t)sms + tiles - 1) / tiles);
  const int64_t slabs = (n + 63) / 64;
  want = std::min(want, slabs);
  kchunk = ((slabs + want - 1) / want) * 64;
  kz = (int)((n + kchunk - 1) / kchunk);
}

OtvTcWs otv_tc_layout(char *base, int N, int M, int64_t n, int sms) {
  OtvTcWs w{};
  w.ldk = align_up(n, 64);
  otv_split(N, M, n, sms, w.kchunk, w.kz);
  int64_t o = 0;
  auto take = [&](int64_t bytes) {
    const int64_t at = o;
    o = align_up(o + bytes, 1024);
    return base ? base + at : nullptr;
  };
  w.a_hi = reinterpret_cast<__half *>(take((int64_t)(M + 1) * w.ldk * 2));
  w.a_lo = reinterpret_cast<__half *>(take((int64_t)(M + 1) * w.ldk * 2));
  w.b_hi = reinterpret_cast<__half *>(take((int64_t)(N + 1) * w.ldk * 2));
  w.b_lo = reinterpret_cast<__half *>(take((int64_t)(N + 1) * w.ldk * 2));
  w.part = reinterpret_cast<float *>(take((int64_t)w.kz * (M + 1) * (N + 1) * 4));
  w.scale = reinterpret_cast<float *>(take(16));
  w.bytes = o + 1024;
  return w;
}

int device_sms() {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

}  // namespace

// scale[0] = split_scale(max |v|) over n values (FP32 or FP64 input).  One block.
template <typename T>
__global__ void __launch_bounds__(1024) abs_max_scale_kernel(const T *__restrict__ v, int64_t n,
                                                             float *scale) {
  __shared__ float red[32];
  float m = 0.0f;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, fabsf((float)v[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t = fmaxf(t, red[k]);
    scale[0] = split_scale(t);
  }
}

// wt_hi / lo[j np + i] = split(W[i M + j] s), zero for i in [N, np).
__global__ void split_wt_kernel(const float *__restrict__ W, int N, int M, int np,
                                const float *__restrict__ scale, __half *__restrict__ hi,
                                __half *__restrict__ lo) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)M * np) return;
  const int j = (int)(e / np), i = (int)(e - (int64_t)j * np);
  __half h = __float2half_rn(0.0f), l = h;
  if (i < N) split_f16(W[(int64_t)i * M + j], *scale, h, l);
  hi[e] = h;
  lo[e] = l;
}

// x_hi[s np + i] = x_si (exact), zero for i in [N, np); x_lo = 0.
__global__ void spins_f16_kernel(const int8_t *__restrict__ x, int64_t n, int N, int np,
                                 __half *__restrict__ hi, __half *__restrict__ lo) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= n * np) return;
  const int64_t s = e / np;
  const int i = (int)(e - s * np);
  hi[e] = __float2half_rn(i < N ? (float)x[s * N + i] : 0.0f);
  lo[e] = __float2half_rn(0.0f);
}

// theta += b; tanh; logpsi = sum_j log_cosh(theta_j) + a.x.  A warp per sample,
// lane-strided sums and a fixed shuffle tree.
__global__ void __launch_bounds__(256) logpsi_epilogue_kernel(
    const float *__restrict__ b, const float *__restrict__ a, const int8_t *__restrict__ x, int N,
    int M, int64_t n, float *__restrict__ acc, float *__restrict__ logpsi, bool keep_theta,
    float *__restrict__ tanh_out) {
  const int64_t s = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (s >= n) return;
  float *row = acc + s * M;
  float part = 0.0f;
  for (int j = lane; j < M; j += 32) {
    const float th = row[j] + b[j];
    part += log_cosh(th);
    if (keep_theta) row[j] = th;
    if (tanh_out) tanh_out[s * M + j] = tanhf(th);
  }
  float v = 0.0f;
  for (int i = lane; i < N; i += 32) v += (float)x[s * N + i] * a[i];
  part = warp_sum(part) + warp_sum(v);
  if (lane == 0) logpsi[s] = part;
}

// a_hi / lo[j ldk + s] = split(v_s t_sj s_v) (j < M), split(v_s s_v) (j = M);
// 0 for s >= n.  32 x 32 tiles through shared memory (coalesced both ways).
__global__ void __launch_bounds__(256) split_vt_transpose_kernel(
    const float *__restrict__ t, const double *__restrict__ v, int M, int64_t n, int64_t ldk,
    const float *__restrict__ scale, __half *__restrict__ hi, __half *__restrict__ lo) {
  __shared__ float tile[32][33];
  const int64_t s0 = (int64_t)blockIdx.x * 32;
  const int j0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int r = ty; r < 32; r += 8) {
    const int64_t s = s0 + r;
    const int j = j0 + tx;
    float val = 0.0f;
    if (s < n && j <= M) val = (float)v[s] * (j < M ? t[s * M + j] : 1.0f);
    tile[r][tx] = val;
  }
  __syncthreads();
  const float sc = *scale;
  for (int r = ty; r < 32; r += 8) {
    const int j = j0 + r;
    const int64_t s = s0 + tx;
    if (j <= M && s < ldk) {
      __half h, l;
      split_f16(tile[tx][r], sc, h, l);
      hi[(int64_t)j * ldk + s] = h;
      lo[(int64_t)j * ldk + s] = l;
    }
  }
}

// b_hi[i ldk + s] = x_si (i < N), 1 (i = N); 0 for s >= n; b_lo = 0.
__global__ void __launch_bounds__(256) spins_transpose_kernel(const int8_t *__restrict__ x,
                                                              int N, int64_t n, int64_t ldk,
                                                              __half *__restrict__ hi,
                                                              __half *__restrict__ lo) {
  __shared__ float tile[32][33];
  const int64_t s0 = (int64_t)blockIdx.x * 32;
  const int i0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int r = ty; r < 32; r += 8) {
    const int64_t s = s0 + r;
    const int i = i0 + tx;
    float val = 0.0f;
    if (s < n && i <= N) val = i < N ? (float)x[s * N + i] : 1.0f;
    tile[r][tx] = val;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + r;
    const int64_t s = s0 + tx;
    if (i <= N && s < ldk) {
      hi[(int64_t)i * ldk + s] = __float2half_rn(tile[tx][r]);
      lo[(int64_t)i * ldk + s] = __float2half_rn(0.0f);
    }
  }
}

// out[j] = sum_z C_z[j + N (M + 1)], out[M + i M + j] = sum_z C_z[j + i (M + 1)],
// out[M + N M + i] = sum_z C_z[M + i (M + 1)]: FP64 sums over the K chunks in
// chunk order.
__global__ void otv_scatter_kernel(const float *__restrict__ part, int kz, int N, int M,
                                   double *__restrict__ out) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;  // C index
  const int64_t ld = M + 1, cs = ld * (N + 1);
  if (e >= cs) return;
  const int i = (int)(e / ld), j = (int)(e - (int64_t)i * ld);
  if (i == N && j == M) return;  // sum of v: not an entry of O^T v
  double acc = 0.0;
  for (int z = 0; z < kz; ++z) acc += (double)part[z * cs + e];
  int64_t o;
  if (i == N) o = j;
  else if (j == M) o = (int64_t)M + (int64_t)N * M + i;
  else o = (int64_t)M + (int64_t)i * M + j;
  out[o] = acc;
}

}  // namespace vmck

using namespace vmck;

extern "C" int64_t vmck_rbm_logpsi_tc_workspace_size(int32_t N, int32_t M, int64_t n,
                                                      int32_t with_theta_out) {
  if (N <= 0 || M <= 0 || n <= 0) return 0;
  return logpsi_tc_layout(nullptr, N, M, n, !with_theta_out).bytes;
}

extern "C" int vmck_rbm_logpsi_tc(vmck_stream s, const float *params, int32_t N, int32_t M,
                                  const int8_t *x, int64_t n, float *logpsi, float *theta_out,
                                  float *tanh_out, void *workspace, int64_t workspace_bytes,
                                  int32_t *status) {
  VMCK_REQUIRE(params && x && logpsi && workspace && N > 0 && M > 0 && n > 0,
               "rbm_logpsi_tc arguments");
  VMCK_REQUIRE(n < (1ll << 31) && M < (1 << 30), "rbm_logpsi_tc sizes");
  VMCK_REQUIRE(workspace_bytes >= vmck_rbm_logpsi_tc_workspace_size(N, M, n, theta_out != nullptr),
               "rbm_logpsi_tc workspace too small");
  cudaStream_t st = as_stream(s);
  char *base = reinterpret_cast<char *>(align_up(reinterpret_cast<int64_t>(workspace), 1024));
  const LogpsiTcWs w = logpsi_tc_layout(base, N, M, n, theta_out == nullptr);
  const int np = (int)align_up(N, 8);
  const float *bvec = params, *W = params + M, *avec = params + M + (int64_t)N * M;
  abs_max_scale_kernel<float><<<1, 1024, 0, st>>>(W, (int64_t)N * M, w.scale);
  int rc = check_launch("rbm_logpsi_tc scale");
  if (rc) return rc;
  split_wt_kernel<<<ceil_div((int64_t)M * np, 256), 256, 0, st>>>(W, N, M, np, w.scale, w.wt_hi,
                                                                   w.wt_lo);
  if ((rc = check_launch("rbm_logpsi_tc split W"))) return rc;
  spins_f16_kernel<<<ceil_div(n * np, 256), 256, 0, st>>>(x, n, N, np, w.x_hi, w.x_lo);
  if ((rc = check_launch("rbm_logpsi_tc spins"))) return rc;
  float *acc = theta_out ? theta_out : w.theta;
  const SplitOperand wa{w.wt_hi, w.wt_lo, np, N, M};
  const SplitOperand xb{w.x_hi, w.x_lo, np, N, n};
  if ((rc = tc_gemm(st, wa, 0, xb, 0, 0, M, (int)n, N, acc, M, 1.0f, 0.0f, w.scale, nullptr, 0,
                    nullptr, nullptr, 0, 0, 0, nullptr, status, 0)))
    return rc;
  logpsi_epilogue_kernel<<<ceil_div(n, 8), 256, 0, st>>>(bvec, avec, x, N, M, n, acc, logpsi,
                                                         theta_out != nullptr, tanh_out);
  return check_launch("rbm_logpsi_tc epilogue");
}

extern "C" int64_t vmck_rbm_ot_v_tc_workspace_size(int32_t N, int32_t M, int64_t n) {
  if (N <= 0 || M <= 0 || n <= 0) return 0;
  return otv_tc_layout(nullptr, N, M, n, device_sms()).bytes;
}

extern "C" int vmck_rbm_ot_v_tc(vmck_stream s, const float *tanh_theta, const int8_t *x,
                                int32_t N, int32_t M, int64_t n, const double *v, double *out,
                                void *workspace, int64_t workspace_bytes, int32_t *status) {
  VMCK_REQUIRE(tanh_theta && x && v && out && workspace && N > 0 && M > 0 && n > 0,
               "rbm_ot_v_tc arguments");
  VMCK_REQUIRE(n < (1ll << 31) && M < (1 << 30), "rbm_ot_v_tc sizes");
  const int sms = device_sms();
  VMCK_REQUIRE(workspace_bytes >= otv_tc_layout(nullptr, N, M, n, sms).bytes,
               "rbm_ot_v_tc workspace too small");
  cudaStream_t st = as_stream(s);
  char *base = reinterpret_cast<char *>(align_up(reinterpret_cast<int64_t>(workspace), 1024));
  const OtvTcWs w = otv_tc_layout(base, N, M, n, sms);
  abs_max_scale_kernel<double><<<1, 1024, 0, st>>>(v, n, w.scale);  // |t| <= 1
  int rc = check_launch("rbm_ot_v_tc scale");
  if (rc) return rc;
  const unsigned sblocks = (unsigned)((w.ldk + 31) / 32);
  split_vt_transpose_kernel<<<dim3(sblocks, (unsigned)((M + 1 + 31) / 32)), 256, 0, st>>>(
      tanh_theta, v, M, n, w.ldk, w.scale, w.a_hi, w.a_lo);
  if ((rc = check_launch("rbm_ot_v_tc split"))) return rc;
  spins_transpose_kernel<<<dim3(sblocks, (unsigned)((N + 1 + 31) / 32)), 256, 0, st>>>(
      x, N, n, w.ldk, w.b_hi, w.b_lo);
  if ((rc = check_launch("rbm_ot_v_tc spins"))) return rc;
  const SplitOperand aop{w.a_hi, w.a_lo, w.ldk, w.ldk, M + 1};
  const SplitOperand bop{w.b_hi, w.b_lo, w.ldk, w.ldk, N + 1};
  const int64_t cs = (int64_t)(M + 1) * (N + 1);
  if ((rc = tc_gemm(st, aop, 0, bop, 0, 0, M + 1, N + 1, (int)w.ldk, w.part, M + 1, 1.0f, 0.0f,
                    w.scale, nullptr, 0, nullptr, nullptr, 0, 0, 0, nullptr, status, 0, 0,
                    (int)w.kchunk, cs)))
    return rc;
  otv_scatter_kernel<<<ceil_div(cs, 256), 256, 0, st>>>(w.part, w.kz, N, M, out);
  return check_launch("rbm_ot_v_tc scatter");
}

// Library context and the dense linear algebra of the SR / minSR step:
// Cholesky solves (FP64, FP32, FP32 factor + FP64 refinement), the pinv_smooth
// fallback, cuBLAS SYRK Gram matrices for the materialised-Jacobian path, and
// the small vector kernels around them.
//
// Matrix convention of the whole ABI: square matrices are row-major and only
// their LOWER triangle (row >= col) is read or written.  Seen by the
// column-major libraries that memory is the UPPER triangle of the same
// symmetric matrix, hence CUBLAS_FILL_MODE_UPPER below.
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstring>

#include "chol_tc.cuh"
#include "common.cuh"

struct vmck_ctx {
  int device = 0;
  cublasHandle_t blas = nullptr;
  cusolverDnHandle_t solver = nullptr;
  cusolverDnParams_t params = nullptr;
  void *dwork = nullptr;
  size_t dwork_bytes = 0;
  void *hwork = nullptr;
  size_t hwork_bytes = 0;
  void *aux = nullptr;
  size_t aux_bytes = 0;
  int *d_info = nullptr;
  // look-ahead Cholesky: a second stream / cuBLAS handle for the trailing
  // updates and a pool of events (two per panel), created on first use
  cudaStream_t side = nullptr;
  cudaStream_t chain = nullptr;  // highest priority: the factorisation's critical path
  cudaStream_t chain2 = nullptr;  // highest priority: the rest of each panel's block-row update
  cublasHandle_t blas2 = nullptr;
  cudaEvent_t *events = nullptr;
  int n_events = 0;
  // tensor-core factorisation (factor_mode 4): split panels, leaf inverses, and
  // the padded copy when n is not a multiple of 4
  void *tcws = nullptr;
  size_t tcws_bytes = 0;
  // the shifted-preconditioner fallback: per-attempt status word
  int32_t *d_attempt = nullptr;
};

namespace vmck {

#define VMCK_BLAS(call)                                                        \
  do {                                                                         \
    cublasStatus_t st_ = (call);                                               \
    if (st_ != CUBLAS_STATUS_SUCCESS) {                                        \
      ::vmck::set_last_error("%s:%d %s: cublas status %d", __FILE__, __LINE__, \
                             #call, (int)st_);                                 \
      return VMCK_ERR_LIBRARY;                                                 \
    }                                                                          \
  } while (0)

#define VMCK_SOLVER(call)                                                      \
  do {                                                                         \
    cusolverStatus_t st_ = (call);                                             \
    if (st_ != CUSOLVER_STATUS_SUCCESS) {                                      \
      ::vmck::set_last_error("%s:%d %s: cusolver status %d", __FILE__,         \
                             __LINE__, #call, (int)st_);                       \
      return VMCK_ERR_LIBRARY;                                                 \
    }                                                                          \
  } while (0)

static int grow(void **p, size_t *cap, size_t need, cudaStream_t st) {
  if (need <= *cap) return VMCK_OK;
  if (*p) {
    VMCK_CUDA(cudaStreamSynchronize(st));
    VMCK_CUDA(cudaFree(*p));
    *p = nullptr;
    *cap = 0;
  }
  size_t bytes = std::max<size_t>(need, 1 << 20);
  if (cudaMalloc(p, bytes) != cudaSuccess) {
    cudaGetLastError();
    set_last_error("workspace allocation of %zu bytes failed", bytes);
    return VMCK_ERR_NOMEM;
  }
  *cap = bytes;
  return VMCK_OK;
}

static int grow_host(vmck_ctx *c, size_t need) {
  if (need <= c->hwork_bytes) return VMCK_OK;
  free(c->hwork);
  c->hwork = malloc(std::max<size_t>(need, 64));
  if (!c->hwork) {
    c->hwork_bytes = 0;
    return VMCK_ERR_NOMEM;
  }
  c->hwork_bytes = std::max<size_t>(need, 64);
  return VMCK_OK;
}

static int bind(vmck_ctx *c, cudaStream_t st) {
  VMCK_BLAS(cublasSetStream(c->blas, st));
  VMCK_SOLVER(cusolverDnSetStream(c->solver, st));
  return VMCK_OK;
}

// ------------------------------------------------------------ small kernels
__global__ void add_diag_kernel(void *A, int dtype, int64_t n, double shift) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (dtype == VMCK_F64)
    static_cast<double *>(A)[i * n + i] += shift;
  else
    static_cast<float *>(A)[i * n + i] += (float)shift;
}

template <typename T>
__global__ void solve_check_kernel(const int *info, const T *x, const T *b, int64_t n,
                                   int32_t *status) {
  __shared__ int red[32];
  int bad = 0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
    bad |= !isfinite((double)x[i]) || !isfinite((double)b[i]);
  bad = block_sum(bad, red);
  if (threadIdx.x == 0 && status) {
    int s = 0;
    if (*info != 0) s |= VMCK_DEV_NOT_SPD;
    if (bad) s |= VMCK_DEV_NONFINITE;
    if (s) atomicOr(status, s);
  }
}

// Kernels of the refinement loop take `done` (nullable): once the residual check
// has set it, they return at entry, so the remaining iterations cost only their
// launches.
__device__ __forceinline__ bool refine_done(const int *done) {
  return done && *reinterpret_cast<const volatile int *>(done) != 0;
}

__global__ void d2f_kernel(const double *in, float *out, int64_t n, const int *done = nullptr) {
  if (refine_done(done)) return;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}

__global__ void axpy_f2d_kernel(double *x, const float *d, int64_t n, const int *done) {
  if (refine_done(done)) return;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) x[i] += (double)d[i];
}

// *done = 1 when ||r|| <= tol ||b|| (FP64 sums of squares, one block) or, with
// prev (nullable), when ||r|| > prev / 2: the residual has stopped falling (the
// FP64 rounding floor of the all-FP64 solve); prev then receives ||r||.
__global__ void __launch_bounds__(256) refine_converged_kernel(const double *__restrict__ r,
                                                               const double *__restrict__ b,
                                                               int64_t n, double tol, int *done,
                                                               double *prev = nullptr) {
  if (refine_done(done)) return;
  __shared__ double red[2][8];
  double sr = 0.0, sb = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    sr += r[i] * r[i];
    sb += b[i] * b[i];
  }
  sr = warp_sum(sr);
  sb = warp_sum(sb);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][w] = sr;
    red[1][w] = sb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tr = 0.0, tb = 0.0;
    for (int k = 0; k < 8; ++k) {
      tr += red[0][k];
      tb += red[1][k];
    }
    const double nr = sqrt(tr);
    if (nr <= tol * sqrt(tb)) *done = 1;  // false for NaN: the loop goes on
    if (prev) {
      if (nr > 0.5 * *prev) *done = 1;
      *prev = nr;
    }
  }
}

__global__ void refine_check_kernel(const double *nr, const double *nb, const int *info,
                                    double tol, int32_t *status, double *res_out) {
  double rel = *nr / *nb;
  if (res_out) *res_out = rel;
  if (status) {
    int s = 0;
    if (*info != 0) s |= VMCK_DEV_NOT_SPD;
    if (!isfinite(rel)) s |= VMCK_DEV_NONFINITE;
    else if (!(rel <= tol)) s |= VMCK_DEV_NO_CONVERGE;
    if (s) atomicOr(status, s);
  }
}

// ---- flexible preconditioned CG (the fallback of a failed FP32 factor)
// One block: fixed reduction order, so the iteration is deterministic.
__device__ __forceinline__ double block_sum_1024(double v, double *red) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
  return t;  // valid in thread 0
}

// sc: [0] r.z, [1] alpha, [2] beta
__global__ void __launch_bounds__(1024) pcg_start_kernel(const double *__restrict__ r,
                                                         const double *__restrict__ z,
                                                         int64_t n, double *sc) {
  __shared__ double red[32];
  double a = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) a = fma(r[i], z[i], a);
  a = block_sum_1024(a, red);
  if (threadIdx.x == 0) sc[0] = a;
}

// alpha = r.z / p.A p with qn = -A p; a direction of non-positive curvature
// (A not positive definite) or a non-finite value ends the iteration.
__global__ void __launch_bounds__(1024) pcg_alpha_kernel(const double *__restrict__ p,
                                                         const double *__restrict__ qn,
                                                         int64_t n, double *sc, int32_t *status,
                                                         int *done) {
  if (refine_done(done)) return;
  __shared__ double red[32];
  double a = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) a = fma(p[i], qn[i], a);
  a = block_sum_1024(a, red);
  if (threadIdx.x == 0) {
    const double pq = -a;
    const double alpha = sc[0] / pq;
    if (!(pq > 0.0) || !isfinite(alpha)) {
      atomicOr(status, isfinite(pq) ? VMCK_DEV_NOT_SPD : VMCK_DEV_NONFINITE);
      *done = 1;
    }
    sc[1] = alpha;
  }
}

__global__ void pcg_update_kernel(double *__restrict__ x, double *__restrict__ r,
                                  const double *__restrict__ p, const double *__restrict__ qn,
                                  int64_t n, const double *sc, const int *done) {
  if (refine_done(done)) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double alpha = sc[1];
  x[i] = fma(alpha, p[i], x[i]);
  r[i] = fma(alpha, qn[i], r[i]);  // r - alpha A p
}

__global__ void f2d_copy_kernel(const float *__restrict__ in, double *__restrict__ out, int64_t n,
                                const int *done) {
  if (refine_done(done)) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)in[i];
}

// Polak-Ribiere beta = z.(r - r_old) / (r_old.z_old), r - r_old = alpha qn:
// stays a conjugate-gradient step when the FP32 preconditioner is not exactly
// the same linear map from one application to the next.
__global__ void __launch_bounds__(1024) pcg_beta_kernel(const double *__restrict__ r,
                                                        const double *__restrict__ z,
                                                        const double *__restrict__ qn,
                                                        int64_t n, double *sc, const int *done) {
  if (refine_done(done)) return;
  __shared__ double red[32];
  double a = 0.0, b = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    a = fma(r[i], z[i], a);
    b = fma(z[i], qn[i], b);
  }
  a = block_sum_1024(a, red);
  b = block_sum_1024(b, red);
  if (threadIdx.x == 0) {
    sc[2] = sc[1] * b / sc[0];
    sc[0] = a;
  }
}

__global__ void pcg_direction_kernel(double *__restrict__ p, const double *__restrict__ z,
                                     int64_t n, const double *sc, const int *done) {
  if (refine_done(done)) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) p[i] = fma(sc[2], p[i], z[i]);
}

__global__ void status_or_kernel(int32_t *status, const int32_t *bits) {
  if (*bits) atomicOr(status, *bits);
}

__global__ void trace_kernel(const double *__restrict__ A, int64_t n, double *out) {
  __shared__ double red[32];
  double a = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) a += A[i * n + i];
  a = block_sum_1024(a, red);
  if (threadIdx.x == 0) *out = a;
}

__global__ void pinv_filter_kernel(const double *w, double *y, int64_t n, double rtol,
                                   double rtol_smooth) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double wmax = w[n - 1];
  const double rel = fabs(w[i] / wmax);
  double inv = rel > rtol ? 1.0 / w[i] : 0.0;
  double q = rtol_smooth / rel;
  double q2 = q * q;
  inv *= 1.0 / (1.0 + q2 * q2 * q2);
  y[i] *= inv;
}

__global__ void center_scale_kernel(const double *e, const double *mean, int64_t n, double f,
                                    double *out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = f * (e[i] - *mean);
}

__global__ void center_update_kernel(const double *raw, const double *obar, const double *aux,
                                     int64_t n, int64_t P, double scale, double *upd) {
  __shared__ double red[32];
  double s = 0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += aux[i];
  s = block_sum(s, red);
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P;
       p += (int64_t)gridDim.x * blockDim.x)
    upd[p] = scale * (raw[p] - obar[p] * s);
}

__global__ void sgd_kernel(double *p, const double *u, int64_t P, double lr, float *p32) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P) return;
  double v = p[i] - lr * u[i];
  p[i] = v;
  if (p32) p32[i] = (float)v;
}

// ------------------------------------------------------------ recursive Cholesky
// Upper Cholesky A = U^T U of a column-major FP32 matrix (our row-major lower
// triangle), in place, by recursive halving (Gustavson / Elmroth style): every
// flop outside the leaves is a GEMM, and the GEMMs run with cuBLAS'
// FP32-accurate BF16x9 tensor-core emulation.  Leaves (<= R.leaf) use
// cuSOLVER POTRF (factor_mode 2) or potrf_leaf_kernel (factor_mode 3), and
// cuBLAS TRSM / SYRK.
constexpr int64_t CHOL_LEAF = 1024;
constexpr int LEAF_B = 128;        // potrf_leaf_kernel block
constexpr int LEAF_THREADS = 512;
constexpr int64_t PANEL_W_DEFAULT = 512;  // blocked factorization panel
// Panel width of the blocked Cholesky: VMCK_CHOL_PANEL (a multiple of 128,
// 128 - 2048) overrides the default, read once per process.
static int64_t chol_panel_width() {
  static const int64_t w = [] {
    const char *e = getenv("VMCK_CHOL_PANEL");
    const long v = e ? strtol(e, nullptr, 10) : 0;
    return (v >= 128 && v <= 2048 && v % 128 == 0) ? (int64_t)v : PANEL_W_DEFAULT;
  }();
  return w;
}
constexpr int64_t STRIP_W = 2048;  // trailing-update GEMM strip width

static int64_t half_split(int64_t n) {
  int64_t h = ((n / 2) + 255) / 256 * 256;
  if (h >= n) h = ((n / 2) + LEAF_B - 1) / LEAF_B * LEAF_B;
  return (h >= n || h <= 0) ? n / 2 : h;
}

__global__ void info_accumulate_kernel(const int *info, int32_t *status) {
  if (*info != 0 && status) atomicOr(status, VMCK_DEV_NOT_SPD);
}

// Leaf kernels of the blocked Cholesky.  Both keep a b x b (b <= 128) upper
// factor in shared memory as Us[i * LEAF_LD + j] (row i, column j, i <= j; rows
// 16-byte aligned) and work in 32-row panels:
//   (a) a latency-bound 32-wide step done in registers with warp shuffles,
//   (b) a rank-32 update of what remains, as 4 x 4 register tiles.
constexpr int LEAF_LD = LEAF_B + 4;
constexpr unsigned FULL_MASK = 0xffffffffu;

// 4-byte asynchronous global -> shared copies (cp.async), so that all of a
// thread's loads are in flight at once; cp_async_wait() completes them.
__device__ __forceinline__ void cp_async4(float *dst, const float *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(
                   static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Load the upper triangle of the b x b column-major block A (lda) into Us
// (LEAF_ROWS x LEAF_LD), zeros elsewhere: the 4 x 4 tiles of a block whose size
// is not a multiple of 4 run up to 3 rows / columns past it.  The caller
// completes the copies with cp_async_wait() and a barrier.
constexpr int LEAF_ROWS = LEAF_B + 4;
__device__ inline void leaf_load_upper(float *Us, const float *A, int64_t lda, int b) {
  for (int e = threadIdx.x; e < LEAF_ROWS * LEAF_LD; e += blockDim.x) {
    const int j = e / LEAF_ROWS, i = e - j * LEAF_ROWS;
    if (i <= j && j < b)
      cp_async4(&Us[i * LEAF_LD + j], A + (int64_t)j * lda + i);
    else
      Us[i * LEAF_LD + j] = 0.0f;
  }
}

// Store the upper triangle of Us back to the b x b column-major block A.
__device__ inline void leaf_store_upper(const float *Us, float *A, int64_t lda, int b) {
  for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
    const int j = e / b, i = e - j * b;
    if (i <= j) A[(int64_t)j * lda + i] = Us[i * LEAF_LD + j];
  }
}

// Forward substitution U_pp^T X = V for one 32-row panel (rows p..p+pw-1) of a
// column held by 4 consecutive lanes: lane quarter q owns rows p + 8q .. p + 8q + 7
// (v[0..7]), so its slice of a row of U_pp is two 16-byte loads.  rinv[i] =
// 1 / u_ii.  All 32 lanes of the warp must call it; p is a multiple of 32.
__device__ __forceinline__ void panel_forward(const float *Us, const float *rinv, int p, int pw,
                                              int q, float (&v)[8]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    if (k < pw) {
      const float mine = v[k & 7] * rinv[p + k];
      const float x = __shfl_sync(FULL_MASK, mine, (lane & ~3) | (k >> 3));
      if (q == (k >> 3)) v[k & 7] = x;
      if (8 * q + 7 > k) {  // rows of this quarter below k
        const float4 u0 = *reinterpret_cast<const float4 *>(&Us[(p + k) * LEAF_LD + p + 8 * q]);
        const float4 u1 = *reinterpret_cast<const float4 *>(&Us[(p + k) * LEAF_LD + p + 8 * q + 4]);
        const float uv[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
#pragma unroll
        for (int r = 0; r < 8; ++r)
          if (8 * q + r > k && 8 * q + r < pw) v[r] = __fmaf_rn(-uv[r], x, v[r]);
      }
    }
  }
}

// Inverse of the upper-triangular 32 x 32 diagonal block at (p, p) of Us (rows
// / columns past pw are treated as the identity), by one warp: lane l computes
// column l of X = U_pp^-1 by back substitution, all rows held in registers
// (fully unrolled, so the indices are compile-time).  Writes X row-major
// (X[i * 32 + l], zeros below the diagonal) to dst.  rinv[p + i] = 1 / u_ii.
__device__ inline void invert_diag32(const float *Us, const float *rinv, int p, int pw,
                                     float *dst) {
  const int lane = threadIdx.x & 31;
  float x[32];
#pragma unroll
  for (int i = 31; i >= 0; --i) {
    float sacc = (i == lane) ? 1.0f : 0.0f;
#pragma unroll
    for (int k = i + 1; k < 32; ++k) {
      const float u = (i < pw && k < pw) ? Us[(p + i) * LEAF_LD + p + k] : 0.0f;
      sacc = __fmaf_rn(-u, x[k], sacc);
    }
    x[i] = (i < pw) ? sacc * rinv[p + i] : sacc;
  }
#pragma unroll
  for (int i = 0; i < 32; ++i) dst[i * 32 + lane] = (i <= lane) ? x[i] : 0.0f;
}

// Right-looking upper Cholesky of one b x b diagonal block (b <= 128) of a
// column-major matrix.  Per 32-row panel: (a) warp 0 factors the 32 x 32
// diagonal block in registers (lane l holds column l; the unused part of a short
// panel is padded with the identity), (b) four lanes per column solve the panel
// row, (c) rank-32 update of the trailing block.  A non-positive (or NaN) pivot
// sets VMCK_DEV_NOT_SPD and is replaced by 1; the caller falls back on the
// status word.
__global__ void __launch_bounds__(LEAF_THREADS) potrf_leaf_kernel(float *A, int64_t lda, int b,
                                                                  int32_t *status, float *dinv) {
  extern __shared__ __align__(16) float Us[];
  __shared__ float rinv[LEAF_B];
  __shared__ __align__(16) float rowk[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  leaf_load_upper(Us, A, lda, b);
  cp_async_wait();
  __syncthreads();
  bool bad = false;
  for (int p = 0; p < b; p += 32) {
    const int pw = (b - p) < 32 ? (b - p) : 32;
    if (warp == 0) {  // (a) lane l holds column p + l of the 32 x 32 diagonal block
      float col[32];
#pragma unroll
      for (int i = 0; i < 32; ++i)
        col[i] = (lane < pw && i <= lane) ? Us[(p + i) * LEAF_LD + p + lane] : (i == lane ? 1.0f : 0.0f);
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        const float d = __shfl_sync(FULL_MASK, col[k], k);
        const bool ok = d > 0.0f;
        if (k < pw) bad |= !ok;
        const float ri = ok ? rsqrtf(d) : 1.0f;
        col[k] = (lane == k) ? (ok ? d * ri : 1.0f) : col[k] * ri;  // row k scaled
        if (k < 31) {  // rank-1 update of the rows below k; lanes left of a row update
                       // lower-triangle entries, which are never read
          rowk[lane] = col[k];
          __syncwarp();
          float rv[32];
#pragma unroll
          for (int g = 0; g < 8; ++g) {
            const float4 t = reinterpret_cast<const float4 *>(rowk)[g];
            rv[4 * g] = t.x;
            rv[4 * g + 1] = t.y;
            rv[4 * g + 2] = t.z;
            rv[4 * g + 3] = t.w;
          }
#pragma unroll
          for (int i = k + 1; i < 32; ++i) col[i] = __fmaf_rn(-rv[i], col[k], col[i]);
          __syncwarp();
        }
      }
#pragma unroll
      for (int i = 0; i < 32; ++i)
        if (lane < pw && i <= lane) Us[(p + i) * LEAF_LD + p + lane] = col[i];
      float dl = 1.0f;
#pragma unroll
      for (int i = 0; i < 32; ++i)
        if (i == lane) dl = col[i];
      if (lane < pw) rinv[p + lane] = 1.0f / dl;
    }
    __syncthreads();
    const int m = b - p - pw;  // trailing size
    if (m <= 0) break;
    {  // (b) panel row: 4 lanes per column j = p + pw + c
      const int c = tid >> 2, q = tid & 3;
      if (warp < (m + 7) / 8) {  // whole warps, 8 columns each
        const bool valid = c < m;
        const int j = p + pw + (valid ? c : 0);
        float v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) v[r] = (valid && 8 * q + r < pw) ? Us[(p + 8 * q + r) * LEAF_LD + j] : 0.0f;
        panel_forward(Us, rinv, p, pw, q, v);
        if (valid) {
#pragma unroll
          for (int r = 0; r < 8; ++r)
            if (8 * q + r < pw) Us[(p + 8 * q + r) * LEAF_LD + j] = v[r];
        }
      }
    }
    __syncthreads();
    {  // (c) U(i, j) -= sum_k X(p+k, i) X(p+k, j), 4 x 4 tiles with ti <= tj
      const int nt = (m + 3) / 4, base = p + pw;
      for (int t = tid; t < nt * nt; t += blockDim.x) {
        const int ti = t / nt, tj = t - ti * nt;
        if (ti > tj) continue;
        const int i0 = base + 4 * ti, j0 = base + 4 * tj;
        float acc[4][4] = {};
#pragma unroll 8
        for (int k = 0; k < 32; ++k) {
          const float4 a = *reinterpret_cast<const float4 *>(&Us[(p + k) * LEAF_LD + i0]);
          const float4 bb = *reinterpret_cast<const float4 *>(&Us[(p + k) * LEAF_LD + j0]);
          const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {bb.x, bb.y, bb.z, bb.w};
#pragma unroll
          for (int x = 0; x < 4; ++x)
#pragma unroll
            for (int y = 0; y < 4; ++y) acc[x][y] = __fmaf_rn(av[x], bv[y], acc[x][y]);
        }
#pragma unroll
        for (int x = 0; x < 4; ++x)
#pragma unroll
          for (int y = 0; y < 4; ++y) Us[(i0 + x) * LEAF_LD + j0 + y] -= acc[x][y];
      }
    }
    __syncthreads();
  }
  if (__syncthreads_or(bad) && tid == 0 && status) atomicOr(status, VMCK_DEV_NOT_SPD);
  // inverses of the 32 x 32 diagonal blocks for trsm_leaf_kernel (warp w: block w)
  if (dinv && warp < (b + 31) / 32) {
    const int p = 32 * warp, pw = (b - p) < 32 ? (b - p) : 32;
    invert_diag32(Us, rinv, p, pw, dinv + warp * 1024);
  }
  leaf_store_upper(Us, A, lda, b);
}

// B (m x nrhs, column-major) <- U^-T B for the m x m upper factor U (m <= 128)
// of one leaf.  CTA c solves columns [64c, 64c + 64) with U and its column block
// (Bs[k * TRSM_LD + c]) in shared memory, in the same 32-row panels: (a) four
// lanes per column do the forward substitution of the panel, (b) a rank-32
// update of the rows below.
constexpr int TRSM_COLS = 64;
constexpr int TRSM_LD = TRSM_COLS + 4;

// Forward substitution Us^T X = Bs in place for an m x m upper Us (m <= 128) and a
// 64-column Bs[k * TRSM_LD + c] in shared memory; rinv[i] = 1 / u_ii.  With Dinv
// (the row-major inverses of the 32 x 32 diagonal blocks, 1024 floats each) the
// panel step is a 32 x 32 x 64 product X_p = Dinv_p^T B_p instead of a 32-step
// substitution.
__device__ void leaf_trsm_core(const float *Us, float *Bs, const float *rinv, int m,
                               const float *Dinv = nullptr) {
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int p = 0; p < m; p += 32) {
    const int pw = (m - p) < 32 ? (m - p) : 32;
    if (Dinv) {  // (a') 128 threads: 4 x 4 tiles of X_p (rows i0.., columns c0..)
      const float *D = Dinv + (p >> 5) * 1024;
      float acc[4][4] = {};
      const int i0 = 4 * (tid >> 4), cc0 = 4 * (tid & 15);
      if (tid < 128) {
#pragma unroll 8
        for (int k = 0; k < 32; ++k) {
          const float4 dv = *reinterpret_cast<const float4 *>(&D[k * 32 + i0]);
          const float4 bv = *reinterpret_cast<const float4 *>(&Bs[(p + k) * TRSM_LD + cc0]);
          const float av[4] = {dv.x, dv.y, dv.z, dv.w}, xv[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
          for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int y = 0; y < 4; ++y) acc[u][y] = __fmaf_rn(av[u], xv[y], acc[u][y]);
        }
      }
      __syncthreads();
      if (tid < 128) {
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (i0 + u < pw) {
#pragma unroll
            for (int y = 0; y < 4; ++y) Bs[(p + i0 + u) * TRSM_LD + cc0 + y] = acc[u][y];
          }
      }
    } else if (warp < 8) {  // (a) 256 threads: column c = tid >> 2, quarter q = tid & 3
      const int c = tid >> 2, q = tid & 3;
      float v[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) v[r] = (8 * q + r < pw) ? Bs[(p + 8 * q + r) * TRSM_LD + c] : 0.0f;
      panel_forward(Us, rinv, p, pw, q, v);
#pragma unroll
      for (int r = 0; r < 8; ++r)
        if (8 * q + r < pw) Bs[(p + 8 * q + r) * TRSM_LD + c] = v[r];
    }
    __syncthreads();
    const int rows = m - p - pw;
    if (rows <= 0) break;
    {  // (b) B(i, c) -= sum_k U(p+k, i) X(p+k, c), 4 x 4 tiles
      const int nti = (rows + 3) / 4, base = p + pw;
      for (int t = tid; t < nti * (TRSM_COLS / 4); t += blockDim.x) {
        const int ti = t / (TRSM_COLS / 4), tc = t - ti * (TRSM_COLS / 4);
        const int i0 = base + 4 * ti, cc0 = 4 * tc;
        float acc[4][4] = {};
#pragma unroll 8
        for (int k = 0; k < 32; ++k) {
          const float4 a = *reinterpret_cast<const float4 *>(&Us[(p + k) * LEAF_LD + i0]);
          const float4 x = *reinterpret_cast<const float4 *>(&Bs[(p + k) * TRSM_LD + cc0]);
          const float av[4] = {a.x, a.y, a.z, a.w}, xv[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
          for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int y = 0; y < 4; ++y) acc[u][y] = __fmaf_rn(av[u], xv[y], acc[u][y]);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int y = 0; y < 4; ++y) Bs[(i0 + u) * TRSM_LD + cc0 + y] -= acc[u][y];
      }
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(LEAF_THREADS) trsm_leaf_kernel(const float *__restrict__ Ug,
                                                                 int64_t ldu, int m, float *B,
                                                                 int64_t ldb, int64_t nrhs,
                                                                 const float *__restrict__ dinv) {
  extern __shared__ __align__(16) float sm[];
  float *Us = sm;                         // LEAF_ROWS x LEAF_LD
  float *Bs = sm + LEAF_ROWS * LEAF_LD;   // LEAF_ROWS x TRSM_LD
  float *Ds = Bs + LEAF_ROWS * TRSM_LD;   // 4 x 1024 (diagonal-block inverses)
  __shared__ float rinv[LEAF_B];
  const int tid = threadIdx.x;
  const int64_t c0 = (int64_t)blockIdx.x * TRSM_COLS;
  const int nc = (int)((nrhs - c0) < TRSM_COLS ? (nrhs - c0) : TRSM_COLS);
  leaf_load_upper(Us, Ug, ldu, m);
  for (int e = tid; e < TRSM_LD * LEAF_ROWS; e += blockDim.x) {
    const int c = e / LEAF_ROWS, k = e - c * LEAF_ROWS;
    if (c < nc && k < m)
      cp_async4(&Bs[k * TRSM_LD + c], B + (c0 + c) * ldb + k);
    else
      Bs[k * TRSM_LD + c] = 0.0f;
  }
  if (dinv)
    for (int e = tid; e < 4 * 1024; e += blockDim.x) cp_async4(&Ds[e], dinv + e);
  cp_async_wait();
  __syncthreads();
  if (tid < m) rinv[tid] = 1.0f / Us[tid * LEAF_LD + tid];
  __syncthreads();
  leaf_trsm_core(Us, Bs, rinv, m, dinv ? Ds : nullptr);
  for (int e = tid; e < TRSM_COLS * m; e += blockDim.x) {
    const int c = e / m, k = e - c * m;
    if (c < nc) B[(c0 + c) * ldb + k] = Bs[k * TRSM_LD + c];
  }
}

// ------------------------------------------------------------ blocked triangular solves
// U^T y = r and U x = y for the FP32 upper factor U (column-major, ld n) in
// 128-row blocks, for the refinement loop.  trsv_inv_kernel stores
// Y_K = U_KK^-T (lower, column-major 128 x 128, zero-padded) for every diagonal
// block, so a block's own solve is a 128 x 128 product.  The two solve kernels
// are persistent: CTAs take block tickets in order from an atomic counter, so
// every block a CTA waits for has been claimed by a CTA that is already running
// and that never waits for a later block; a finished block is published with a
// release store of the call's epoch into its flag.  Waits are bounded (the
// library's wait limit, 2 s of wall time by default); a wait that runs out raises
// VMCK_DEV_TIMEOUT and sets the abort word, which makes every other wait give up
// at once.  A CTA holds nothing when it gives up (no copies or MMAs in flight).
constexpr int TB = 128;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long wall_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Every lane of the warp spins; returns false if the solve was aborted.
__device__ __forceinline__ bool trsv_wait(const unsigned *flag, unsigned epoch, unsigned *abort_w,
                          int32_t *status, unsigned long long limit) {
  const unsigned long long t0 = wall_ns();
  for (unsigned it = 0;; ++it) {
    if (ld_acquire_u32(flag) == epoch) return true;
    if (ld_acquire_u32(abort_w) == epoch) return false;
    if (it >= 4 && wall_ns() - t0 > limit) {
      if (status) atomicOr(status, VMCK_DEV_TIMEOUT);
      atomicExch(abort_w, epoch);
      return false;
    }
  }
}

__global__ void __launch_bounds__(LEAF_THREADS) trsv_inv_kernel(const float *__restrict__ U,
                                                                int64_t n, float *Yinv) {
  extern __shared__ __align__(16) float sm[];
  float *Us = sm;
  float *Bs = sm + LEAF_ROWS * LEAF_LD;
  __shared__ float rinv[LEAF_B];
  const int tid = threadIdx.x;
  const int64_t K = blockIdx.y, k0 = K * TB;
  const int m = (int)((n - k0) < TB ? (n - k0) : TB);
  const int cbase = blockIdx.x * TRSM_COLS;  // identity columns [cbase, cbase + 64)
  leaf_load_upper(Us, U + k0 + k0 * n, n, m);
  for (int e = tid; e < TRSM_LD * LEAF_ROWS; e += blockDim.x) {
    const int c = e / LEAF_ROWS, k = e - c * LEAF_ROWS;
    Bs[k * TRSM_LD + c] = (c < TRSM_COLS && k < m && k == cbase + c) ? 1.0f : 0.0f;
  }
  cp_async_wait();
  __syncthreads();
  if (tid < m) rinv[tid] = 1.0f / Us[tid * LEAF_LD + tid];
  __syncthreads();
  leaf_trsm_core(Us, Bs, rinv, m);
  float *Y = Yinv + K * TB * TB;
  for (int e = tid; e < TRSM_COLS * TB; e += blockDim.x) {
    const int c = e / TB, k = e - c * TB;
    Y[(int64_t)(cbase + c) * TB + k] = (k < m && cbase + c < m) ? Bs[k * TRSM_LD + c] : 0.0f;
  }
}

struct TrsvSync {
  unsigned *flags;   // nb
  unsigned *ticket;  // 1
  unsigned *abort_w; // 1
  unsigned long long wait_ns;  // limit of each wait
};

// y = U^-T r.  Block K: z = r_K - sum_{J<K} U_JK^T y_J (warp w: columns 8w..8w+7 of
// block K, each a 128-long contiguous column segment per J), then y_K = Y_K z.
__global__ void __launch_bounds__(LEAF_THREADS) trsv_fwd_kernel(const float *__restrict__ U,
                                                                int64_t n,
                                                                const float *__restrict__ Yinv,
                                                                const float *__restrict__ r,
                                                                float *y, TrsvSync sy,
                                                                unsigned epoch, int32_t *status,
                                                                const int *done) {
  if (refine_done(done)) return;  // before any ticket: every CTA leaves
  __shared__ float z[TB];
  __shared__ float part[4][TB];
  __shared__ int K_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nb = (int)((n + TB - 1) / TB);
  while (true) {
    __syncthreads();
    if (tid == 0) K_s = (int)atomicAdd(sy.ticket, 1u);
    __syncthreads();
    const int K = K_s;
    if (K >= nb) break;
    const int64_t k0 = (int64_t)K * TB;
    const int mk = (int)((n - k0) < TB ? (n - k0) : TB);
    // this thread's share of Y_K for the final product, loaded before any wait
    const int yc = tid & (TB - 1), yh = tid >> 7;
    float ys[32];
    {
      const float *Y = Yinv + (int64_t)K * TB * TB;
#pragma unroll
      for (int i = 0; i < 32; ++i) ys[i] = __ldg(Y + (32 * yh + i) * TB + yc);
    }
    float acc[8] = {};
    bool alive = true;
    for (int J = 0; J < K && alive; ++J) {
      float4 u[8];  // U_JK does not depend on y: load it before waiting for y_J
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int c = 8 * warp + q;
        u[q] = (c < mk) ? __ldg(reinterpret_cast<const float4 *>(U + (k0 + c) * n + (int64_t)J * TB) + lane)
                        : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
      alive = trsv_wait(sy.flags + J, epoch, sy.abort_w, status, sy.wait_ns);
      if (!alive) break;
      const float4 yj = __ldcg(reinterpret_cast<const float4 *>(y + (int64_t)J * TB) + lane);
#pragma unroll
      for (int q = 0; q < 8; ++q)
        acc[q] = __fmaf_rn(u[q].x, yj.x, __fmaf_rn(u[q].y, yj.y, __fmaf_rn(u[q].z, yj.z, __fmaf_rn(u[q].w, yj.w, acc[q]))));
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float v = warp_sum(acc[q]);
      const int c = 8 * warp + q;
      if (lane == 0) z[c] = (c < mk) ? r[k0 + c] - v : 0.0f;
    }
    __syncthreads();
    {  // y_K[c] = sum_c' Y_K(c, c') z[c'], thread (h, c): c' in [32h, 32h + 32)
      float sacc = 0.0f;
#pragma unroll
      for (int i = 0; i < 32; ++i) sacc = __fmaf_rn(ys[i], z[32 * yh + i], sacc);
      part[yh][yc] = sacc;
    }
    __syncthreads();
    if (tid < mk) {
      __stcg(y + k0 + tid, (part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]));
      __threadfence();
    }
    __syncthreads();
    if (tid == 0) st_release_u32(sy.flags + K, epoch);
  }
}

// x = U^-1 y.  Block K (taken from the last): w = y_K - sum_{J>K} U_KJ x_J (warp w:
// columns 8w..8w+7 of every later block J; lane: rows 4 lane..4 lane+3), then
// x_K = Y_K^T w.
__global__ void __launch_bounds__(LEAF_THREADS) trsv_bwd_kernel(const float *__restrict__ U,
                                                                int64_t n,
                                                                const float *__restrict__ Yinv,
                                                                const float *__restrict__ yv,
                                                                float *x, TrsvSync sy,
                                                                unsigned epoch, int32_t *status,
                                                                const int *done) {
  if (refine_done(done)) return;
  __shared__ __align__(16) float wv[TB];
  __shared__ float part[16][TB];
  __shared__ int K_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nb = (int)((n + TB - 1) / TB);
  while (true) {
    __syncthreads();
    if (tid == 0) K_s = nb - 1 - (int)atomicAdd(sy.ticket, 1u);
    __syncthreads();
    const int K = K_s;
    if (K < 0) break;
    const int64_t k0 = (int64_t)K * TB;
    const int mk = (int)((n - k0) < TB ? (n - k0) : TB);
    const bool full = (4 * lane + 3) < mk;
    // this warp's columns of Y_K for the final product, loaded before any wait
    float4 ycol[8];
    {
      const float *Y = Yinv + (int64_t)K * TB * TB;
#pragma unroll
      for (int q = 0; q < 8; ++q)
        ycol[q] = __ldg(reinterpret_cast<const float4 *>(Y + (int64_t)(8 * warp + q) * TB) + lane);
    }
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
    bool alive = true;
    for (int J = nb - 1; J > K && alive; --J) {
      const int64_t j0 = (int64_t)J * TB;
      const int mj = (int)((n - j0) < TB ? (n - j0) : TB);
      float4 u[8];  // U_KJ does not depend on x: load it before waiting for x_J
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int cj = 8 * warp + q;
        const float *col = U + (j0 + cj) * n + k0;
        if (cj >= mj) {
          u[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        } else if (full) {
          u[q] = __ldg(reinterpret_cast<const float4 *>(col) + lane);
        } else {
          const int rr = 4 * lane;
          u[q] = make_float4(rr < mk ? col[rr] : 0.0f, rr + 1 < mk ? col[rr + 1] : 0.0f,
                             rr + 2 < mk ? col[rr + 2] : 0.0f, 0.0f);
        }
      }
      alive = trsv_wait(sy.flags + J, epoch, sy.abort_w, status, sy.wait_ns);
      if (!alive) break;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float xj = (8 * warp + q < mj) ? __ldcg(x + j0 + 8 * warp + q) : 0.0f;
        a0 = __fmaf_rn(u[q].x, xj, a0);
        a1 = __fmaf_rn(u[q].y, xj, a1);
        a2 = __fmaf_rn(u[q].z, xj, a2);
        a3 = __fmaf_rn(u[q].w, xj, a3);
      }
    }
    part[warp][4 * lane] = a0;
    part[warp][4 * lane + 1] = a1;
    part[warp][4 * lane + 2] = a2;
    part[warp][4 * lane + 3] = a3;
    __syncthreads();
    if (tid < TB) {
      float sum = 0.0f;
#pragma unroll
      for (int w = 0; w < 16; ++w) sum += part[w][tid];
      wv[tid] = (tid < mk) ? yv[k0 + tid] - sum : 0.0f;
    }
    __syncthreads();
    {  // x_K[c] = sum_c' Y_K(c', c) w[c'] (column c of Y_K is contiguous): warp per 8 c
      const float4 w4 = reinterpret_cast<const float4 *>(wv)[lane];
      float v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        v[q] = warp_sum(ycol[q].x * w4.x + ycol[q].y * w4.y + ycol[q].z * w4.z + ycol[q].w * w4.w);
      if (lane == 0) {
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (8 * warp + q < mk) __stcg(x + k0 + 8 * warp + q, v[q]);
        __threadfence();
      }
    }
    __syncthreads();
    if (tid == 0) st_release_u32(sy.flags + K, epoch);
  }
}

constexpr size_t LEAF_SMEM = (size_t)LEAF_ROWS * LEAF_LD * sizeof(float);
constexpr size_t TRSM_SMEM = ((size_t)LEAF_ROWS * (LEAF_LD + TRSM_LD) + 4 * 1024) * sizeof(float);

static int num_sms() {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

struct RecChol {
  vmck_ctx *c;
  cudaStream_t st;
  int32_t *status;
  size_t dsize, hsize;
  int64_t leaf;
  bool own_leaf;
  const float *A0 = nullptr;  // the matrix being factored (leaves sit on its diagonal)
  int64_t lda0 = 0;
  float *dinv = nullptr;      // per 128-row leaf: four 32 x 32 diagonal-block inverses
};

// Inverse store of the leaf whose diagonal block starts at U (a multiple of 128
// rows down the diagonal of R.A0), or nullptr.
static float *leaf_dinv(const RecChol &R, const float *U) {
  if (!R.dinv || !R.A0) return nullptr;
  const int64_t k0 = (U - R.A0) / (R.lda0 + 1);
  return R.dinv + (k0 / LEAF_B) * 4096;
}

// C (n x n, upper) -= A^T A with A (k x n)
static int syrk_rec(RecChol &R, float *C, int64_t ldc, int64_t n, const float *A, int64_t lda,
                    int64_t k) {
  const float mone = -1.0f, one = 1.0f;
  if (n <= R.leaf) {
    VMCK_BLAS(cublasSsyrk(R.c->blas, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_T, (int)n, (int)k, &mone, A,
                          (int)lda, &one, C, (int)ldc));
    return VMCK_OK;
  }
  const int64_t n1 = half_split(n), n2 = n - n1;
  int rc = syrk_rec(R, C, ldc, n1, A, lda, k);
  if (rc) return rc;
  VMCK_BLAS(cublasSgemm(R.c->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)n1, (int)n2, (int)k, &mone, A,
                        (int)lda, A + n1 * lda, (int)lda, &one, C + n1 * ldc, (int)ldc));
  return syrk_rec(R, C + n1 + n1 * ldc, ldc, n2, A + n1 * lda, lda, k);
}

// B (m x nrhs) <- U^-T B, U upper (m x m)
static int trsm_rec(RecChol &R, const float *U, int64_t ldu, int64_t m, float *B, int64_t ldb,
                    int64_t nrhs) {
  const float mone = -1.0f, one = 1.0f;
  if (m <= R.leaf && R.own_leaf) {
    trsm_leaf_kernel<<<(unsigned)((nrhs + TRSM_COLS - 1) / TRSM_COLS), LEAF_THREADS, TRSM_SMEM,
                       R.st>>>(U, ldu, (int)m, B, ldb, nrhs, leaf_dinv(R, U));
    return check_launch("trsm leaf");
  }
  if (m <= R.leaf) {
    VMCK_BLAS(cublasStrsm(R.c->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_T,
                          CUBLAS_DIAG_NON_UNIT, (int)m, (int)nrhs, &one, U, (int)ldu, B, (int)ldb));
    return VMCK_OK;
  }
  const int64_t m1 = half_split(m), m2 = m - m1;
  int rc = trsm_rec(R, U, ldu, m1, B, ldb, nrhs);
  if (rc) return rc;
  VMCK_BLAS(cublasSgemm(R.c->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)m2, (int)nrhs, (int)m1, &mone,
                        U + m1 * ldu, (int)ldu, B, (int)ldb, &one, B + m1, (int)ldb));
  return trsm_rec(R, U + m1 + m1 * ldu, ldu, m2, B + m1, ldb, nrhs);
}

static int chol_rec(RecChol &R, float *A, int64_t lda, int64_t n) {
  if (n <= R.leaf) {
    if (R.own_leaf) {
      potrf_leaf_kernel<<<1, LEAF_THREADS, LEAF_SMEM, R.st>>>(
          A, lda, (int)n, R.status, leaf_dinv(R, A));
      return check_launch("cholesky leaf");
    }
    VMCK_SOLVER(cusolverDnXpotrf(R.c->solver, R.c->params, CUBLAS_FILL_MODE_UPPER, n, CUDA_R_32F,
                                 A, lda, CUDA_R_32F, R.c->dwork, R.dsize, R.c->hwork, R.hsize,
                                 R.c->d_info));
    info_accumulate_kernel<<<1, 1, 0, R.st>>>(R.c->d_info, R.status);
    return check_launch("cholesky leaf info");
  }
  const int64_t n1 = half_split(n), n2 = n - n1;
  int rc = chol_rec(R, A, lda, n1);
  if (rc) return rc;
  if ((rc = trsm_rec(R, A, lda, n1, A + n1 * lda, lda, n2))) return rc;
  if ((rc = syrk_rec(R, A + n1 + n1 * lda, lda, n2, A + n1 * lda, lda, n1))) return rc;
  return chol_rec(R, A + n1 + n1 * lda, lda, n2);
}

// Blocked right-looking upper Cholesky with look-ahead.  Panel q (rows
// [k_q, k_q+1) of the upper factor) is factored on the caller's stream: its
// diagonal block by chol_rec (potrf_leaf_kernel leaves), its row by trsm_rec
// (trsm_leaf_kernel leaves + emulated GEMMs), then the update of the next block
// row by this panel.  The update of every later block row runs on the side
// stream (first the block row q+2 as one GEMM, then column strips of what is
// left), overlapping the next panels' latency-bound factorisation.  Events:
// F[q] (panel q final) orders the side stream's use of it; U[q] (block row q+2
// updated by panel q) orders the caller's update of that row by panel q+1.
// The context's look-ahead streams (chain: highest priority; side: lowest) and
// at least `need` events, created on first use.
static int streams_setup(vmck_ctx *c, int need) {
  if (!c->side) {
    int lo = 0, hi = 0;
    VMCK_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    VMCK_CUDA(cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, lo));
    VMCK_CUDA(cudaStreamCreateWithPriority(&c->chain, cudaStreamNonBlocking, hi));
    VMCK_CUDA(cudaStreamCreateWithPriority(&c->chain2, cudaStreamNonBlocking, hi));
  }
  if (c->n_events < need) {
    cudaEvent_t *ev = static_cast<cudaEvent_t *>(malloc(sizeof(cudaEvent_t) * need));
    if (!ev) return VMCK_ERR_NOMEM;
    for (int i = 0; i < c->n_events; ++i) ev[i] = c->events[i];
    for (int i = c->n_events; i < need; ++i)
      VMCK_CUDA(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
    free(c->events);
    c->events = ev;
    c->n_events = need;
  }
  return VMCK_OK;
}

static int chol_lookahead_setup(vmck_ctx *c, int panels) {
  int rc = streams_setup(c, 2 * panels + 2);
  if (rc) return rc;
  if (!c->blas2) VMCK_BLAS(cublasCreate(&c->blas2));
  VMCK_BLAS(cublasSetStream(c->blas2, c->side));
  VMCK_BLAS(cublasSetMathMode(c->blas2, CUBLAS_FP32_EMULATED_BF16X9_MATH));
  VMCK_BLAS(cublasSetEmulationStrategy(c->blas2, CUBLAS_EMULATION_STRATEGY_EAGER));
  VMCK_BLAS(cublasSetEmulationSpecialValuesSupport(c->blas2,
                                                    CUDA_EMULATION_SPECIAL_VALUES_SUPPORT_NONE));
  return VMCK_OK;
}

static int chol_blocked_on(RecChol &R, float *A, int64_t lda, int64_t n);

// The chain runs on the context's highest-priority stream so that its short,
// latency-bound kernels are scheduled ahead of the side stream's GEMM blocks;
// the caller's stream waits for both at the end.
static int chol_blocked(RecChol &R, float *A, int64_t lda, int64_t n) {
  vmck_ctx *c = R.c;
  const int64_t PANEL_W = chol_panel_width();
  const int panels = (int)((n + PANEL_W - 1) / PANEL_W);
  int rc = chol_lookahead_setup(c, panels);
  if (rc) return rc;
  cudaStream_t caller = R.st;
  cudaEvent_t start = c->events[2 * panels], done = c->events[2 * panels + 1];
  VMCK_CUDA(cudaEventRecord(start, caller));
  VMCK_CUDA(cudaStreamWaitEvent(c->chain, start, 0));
  VMCK_CUDA(cudaStreamWaitEvent(c->side, start, 0));
  VMCK_BLAS(cublasSetStream(c->blas, c->chain));
  R.st = c->chain;
  rc = chol_blocked_on(R, A, lda, n);
  R.st = caller;
  cublasSetStream(c->blas, caller);
  if (rc) return rc;
  VMCK_CUDA(cudaEventRecord(done, c->chain));
  VMCK_CUDA(cudaStreamWaitEvent(caller, done, 0));
  VMCK_CUDA(cudaEventRecord(done, c->side));
  VMCK_CUDA(cudaStreamWaitEvent(caller, done, 0));
  return VMCK_OK;
}

static int chol_blocked_on(RecChol &R, float *A, int64_t lda, int64_t n) {
  const float mone = -1.0f, one = 1.0f;
  vmck_ctx *c = R.c;
  const int64_t PANEL_W = chol_panel_width();
  const int panels = (int)((n + PANEL_W - 1) / PANEL_W);
  int rc = VMCK_OK;
  cudaEvent_t *F = c->events, *U = c->events + panels;
  for (int q = 0; q < panels; ++q) {
    const int64_t k0 = q * PANEL_W, k1 = std::min<int64_t>(n, k0 + PANEL_W), w = k1 - k0;
    const int64_t m = n - k1;
    float *D = A + k0 + k0 * lda;
    if ((rc = chol_rec(R, D, lda, w))) return rc;
    if (m == 0) break;
    float *P = A + k0 + k1 * lda;  // w x m panel row
    if ((rc = trsm_rec(R, D, lda, w, P, lda, m))) return rc;
    VMCK_CUDA(cudaEventRecord(F[q], R.st));
    // caller's stream: block row q+1 (rows [k1, k2), columns [k1, n)) by panel q
    const int64_t k2 = std::min<int64_t>(n, k1 + PANEL_W);
    if (q >= 1) VMCK_CUDA(cudaStreamWaitEvent(R.st, U[q - 1], 0));
    VMCK_BLAS(cublasSgemm(c->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)(k2 - k1), (int)m, (int)w, &mone,
                          P, (int)lda, P, (int)lda, &one, A + k1 + k1 * lda, (int)lda));
    if (k2 == n) continue;
    // side stream: block row q+2, then the rest in column strips
    VMCK_CUDA(cudaStreamWaitEvent(c->side, F[q], 0));
    const int64_t k3 = std::min<int64_t>(n, k2 + PANEL_W);
    VMCK_BLAS(cublasSgemm(c->blas2, CUBLAS_OP_T, CUBLAS_OP_N, (int)(k3 - k2), (int)(n - k2), (int)w,
                          &mone, P + (k2 - k1) * lda, (int)lda, P + (k2 - k1) * lda, (int)lda, &one,
                          A + k2 + k2 * lda, (int)lda));
    VMCK_CUDA(cudaEventRecord(U[q], c->side));
    const float *P3 = P + (k3 - k1) * lda;
    const int64_t m3 = n - k3;
    for (int64_t c0 = 0; c0 < m3; c0 += STRIP_W) {
      const int64_t c1 = std::min<int64_t>(m3, c0 + STRIP_W);
      // C[0:c1, c0:c1] -= P3[:, 0:c1]^T P3[:, c0:c1] (trailing matrix from k3)
      VMCK_BLAS(cublasSgemm(c->blas2, CUBLAS_OP_T, CUBLAS_OP_N, (int)c1, (int)(c1 - c0), (int)w,
                            &mone, P3, (int)lda, P3 + c0 * lda, (int)lda, &one,
                            A + k3 + (k3 + c0) * lda, (int)lda));
    }
  }
  return VMCK_OK;
}

// ------------------------------------------------------------ symmetric residual
// r = b - A x for a symmetric A stored as its lower triangle (row-major), each
// stored element read exactly once.  Tile (I, J), I >= J, of 64 x 64 adds
// A_IJ x_J to the rows of block I (slot J) and A_IJ^T x_I to the rows of block J
// (slot I); on a diagonal tile both go to slot I.  Every (slot, row) of
// ws[n_tiles][n] is written exactly once; the second kernel sums the slots in
// a fixed order.
//
// GB300 issues about 1.4 FP64 instructions per clock per SM, so a plain FP64
// symv is bound by the FP64 pipe (~0.6 ms at n = 16,384 even with two FMAs per
// element) rather than by HBM.  Here each double is split into a (hi, lo) pair
// of floats with integer operations only and the products are accumulated in
// double-float arithmetic (~2^-46 relative per term) on the FP32 pipe, which
// leaves the kernel HBM-bound: n(n+1)/2 * 8 bytes per call.
constexpr int SY_T = 64;
constexpr int SY_LD = SY_T + 1;  // smem row stride (floats): conflict-free rows and columns

__device__ inline void sy_tri_tile(int64_t bid, int64_t &I, int64_t &J) {
  int64_t i = (int64_t)((sqrt(8.0 * (double)bid + 1.0) - 1.0) * 0.5);
  while (i * (i + 1) / 2 > bid) --i;
  while ((i + 1) * (i + 2) / 2 <= bid) ++i;
  I = i;
  J = bid - i * (i + 1) / 2;
}

// hi = the leading 24 significand bits of a, lo = the next 24 (both truncated,
// same sign), from the IEEE bit fields: no FP64 instruction.  |a| < 2^-100
// maps to (0, 0).
__device__ __forceinline__ df32 df_split_bits(double a) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(a);
  const unsigned sign = (unsigned)(bits >> 32) & 0x80000000u;
  const int e = (int)((bits >> 52) & 0x7FF);
  if (e < 1023 - 100) return {0.0f, 0.0f};
  if (e > 1023 + 127) return {__int_as_float(sign | 0x7F800000u), 0.0f};
  const unsigned long long m = bits & ((1ull << 52) - 1);
  const float hi = __uint_as_float(sign | ((unsigned)(e - 1023 + 127) << 23) | (unsigned)(m >> 29));
  const unsigned rem = (unsigned)(m & ((1u << 29) - 1));
  // rem's bit 0 weighs 2^(e - 1075): scale by 2^(e - 1075 + 64) (a normal float for
  // e >= 923), then by 2^-64 so that a subnormal lo rounds instead of vanishing
  const float lo = __uint2float_rz(rem) * __uint_as_float((unsigned)(e - 1075 + 64 + 127) << 23) *
                   __uint_as_float(0x1F800000u);
  return {hi, __uint_as_float(__float_as_uint(lo) | sign)};
}

// acc += a * x for double-float a, x (the lo * lo term is below the pair's precision)
__device__ __forceinline__ df32 df_fma(df32 acc, df32 a, df32 x) {
  df32 p = df_two_prod(a.hi, x.hi);
  p.lo = __fmaf_rn(a.hi, x.lo, __fmaf_rn(a.lo, x.hi, p.lo));
  return df_add(acc, p);
}

__global__ void __launch_bounds__(256) symv_lower_partial_kernel(const double *__restrict__ A,
                                                                 int64_t n,
                                                                 const double *__restrict__ x,
                                                                 double *__restrict__ ws,
                                                                 const int *done) {
  if (refine_done(done)) return;
  __shared__ float ahi[SY_T * SY_LD], alo[SY_T * SY_LD];
  __shared__ df32 xr[SY_T], xc[SY_T];
  __shared__ df32 part[4][SY_T];  // [row half 0, row half 1, col half 0, col half 1]
  int64_t I, J;
  sy_tri_tile(blockIdx.x, I, J);
  const int tid = threadIdx.x;
  const int64_t r0 = I * SY_T, c0 = J * SY_T;
  const bool diag = (I == J);
  if (tid < SY_T) xc[tid] = (c0 + tid < n) ? df_split_bits(x[c0 + tid]) : df32{0.0f, 0.0f};
  else if (tid < 2 * SY_T)
    xr[tid - SY_T] = (r0 + tid - SY_T < n) ? df_split_bits(x[r0 + tid - SY_T]) : df32{0.0f, 0.0f};
  {
    const int c = tid & 63, g = tid >> 6;
    const bool cok = (c0 + c) < n;
#pragma unroll 4
    for (int k = 0; k < 16; ++k) {
      const int r = g + 4 * k;
      df32 v{0.0f, 0.0f};
      if (cok && (r0 + r) < n && (!diag || r >= c)) v = df_split_bits(A[(r0 + r) * n + c0 + c]);
      ahi[r * SY_LD + c] = v.hi;
      alo[r * SY_LD + c] = v.lo;
    }
  }
  __syncthreads();
  // threads 0-127: row sums (row = tid & 63, column half = tid >> 6);
  // threads 128-255: column sums over the strict lower part of a diagonal tile
  const int u = tid & 63, h = (tid >> 6) & 1;
  df32 acc{0.0f, 0.0f};
  if (tid < 128) {
#pragma unroll 8
    for (int i = 0; i < 32; ++i) {
      const int c = 32 * h + i;
      acc = df_fma(acc, df32{ahi[u * SY_LD + c], alo[u * SY_LD + c]}, xc[c]);
    }
  } else {
#pragma unroll 8
    for (int i = 0; i < 32; ++i) {
      const int r = 32 * h + i;
      if (diag && r == u) continue;
      acc = df_fma(acc, df32{ahi[r * SY_LD + u], alo[r * SY_LD + u]}, xr[r]);
    }
  }
  part[tid >> 6][u] = acc;
  __syncthreads();
  if (tid < SY_T) {
    const int r = tid;
    const df32 rs = df_add(part[0][r], part[1][r]);
    const df32 cs = df_add(part[2][r], part[3][r]);
    if (diag) {
      if (r0 + r < n) ws[I * n + r0 + r] = df_to_double(df_add(rs, cs));
    } else {
      if (r0 + r < n) ws[J * n + r0 + r] = df_to_double(rs);
      if (c0 + r < n) ws[I * n + c0 + r] = df_to_double(cs);
    }
  }
}

__global__ void symv_residual_reduce_kernel(const double *__restrict__ ws, int64_t n, int nt,
                                            const double *__restrict__ b, double *__restrict__ r,
                                            const int *done) {
  if (refine_done(done)) return;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int k = 0; k < nt; ++k) s += ws[k * n + i];
  r[i] = b[i] - s;
}

// The same tiling in plain FP64 arithmetic (FP64-pipe-bound): the residual of
// the all-FP64 solve, whose accuracy must match a direct FP64 factorisation.
__global__ void __launch_bounds__(256) symv_lower_partial_f64_kernel(
    const double *__restrict__ A, int64_t n, const double *__restrict__ x,
    double *__restrict__ ws, const int *done) {
  if (refine_done(done)) return;
  __shared__ double as[SY_T * SY_LD];
  __shared__ double xr[SY_T], xc[SY_T];
  __shared__ double part[4][SY_T];
  int64_t I, J;
  sy_tri_tile(blockIdx.x, I, J);
  const int tid = threadIdx.x;
  const int64_t r0 = I * SY_T, c0 = J * SY_T;
  const bool diag = (I == J);
  if (tid < SY_T) xc[tid] = (c0 + tid < n) ? x[c0 + tid] : 0.0;
  else if (tid < 2 * SY_T) xr[tid - SY_T] = (r0 + tid - SY_T < n) ? x[r0 + tid - SY_T] : 0.0;
  {
    const int c = tid & 63, g = tid >> 6;
    const bool cok = (c0 + c) < n;
#pragma unroll 4
    for (int k = 0; k < 16; ++k) {
      const int r = g + 4 * k;
      double v = 0.0;
      if (cok && (r0 + r) < n && (!diag || r >= c)) v = A[(r0 + r) * n + c0 + c];
      as[r * SY_LD + c] = v;
    }
  }
  __syncthreads();
  const int u = tid & 63, h = (tid >> 6) & 1;
  double acc = 0.0;
  if (tid < 128) {
#pragma unroll 8
    for (int i = 0; i < 32; ++i) {
      const int c = 32 * h + i;
      acc = fma(as[u * SY_LD + c], xc[c], acc);
    }
  } else {
#pragma unroll 8
    for (int i = 0; i < 32; ++i) {
      const int r = 32 * h + i;
      if (diag && r == u) continue;
      acc = fma(as[r * SY_LD + u], xr[r], acc);
    }
  }
  part[tid >> 6][u] = acc;
  __syncthreads();
  if (tid < SY_T) {
    const int r = tid;
    const double rs = part[0][r] + part[1][r];
    const double cs = part[2][r] + part[3][r];
    if (diag) {
      if (r0 + r < n) ws[I * n + r0 + r] = rs + cs;
    } else {
      if (r0 + r < n) ws[J * n + r0 + r] = rs;
      if (c0 + r < n) ws[I * n + c0 + r] = cs;
    }
  }
}

static int symv_residual(cudaStream_t st, const double *A, int64_t n, const double *x,
                         const double *b, double *r, double *ws, const int *done,
                         bool exact = false) {
  const int64_t nt = (n + SY_T - 1) / SY_T;
  if (exact)
    symv_lower_partial_f64_kernel<<<(unsigned)(nt * (nt + 1) / 2), 256, 0, st>>>(A, n, x, ws,
                                                                                 done);
  else
    symv_lower_partial_kernel<<<(unsigned)(nt * (nt + 1) / 2), 256, 0, st>>>(A, n, x, ws, done);
  int rc = check_launch("symv partial");
  if (rc) return rc;
  symv_residual_reduce_kernel<<<ceil_div(n, 256), 256, 0, st>>>(ws, n, (int)nt, b, r, done);
  return check_launch("symv reduce");
}

// norms[0] = ||r||, norms[1] = ||b|| (FP64, one block, fixed reduction order).
__global__ void __launch_bounds__(256) norms_kernel(const double *__restrict__ r,
                                                    const double *__restrict__ b, int64_t n,
                                                    double *norms) {
  __shared__ double red[2][8];
  double sr = 0.0, sb = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    sr = fma(r[i], r[i], sr);
    sb = fma(b[i], b[i], sb);
  }
  sr = warp_sum(sr);
  sb = warp_sum(sb);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][w] = sr;
    red[1][w] = sb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tr = 0.0, tb = 0.0;
    for (int k = 0; k < 8; ++k) {
      tr += red[0][k];
      tb += red[1][k];
    }
    norms[0] = sqrt(tr);
    norms[1] = sqrt(tb);
  }
}


}  // namespace vmck

using namespace vmck;

extern "C" int vmck_ctx_create(vmck_ctx **out) {
  VMCK_REQUIRE(out, "ctx out pointer");
  vmck_ctx *c = new vmck_ctx();
  cudaGetDevice(&c->device);
  if (cublasCreate(&c->blas) != CUBLAS_STATUS_SUCCESS ||
      cusolverDnCreate(&c->solver) != CUSOLVER_STATUS_SUCCESS ||
      cusolverDnCreateParams(&c->params) != CUSOLVER_STATUS_SUCCESS ||
      cudaMalloc(&c->d_info, sizeof(int)) != cudaSuccess) {
    set_last_error("vmck_ctx_create: cuBLAS / cuSOLVER initialisation failed");
    vmck_ctx_destroy(c);
    return VMCK_ERR_LIBRARY;
  }
  *out = c;
  return VMCK_OK;
}

extern "C" int vmck_ctx_destroy(vmck_ctx *c) {
  if (!c) return VMCK_OK;
  cudaDeviceSynchronize();
  for (int i = 0; i < c->n_events; ++i) cudaEventDestroy(c->events[i]);
  free(c->events);
  if (c->blas2) cublasDestroy(c->blas2);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->chain) cudaStreamDestroy(c->chain);
  if (c->chain2) cudaStreamDestroy(c->chain2);
  if (c->params) cusolverDnDestroyParams(c->params);
  if (c->solver) cusolverDnDestroy(c->solver);
  if (c->blas) cublasDestroy(c->blas);
  cudaFree(c->dwork);
  cudaFree(c->aux);
  cudaFree(c->tcws);
  cudaFree(c->d_attempt);
  cudaFree(c->d_info);
  free(c->hwork);
  delete c;
  return VMCK_OK;
}

namespace vmck {

__global__ void pad_identity_kernel(float *F, int64_t n, int64_t np) {
  for (int64_t i = n + threadIdx.x; i < np; i += blockDim.x) F[i + i * np] = 1.0f;
}

__global__ void refine_init_kernel(double *norms, double *prev, int *done) {
  if (threadIdx.x == 0) {
    norms[0] = norms[1] = 0.0;
    *prev = 1e300;
    *done = 0;
  }
}

struct RefineOpts {
  int max_iter;
  double stop_tol;   // stop once ||r|| <= stop_tol ||b||
  double fail_tol;   // VMCK_DEV_NO_CONVERGE if the final ||r|| > fail_tol ||b||
  int factor_mode;
  bool exact;        // FP64 residual (else double-float, ~2^-46 per term)
  bool stagnation;   // also stop when the residual stops falling
  bool pcg = false;  // flexible PCG with the factor as preconditioner (factor_mode 4)
  bool *factor_failed = nullptr;  // pcg: set when the factor failed (no iteration ran)
};

// FP32 factor of A32 (overwritten) + iterative refinement against A64.
static int refined_solve(vmck_ctx *c, cudaStream_t st, const double *A64, float *A32,
                         const double *b, double *x, int64_t n, const RefineOpts &o,
                         int32_t *status, double *residual_out) {
  const int factor_mode = o.factor_mode;
  int rc = VMCK_OK;
  size_t dsize = 0, hsize = 0;
  if (factor_mode <= 3) {
    if ((rc = bind(c, st))) return rc;
    const bool emulate = factor_mode != 0;
    VMCK_SOLVER(cusolverDnSetMathMode(c->solver, emulate ? CUSOLVER_FP32_EMULATED_BF16X9_MATH
                                                         : CUSOLVER_DEFAULT_MATH));
    if (emulate)
      VMCK_SOLVER(cusolverDnSetEmulationStrategy(c->solver, CUDA_EMULATION_STRATEGY_EAGER));
    const int64_t fn = factor_mode == 2 ? std::min<int64_t>(n, CHOL_LEAF) : n;
    VMCK_SOLVER(cusolverDnXpotrf_bufferSize(c->solver, c->params, CUBLAS_FILL_MODE_UPPER, fn,
                                            CUDA_R_32F, A32, n, CUDA_R_32F, &dsize, &hsize));
    if ((rc = grow(&c->dwork, &c->dwork_bytes, dsize + 256, st))) return rc;
    if ((rc = grow_host(c, hsize))) return rc;
  }
  // the triangular solves run on the factor F (ld np); mode 4 pads n to a
  // multiple of 4 (identity rows) for their vector loads
  const int64_t np = factor_mode == 4 ? ((n + 3) & ~int64_t(3)) : n;
  const bool own_trsv = (factor_mode == 3 && n % 4 == 0) || factor_mode == 4;
  // aux: r (n double), r32 (np float), two norms + done + prev, symv slots
  // (n_tiles x n double), inverse diagonal blocks (mode 3), y32 (np float), flags
  // and tickets (2 nb + 4 uint), leaf inverses (mode 3)
  const int64_t nt = (n + SY_T - 1) / SY_T;
  const int64_t nb = (np + TB - 1) / TB;
  const size_t r32_off = ((size_t)n * 8 + 255) & ~size_t(255);
  const size_t norms_off = (r32_off + (size_t)np * 4 + 255) & ~size_t(255);
  const size_t ws_off = norms_off + 256;
  const size_t yinv_off = (ws_off + (size_t)nt * n * 8 + 255) & ~size_t(255);
  const size_t y32_off =
      (yinv_off + (factor_mode == 3 && own_trsv ? (size_t)nb * TB * TB * 4 : 0) + 255) &
      ~size_t(255);
  const size_t sync_off = (y32_off + (own_trsv ? (size_t)np * 4 : 0) + 255) & ~size_t(255);
  const size_t dinv_off = (sync_off + (own_trsv ? (size_t)(2 * nb + 4) * 4 : 0) + 255) & ~size_t(255);
  const size_t pcg_off = (dinv_off + (factor_mode == 3 ? (size_t)nb * 4096 * 4 : 0) + 255) &
                        ~size_t(255);
  const size_t vec_bytes = ((size_t)n * 8 + 255) & ~size_t(255);
  const size_t need = pcg_off + (o.pcg ? 4 * vec_bytes + 256 : 0);
  if ((rc = grow(&c->aux, &c->aux_bytes, need, st))) return rc;
  char *aux = static_cast<char *>(c->aux);
  double *r = static_cast<double *>(c->aux);
  float *r32 = reinterpret_cast<float *>(aux + r32_off);
  double *norms = reinterpret_cast<double *>(aux + norms_off);
  double *prev = norms + 2;
  int *done = reinterpret_cast<int *>(norms + 3);
  double *sws = reinterpret_cast<double *>(aux + ws_off);
  float *yinv = reinterpret_cast<float *>(aux + yinv_off);
  float *y32 = reinterpret_cast<float *>(aux + y32_off);
  unsigned *sync = reinterpret_cast<unsigned *>(aux + sync_off);
  const TrsvSync sync_f{sync, sync + 2 * nb, sync + 2 * nb + 2, wait_limit_ns()};
  const TrsvSync sync_b{sync + nb, sync + 2 * nb + 1, sync + 2 * nb + 2, wait_limit_ns()};
  float *F = A32;  // the factor the solves read
  if (factor_mode == 4) {
    const size_t pad_bytes = np != n ? (size_t)np * np * 4 : 0;
    const size_t tc_off = (pad_bytes + 1023) & ~size_t(1023);
    if ((rc = grow(&c->tcws, &c->tcws_bytes, tc_off + (size_t)chol_tc_workspace_bytes(np), st)))
      return rc;
    if (np != n) {
      F = static_cast<float *>(c->tcws);
      VMCK_CUDA(cudaMemsetAsync(F, 0, pad_bytes, st));
      VMCK_CUDA(cudaMemcpy2DAsync(F, np * 4, A32, n * 4, n * 4, n, cudaMemcpyDeviceToDevice, st));
      pad_identity_kernel<<<1, 32, 0, st>>>(F, n, np);
      if ((rc = check_launch("refined solve padding"))) return rc;
    }
    if ((rc = streams_setup(c, chol_events_needed(np)))) return rc;
    const CholStreams ls{c->chain, c->side, c->events, c->n_events, c->chain2};
    rc = chol_tc_factor(st, F, np, static_cast<char *>(c->tcws) + tc_off, status, &yinv, &ls);
    if (rc) return rc;
    if (np != n)
      VMCK_CUDA(cudaMemcpy2DAsync(A32, n * 4, F, np * 4, n * 4, n, cudaMemcpyDeviceToDevice, st));
    VMCK_CUDA(cudaMemsetAsync(c->d_info, 0, sizeof(int), st));
    VMCK_CUDA(cudaMemsetAsync(sync, 0, (size_t)(2 * nb + 4) * 4, st));
  } else if (factor_mode >= 2) {
    VMCK_BLAS(cublasSetMathMode(c->blas, CUBLAS_FP32_EMULATED_BF16X9_MATH));
    VMCK_BLAS(cublasSetEmulationStrategy(c->blas, CUBLAS_EMULATION_STRATEGY_EAGER));
    if (factor_mode == 2) {
      RecChol R{c, st, status, dsize, hsize, CHOL_LEAF, false};
      rc = chol_rec(R, A32, n, n);
    } else {
      VMCK_CUDA(cudaFuncSetAttribute(potrf_leaf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)LEAF_SMEM));
      VMCK_CUDA(cudaFuncSetAttribute(trsm_leaf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)TRSM_SMEM));
      // finite inputs: a NaN or Inf in A32 still ends as a failed pivot or an
      // unconverged refinement, both reported in the status word
      VMCK_BLAS(cublasSetEmulationSpecialValuesSupport(c->blas,
                                                        CUDA_EMULATION_SPECIAL_VALUES_SUPPORT_NONE));
      RecChol R{c, st, status, dsize, hsize, LEAF_B, true};
      R.A0 = A32;
      R.lda0 = n;
      R.dinv = reinterpret_cast<float *>(aux + dinv_off);
      rc = chol_blocked(R, A32, n, n);
      cublasSetEmulationSpecialValuesSupport(c->blas, CUDA_EMULATION_SPECIAL_VALUES_SUPPORT_DEFAULT);
    }
    cublasSetMathMode(c->blas, CUBLAS_DEFAULT_MATH);
    cusolverDnSetMathMode(c->solver, CUSOLVER_DEFAULT_MATH);
    if (rc) return rc;
    if (factor_mode == 3) VMCK_CUDA(cudaMemsetAsync(c->d_info, 0, sizeof(int), st));
    if (own_trsv) {
      VMCK_CUDA(cudaFuncSetAttribute(trsv_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)TRSM_SMEM));
      trsv_inv_kernel<<<dim3(2, (unsigned)nb), LEAF_THREADS, TRSM_SMEM, st>>>(A32, n, yinv);
      if ((rc = check_launch("refined solve inverse blocks"))) return rc;
      VMCK_CUDA(cudaMemsetAsync(sync, 0, (size_t)(2 * nb + 4) * 4, st));
    }
  } else {
    cusolverStatus_t fs = cusolverDnXpotrf(c->solver, c->params, CUBLAS_FILL_MODE_UPPER, n,
                                           CUDA_R_32F, A32, n, CUDA_R_32F, c->dwork, dsize,
                                           c->hwork, hsize, c->d_info);
    cusolverDnSetMathMode(c->solver, CUSOLVER_DEFAULT_MATH);
    if (fs != CUSOLVER_STATUS_SUCCESS) {
      set_last_error("refined solve: cusolverDnXpotrf status %d", (int)fs);
      return VMCK_ERR_LIBRARY;
    }
    info_accumulate_kernel<<<1, 1, 0, st>>>(c->d_info, status);
    if ((rc = check_launch("refined solve info"))) return rc;
  }
  if (o.pcg) {
    VMCK_REQUIRE(own_trsv, "the PCG fallback runs on the tensor-core factor (factor_mode 4)");
    // a failed factor is reported before any iteration: the caller retries with
    // a larger shift
    int32_t fstat = 0;
    VMCK_CUDA(cudaMemcpyAsync(&fstat, status, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    VMCK_CUDA(cudaStreamSynchronize(st));
    if (fstat & (VMCK_DEV_NOT_SPD | VMCK_DEV_NONFINITE | VMCK_DEV_TIMEOUT)) {
      if (o.factor_failed) *o.factor_failed = !(fstat & VMCK_DEV_TIMEOUT);
      return VMCK_OK;
    }
    double *z = reinterpret_cast<double *>(aux + pcg_off);
    double *p = reinterpret_cast<double *>(aux + pcg_off + vec_bytes);
    double *qn = reinterpret_cast<double *>(aux + pcg_off + 2 * vec_bytes);
    double *zero = reinterpret_cast<double *>(aux + pcg_off + 3 * vec_bytes);
    double *sc = reinterpret_cast<double *>(aux + pcg_off + 4 * vec_bytes);
    const int blocks = ceil_div(n, 256);
    const unsigned grid = (unsigned)std::min<int64_t>(nb, 2 * (int64_t)num_sms());
    VMCK_CUDA(cudaMemsetAsync(x, 0, (size_t)n * 8, st));
    VMCK_CUDA(cudaMemsetAsync(zero, 0, (size_t)n * 8, st));
    VMCK_CUDA(cudaMemcpyAsync(r, b, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
    refine_init_kernel<<<1, 32, 0, st>>>(norms, prev, done);
    if ((rc = check_launch("pcg init"))) return rc;
    if (np != n) VMCK_CUDA(cudaMemsetAsync(r32, 0, (size_t)np * 4, st));
    unsigned epoch = 0;
    // z = M^-1 r: the two triangular solves on the factor of A32
    auto precondition = [&]() -> int {
      int e;
      d2f_kernel<<<blocks, 256, 0, st>>>(r, r32, n, done);
      if ((e = check_launch("pcg cast"))) return e;
      ++epoch;
      VMCK_CUDA(cudaMemsetAsync(sync + 2 * nb, 0, 2 * sizeof(unsigned), st));  // tickets
      trsv_fwd_kernel<<<grid, LEAF_THREADS, 0, st>>>(F, np, yinv, r32, y32, sync_f, epoch,
                                                     status, done);
      if ((e = check_launch("pcg forward"))) return e;
      trsv_bwd_kernel<<<grid, LEAF_THREADS, 0, st>>>(F, np, yinv, y32, r32, sync_b, epoch,
                                                     status, done);
      if ((e = check_launch("pcg backward"))) return e;
      f2d_copy_kernel<<<blocks, 256, 0, st>>>(r32, z, n, done);
      return check_launch("pcg z");
    };
    if ((rc = precondition())) return rc;
    VMCK_CUDA(cudaMemcpyAsync(p, z, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
    pcg_start_kernel<<<1, 1024, 0, st>>>(r, z, n, sc);
    if ((rc = check_launch("pcg start"))) return rc;
    for (int it = 0; it < o.max_iter; ++it) {
      if ((rc = symv_residual(st, A64, n, p, zero, qn, sws, done, o.exact))) return rc;
      pcg_alpha_kernel<<<1, 1024, 0, st>>>(p, qn, n, sc, status, done);
      if ((rc = check_launch("pcg alpha"))) return rc;
      pcg_update_kernel<<<blocks, 256, 0, st>>>(x, r, p, qn, n, sc, done);
      if ((rc = check_launch("pcg update"))) return rc;
      // every 32nd iteration the recursive residual is replaced by the true
      // b - A x (FP64 rounding makes them drift apart), and the loop also stops
      // once that has not halved since the last replacement: its FP64 floor
      // ~eps ||A|| ||x||
      const bool replace = (it & 31) == 31;
      if (replace && (rc = symv_residual(st, A64, n, x, b, r, sws, done, o.exact))) return rc;
      refine_converged_kernel<<<1, 256, 0, st>>>(r, b, n, o.stop_tol, done,
                                                 replace ? prev : nullptr);
      if ((rc = check_launch("pcg convergence"))) return rc;
      if ((rc = precondition())) return rc;
      pcg_beta_kernel<<<1, 1024, 0, st>>>(r, z, qn, n, sc, done);
      if ((rc = check_launch("pcg beta"))) return rc;
      pcg_direction_kernel<<<blocks, 256, 0, st>>>(p, z, n, sc, done);
      if ((rc = check_launch("pcg direction"))) return rc;
      if ((it & 31) == 31) {  // stop enqueueing once the device has converged
        int h_done = 0;
        VMCK_CUDA(cudaMemcpyAsync(&h_done, done, sizeof(int), cudaMemcpyDeviceToHost, st));
        VMCK_CUDA(cudaStreamSynchronize(st));
        if (h_done) break;
      }
    }
    // the true residual b - A x (the recursive one drifts)
    VMCK_CUDA(cudaMemsetAsync(done, 0, sizeof(int), st));
    if ((rc = symv_residual(st, A64, n, x, b, r, sws, done, o.exact))) return rc;
    norms_kernel<<<1, 256, 0, st>>>(r, b, n, norms);
    if ((rc = check_launch("pcg norms"))) return rc;
    refine_check_kernel<<<1, 1, 0, st>>>(norms, norms + 1, c->d_info, o.fail_tol, status,
                                         residual_out);
    return check_launch("pcg check");
  }
  VMCK_CUDA(cudaMemsetAsync(x, 0, (size_t)n * 8, st));
  refine_init_kernel<<<1, 32, 0, st>>>(norms, prev, done);  // norms 0, prev huge, done 0
  if ((rc = check_launch("refined solve init"))) return rc;
  if (np != n) VMCK_CUDA(cudaMemsetAsync(r32, 0, (size_t)np * 4, st));
  const int blocks = ceil_div(n, 256);
  // Iteration it > 0 first forms r = b - A x and stops the loop (on the device)
  // once it is small enough; the kernels after that return at entry.
  for (int it = 0; it < o.max_iter; ++it) {
    if (it == 0) {
      VMCK_CUDA(cudaMemcpyAsync(r, b, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
    } else {
      if ((rc = symv_residual(st, A64, n, x, b, r, sws, done, o.exact))) return rc;
      refine_converged_kernel<<<1, 256, 0, st>>>(r, b, n, o.stop_tol, done,
                                                 o.stagnation ? prev : nullptr);
      if ((rc = check_launch("refined solve convergence"))) return rc;
    }
    d2f_kernel<<<blocks, 256, 0, st>>>(r, r32, n, done);
    if ((rc = check_launch("refined solve cast"))) return rc;
    if (own_trsv) {
      const unsigned grid = (unsigned)std::min<int64_t>(nb, 2 * (int64_t)num_sms());
      VMCK_CUDA(cudaMemsetAsync(sync + 2 * nb, 0, 2 * sizeof(unsigned), st));  // tickets
      trsv_fwd_kernel<<<grid, LEAF_THREADS, 0, st>>>(F, np, yinv, r32, y32, sync_f,
                                                     (unsigned)(it + 1), status, done);
      if ((rc = check_launch("refined solve forward"))) return rc;
      trsv_bwd_kernel<<<grid, LEAF_THREADS, 0, st>>>(F, np, yinv, y32, r32, sync_b,
                                                     (unsigned)(it + 1), status, done);
      if ((rc = check_launch("refined solve backward"))) return rc;
    } else {
      VMCK_SOLVER(cusolverDnXpotrs(c->solver, c->params, CUBLAS_FILL_MODE_UPPER, n, 1, CUDA_R_32F,
                                   A32, n, CUDA_R_32F, r32, n, c->d_info));
    }
    axpy_f2d_kernel<<<blocks, 256, 0, st>>>(x, r32, n, done);
    if ((rc = check_launch("refined solve update"))) return rc;
  }
  // the final residual (skipped when the loop stopped early: r already belongs to x)
  if ((rc = symv_residual(st, A64, n, x, b, r, sws, done, o.exact))) return rc;
  norms_kernel<<<1, 256, 0, st>>>(r, b, n, norms);
  if ((rc = check_launch("refined solve norms"))) return rc;
  refine_check_kernel<<<1, 1, 0, st>>>(norms, norms + 1, c->d_info, o.fail_tol, status,
                                       residual_out);
  return check_launch("refined solve");
}

}  // namespace vmck

__global__ void lower_f64_to_f32_kernel(const double *__restrict__ A, float *__restrict__ F,
                                        int64_t n) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= n * n) return;
  const int64_t i = e / n, j = e - i * n;
  F[e] = j <= i ? (float)A[e] : 0.0f;
}

extern "C" int vmck_cholesky_solve(vmck_ctx *c, vmck_stream s, int32_t dtype, const void *A,
                                   const void *b, void *x, int64_t n, int32_t *status) {
  VMCK_REQUIRE(c && A && b && x && n > 0, "cholesky_solve arguments");
  VMCK_REQUIRE(dtype == VMCK_F64 || dtype == VMCK_F32, "cholesky_solve dtype");
  cudaStream_t st = as_stream(s);
  int rc;
  if (dtype == VMCK_F64) {
    // FP32 tensor-core factor of fp32(A), then refinement with the FP64 residual
    // b - A x until it stops falling (its FP64 rounding floor): the solution of
    // a direct FP64 factorisation, to FP64 rounding.  A factor that fails or a
    // refinement that does not converge (cond(A) beyond ~1e6) is reported.
    VMCK_REQUIRE(n < (1ll << 30), "cholesky_solve size");
    const size_t fbytes = ((size_t)n * n * 4 + 255) & ~size_t(255);
    if ((rc = grow(&c->dwork, &c->dwork_bytes, fbytes, st))) return rc;
    float *F = static_cast<float *>(c->dwork);
    lower_f64_to_f32_kernel<<<ceil_div(n * n, 256), 256, 0, st>>>(static_cast<const double *>(A),
                                                                    F, n);
    if ((rc = check_launch("cholesky_solve cast"))) return rc;
    const RefineOpts o{30, 0.0, 1e-10, 4, true, true};
    if ((rc = refined_solve(c, st, static_cast<const double *>(A), F, static_cast<const double *>(b),
                            static_cast<double *>(x), n, o, status, nullptr)))
      return rc;
    solve_check_kernel<double><<<1, 1024, 0, st>>>(c->d_info, static_cast<const double *>(x),
                                                   static_cast<const double *>(b), n, status);
    return check_launch("cholesky_solve check");
  }
  // FP32: cuSOLVER SPOTRF / SPOTRS (the plain FP32 path the benchmark compares against)
  if ((rc = bind(c, st))) return rc;
  size_t dsize = 0, hsize = 0;
  VMCK_SOLVER(cusolverDnXpotrf_bufferSize(c->solver, c->params, CUBLAS_FILL_MODE_UPPER, n,
                                          CUDA_R_32F, A, n, CUDA_R_32F, &dsize, &hsize));
  const size_t fbytes = (size_t)n * n * 4;
  const size_t off = (fbytes + 255) & ~size_t(255);
  if ((rc = grow(&c->dwork, &c->dwork_bytes, off + dsize + 256, st))) return rc;
  if ((rc = grow_host(c, hsize))) return rc;
  void *Fm = c->dwork;
  void *work = static_cast<char *>(c->dwork) + off;
  VMCK_CUDA(cudaMemcpyAsync(Fm, A, fbytes, cudaMemcpyDeviceToDevice, st));
  VMCK_CUDA(cudaMemcpyAsync(x, b, (size_t)n * 4, cudaMemcpyDeviceToDevice, st));
  VMCK_SOLVER(cusolverDnXpotrf(c->solver, c->params, CUBLAS_FILL_MODE_UPPER, n, CUDA_R_32F, Fm, n,
                               CUDA_R_32F, work, dsize, c->hwork, hsize, c->d_info));
  VMCK_SOLVER(cusolverDnXpotrs(c->solver, c->params, CUBLAS_FILL_MODE_UPPER, n, 1, CUDA_R_32F, Fm,
                               n, CUDA_R_32F, x, n, c->d_info));
  solve_check_kernel<float><<<1, 1024, 0, st>>>(c->d_info, static_cast<const float *>(x),
                                                static_cast<const float *>(b), n, status);
  return check_launch("cholesky_solve check");
}


extern "C" int vmck_cholesky_solve_refined(vmck_ctx *c, vmck_stream s, const double *A64,
                                           float *A32, const double *b, double *x, int64_t n,
                                           int32_t max_iter, double tol, int32_t factor_mode,
                                           int32_t *status, double *residual_out) {
  VMCK_REQUIRE(c && A64 && A32 && b && x && n > 0 && max_iter >= 1, "refined solve arguments");
  VMCK_REQUIRE(factor_mode >= 0 && factor_mode <= 4, "factor_mode must be 0 - 4");
  VMCK_REQUIRE(n < (1ll << 30), "refined solve size");
  const RefineOpts o{max_iter, tol, tol, factor_mode, false, false};
  return refined_solve(c, as_stream(s), A64, A32, b, x, n, o, status, residual_out);
}

extern "C" int vmck_cholesky_solve_pcg(vmck_ctx *c, vmck_stream s, const double *A64,
                                       float *A32, const double *b, double *x, int64_t n,
                                       int32_t max_iter, double tol, double shift_rel,
                                       int32_t *status, double *residual_out,
                                       double *shift_out) {
  VMCK_REQUIRE(c && A64 && b && x && status && n > 0 && max_iter >= 1 && shift_rel > 0.0,
               "pcg solve arguments");
  VMCK_REQUIRE(n < (1ll << 30), "pcg solve size");
  cudaStream_t st = as_stream(s);
  int rc;
  float *F = A32;
  if (!F) {
    const size_t fbytes = ((size_t)n * n * 4 + 255) & ~size_t(255);
    if ((rc = grow(&c->dwork, &c->dwork_bytes, fbytes, st))) return rc;
    F = static_cast<float *>(c->dwork);
  }
  if (!c->d_attempt && cudaMalloc(&c->d_attempt, 16) != cudaSuccess) {
    set_last_error("pcg solve: status word allocation failed");
    return VMCK_ERR_NOMEM;
  }
  double *d_trace = reinterpret_cast<double *>(c->d_attempt + 2);
  trace_kernel<<<1, 1024, 0, st>>>(A64, n, d_trace);
  if ((rc = check_launch("pcg trace"))) return rc;
  double trace = 0.0;
  VMCK_CUDA(cudaMemcpyAsync(&trace, d_trace, sizeof(double), cudaMemcpyDeviceToHost, st));
  VMCK_CUDA(cudaStreamSynchronize(st));
  if (!(std::isfinite(trace) && trace > 0.0)) {  // not SPD, or not finite: no attempt
    const int32_t bits = std::isfinite(trace) ? VMCK_DEV_NOT_SPD : VMCK_DEV_NONFINITE;
    VMCK_CUDA(cudaMemcpyAsync(c->d_attempt, &bits, sizeof(bits), cudaMemcpyHostToDevice, st));
    VMCK_CUDA(cudaStreamSynchronize(st));
    status_or_kernel<<<1, 1, 0, st>>>(status, c->d_attempt);
    return check_launch("pcg status");
  }
  double mu = shift_rel * trace;
  RefineOpts o{max_iter, tol, tol, 4, true, false};
  o.pcg = true;
  bool failed = false;
  o.factor_failed = &failed;
  for (int attempt = 0; attempt < 6; ++attempt, mu *= 16.0) {
    failed = false;
    lower_f64_to_f32_kernel<<<ceil_div(n * n, 256), 256, 0, st>>>(A64, F, n);
    if ((rc = check_launch("pcg cast"))) return rc;
    add_diag_kernel<<<ceil_div(n, 256), 256, 0, st>>>(F, VMCK_F32, n, mu);
    if ((rc = check_launch("pcg shift"))) return rc;
    VMCK_CUDA(cudaMemsetAsync(c->d_attempt, 0, sizeof(int32_t), st));
    if ((rc = refined_solve(c, st, A64, F, b, x, n, o, c->d_attempt, residual_out))) return rc;
    // the factor of A + mu I failed (mu below its rounding error): a larger
    // shift.  (CG meeting non-positive curvature -- A itself not positive
    // definite -- also reports NOT_SPD, after a successful factor: no retry.)
    if (!(failed && attempt < 5)) break;
  }
  if (shift_out) *shift_out = mu;
  status_or_kernel<<<1, 1, 0, st>>>(status, c->d_attempt);
  return check_launch("pcg status");
}

extern "C" int vmck_pinv_smooth_solve(vmck_ctx *c, vmck_stream s, const double *A, const double *b,
                                      double *x, int64_t n, double rtol, double rtol_smooth) {
  VMCK_REQUIRE(c && A && b && x && n > 0, "pinv_smooth arguments");
  cudaStream_t st = as_stream(s);
  int rc = bind(c, st);
  if (rc) return rc;
  const size_t fbytes = (size_t)n * n * 8;
  const size_t off = (fbytes + 255) & ~size_t(255);
  // aux: eigenvalues w (n), y (n)
  if ((rc = grow(&c->aux, &c->aux_bytes, (size_t)n * 16 + 64, st))) return rc;
  double *w = static_cast<double *>(c->aux);
  double *y = w + n;
  size_t dsize = 0, hsize = 0;
  VMCK_SOLVER(cusolverDnXsyevd_bufferSize(c->solver, c->params, CUSOLVER_EIG_MODE_VECTOR,
                                          CUBLAS_FILL_MODE_UPPER, n, CUDA_R_64F, A, n, CUDA_R_64F,
                                          w, CUDA_R_64F, &dsize, &hsize));
  if ((rc = grow(&c->dwork, &c->dwork_bytes, off + dsize + 256, st))) return rc;
  if ((rc = grow_host(c, hsize))) return rc;
  double *U = static_cast<double *>(c->dwork);
  void *work = static_cast<char *>(c->dwork) + off;
  VMCK_CUDA(cudaMemcpyAsync(U, A, fbytes, cudaMemcpyDeviceToDevice, st));
  VMCK_SOLVER(cusolverDnXsyevd(c->solver, c->params, CUSOLVER_EIG_MODE_VECTOR,
                               CUBLAS_FILL_MODE_UPPER, n, CUDA_R_64F, U, n, CUDA_R_64F, w,
                               CUDA_R_64F, work, dsize, c->hwork, hsize, c->d_info));
  const double one = 1.0, zero = 0.0;
  VMCK_BLAS(cublasDgemv(c->blas, CUBLAS_OP_T, (int)n, (int)n, &one, U, (int)n, b, 1, &zero, y, 1));
  pinv_filter_kernel<<<ceil_div(n, 256), 256, 0, st>>>(w, y, n, rtol, rtol_smooth);
  if ((rc = check_launch("pinv_smooth filter"))) return rc;
  VMCK_BLAS(cublasDgemv(c->blas, CUBLAS_OP_N, (int)n, (int)n, &one, U, (int)n, y, 1, &zero, x, 1));
  return VMCK_OK;
}

extern "C" int vmck_gram_dense(vmck_ctx *c, vmck_stream s, int32_t dtype, const void *O_L,
                               int64_t rows, int64_t cols, int32_t transpose, double diag_shift,
                               void *out) {
  VMCK_REQUIRE(c && O_L && out && rows > 0 && cols > 0, "gram_dense arguments");
  VMCK_REQUIRE(rows < (1ll << 31) && cols < (1ll << 31), "gram_dense sizes");
  cudaStream_t st = as_stream(s);
  int rc = bind(c, st);
  if (rc) return rc;
  // O_L row-major (rows, cols) == column-major X (cols x rows), ld = cols
  const int64_t m = transpose ? cols : rows;
  const cublasOperation_t op = transpose ? CUBLAS_OP_N : CUBLAS_OP_T;
  const int k = (int)(transpose ? rows : cols);
  if (dtype == VMCK_F64) {
    const double one = 1.0, zero = 0.0;
    VMCK_BLAS(cublasDsyrk(c->blas, CUBLAS_FILL_MODE_UPPER, op, (int)m, k, &one,
                          static_cast<const double *>(O_L), (int)cols, &zero,
                          static_cast<double *>(out), (int)m));
  } else if (dtype == VMCK_F32) {
    const float one = 1.0f, zero = 0.0f;
    VMCK_BLAS(cublasSsyrk(c->blas, CUBLAS_FILL_MODE_UPPER, op, (int)m, k, &one,
                          static_cast<const float *>(O_L), (int)cols, &zero,
                          static_cast<float *>(out), (int)m));
  } else {
    set_last_error("gram_dense dtype");
    return VMCK_ERR_UNSUPPORTED;
  }
  if (diag_shift == 0.0) return VMCK_OK;
  add_diag_kernel<<<ceil_div(m, 256), 256, 0, st>>>(out, dtype, m, diag_shift);
  return check_launch("gram_dense");
}

extern "C" int vmck_center_scale(vmck_stream s, const double *e, const double *mean_dev, int64_t n,
                                 double factor, double *out) {
  VMCK_REQUIRE(e && mean_dev && out && n > 0, "center_scale arguments");
  center_scale_kernel<<<ceil_div(n, 256), 256, 0, as_stream(s)>>>(e, mean_dev, n, factor, out);
  return check_launch("center_scale");
}

extern "C" int vmck_center_update(vmck_stream s, const double *raw, const double *obar,
                                  const double *aux, int64_t n, int64_t P, double scale,
                                  double *update) {
  VMCK_REQUIRE(raw && obar && aux && update && n > 0 && P > 0, "center_update arguments");
  int grid = (int)std::min<int64_t>(ceil_div(P, 256), (int64_t)num_sms() * 2);
  center_update_kernel<<<grid, 256, 0, as_stream(s)>>>(raw, obar, aux, n, P, scale, update);
  return check_launch("center_update");
}

extern "C" int vmck_sgd(vmck_stream s, double *p64, const double *update, int64_t P, double lr,
                        float *p32) {
  VMCK_REQUIRE(p64 && update && P > 0, "sgd arguments");
  sgd_kernel<<<ceil_div(P, 256), 256, 0, as_stream(s)>>>(p64, update, P, lr, p32);
  return check_launch("sgd");
}

extern "C" int vmck_cast_f64_f32(vmck_stream s, const double *in, float *out, int64_t n) {
  VMCK_REQUIRE(in && out && n >= 0, "cast arguments");
  if (n == 0) return VMCK_OK;
  d2f_kernel<<<ceil_div(n, 256), 256, 0, as_stream(s)>>>(in, out, n);
  return check_launch("cast");
}

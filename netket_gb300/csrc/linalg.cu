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

__global__ void d2f_kernel(const double *in, float *out, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}

__global__ void axpy_f2d_kernel(double *x, const float *d, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) x[i] += (double)d[i];
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
// FP32-accurate BF16x9 tensor-core emulation.  Leaves (<= CHOL_LEAF) use
// cuSOLVER POTRF, cuBLAS TRSM / SYRK.
constexpr int64_t CHOL_LEAF = 1024;

static int64_t half_split(int64_t n) {
  int64_t h = ((n / 2) + 255) / 256 * 256;
  return (h >= n) ? n / 2 : h;
}

__global__ void info_accumulate_kernel(const int *info, int32_t *status) {
  if (*info != 0 && status) atomicOr(status, VMCK_DEV_NOT_SPD);
}

struct RecChol {
  vmck_ctx *c;
  cudaStream_t st;
  int32_t *status;
  size_t dsize, hsize;
};

// C (n x n, upper) -= A^T A with A (k x n)
static int syrk_rec(RecChol &R, float *C, int64_t ldc, int64_t n, const float *A, int64_t lda,
                    int64_t k) {
  const float mone = -1.0f, one = 1.0f;
  if (n <= CHOL_LEAF) {
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
  if (m <= CHOL_LEAF) {
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
  if (n <= CHOL_LEAF) {
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

// ------------------------------------------------------------ symmetric residual
// r = b - A x for a symmetric A stored as its lower triangle (row-major), each
// stored element read exactly once.  Tile (I, J), I >= J, of 64 x 64 adds
// A_IJ x_J to the rows of block I (slot J) and A_IJ^T x_I to the rows of block J
// (slot I); on a diagonal tile both go to slot I.  Every (slot, row) of
// ws[n_tiles][n] is written exactly once; the second kernel sums the slots in
// a fixed order.  HBM-bound: n(n+1)/2 * 8 bytes per call.
constexpr int SY_T = 64;

__device__ inline void sy_tri_tile(int64_t bid, int64_t &I, int64_t &J) {
  int64_t i = (int64_t)((sqrt(8.0 * (double)bid + 1.0) - 1.0) * 0.5);
  while (i * (i + 1) / 2 > bid) --i;
  while ((i + 1) * (i + 2) / 2 <= bid) ++i;
  I = i;
  J = bid - i * (i + 1) / 2;
}

__global__ void __launch_bounds__(256) symv_lower_partial_kernel(const double *__restrict__ A,
                                                                 int64_t n,
                                                                 const double *__restrict__ x,
                                                                 double *__restrict__ ws) {
  __shared__ double xr[SY_T], xc[SY_T];
  __shared__ double rowpart[2][SY_T];
  __shared__ double colpart[4][SY_T];
  int64_t I, J;
  sy_tri_tile(blockIdx.x, I, J);
  const int tid = threadIdx.x, c = tid & 63, g = tid >> 6, half = (tid >> 5) & 1;
  const int lane = tid & 31;
  const int64_t r0 = I * SY_T, c0 = J * SY_T;
  if (tid < SY_T) xc[tid] = (c0 + tid < n) ? x[c0 + tid] : 0.0;
  else if (tid < 2 * SY_T) xr[tid - SY_T] = (r0 + tid - SY_T < n) ? x[r0 + tid - SY_T] : 0.0;
  __syncthreads();
  const bool diag = (I == J);
  const bool cok = (c0 + c) < n;
  double colacc = 0.0;
#pragma unroll 4
  for (int k = 0; k < 16; ++k) {
    const int r = g + 4 * k;
    const bool rok = (r0 + r) < n;
    double a = 0.0;
    if (rok && cok && (!diag || r >= c)) a = A[(r0 + r) * n + c0 + c];
    double v = a * xc[c];
    v = warp_sum(v);
    if (lane == 0) rowpart[half][r] = v;
    if (!diag || r > c) colacc += a * xr[r];
  }
  colpart[g][c] = colacc;
  __syncthreads();
  if (tid < SY_T) {
    const int r = tid;
    const double rs = rowpart[0][r] + rowpart[1][r];
    const double cs = colpart[0][r] + colpart[1][r] + colpart[2][r] + colpart[3][r];
    if (diag) {
      if (r0 + r < n) ws[I * n + r0 + r] = rs + cs;
    } else {
      if (r0 + r < n) ws[J * n + r0 + r] = rs;
      if (c0 + r < n) ws[I * n + c0 + r] = cs;
    }
  }
}

__global__ void symv_residual_reduce_kernel(const double *__restrict__ ws, int64_t n, int nt,
                                            const double *__restrict__ b, double *__restrict__ r) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int k = 0; k < nt; ++k) s += ws[k * n + i];
  r[i] = b[i] - s;
}

static int symv_residual(cudaStream_t st, const double *A, int64_t n, const double *x,
                         const double *b, double *r, double *ws) {
  const int64_t nt = (n + SY_T - 1) / SY_T;
  symv_lower_partial_kernel<<<(unsigned)(nt * (nt + 1) / 2), 256, 0, st>>>(A, n, x, ws);
  int rc = check_launch("symv partial");
  if (rc) return rc;
  symv_residual_reduce_kernel<<<ceil_div(n, 256), 256, 0, st>>>(ws, n, (int)nt, b, r);
  return check_launch("symv reduce");
}

static int num_sms() {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
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
  if (c->params) cusolverDnDestroyParams(c->params);
  if (c->solver) cusolverDnDestroy(c->solver);
  if (c->blas) cublasDestroy(c->blas);
  cudaFree(c->dwork);
  cudaFree(c->aux);
  cudaFree(c->d_info);
  free(c->hwork);
  delete c;
  return VMCK_OK;
}

extern "C" int vmck_cholesky_solve(vmck_ctx *c, vmck_stream s, int32_t dtype, const void *A,
                                   const void *b, void *x, int64_t n, int32_t *status) {
  VMCK_REQUIRE(c && A && b && x && n > 0, "cholesky_solve arguments");
  VMCK_REQUIRE(dtype == VMCK_F64 || dtype == VMCK_F32, "cholesky_solve dtype");
  cudaStream_t st = as_stream(s);
  int rc = bind(c, st);
  if (rc) return rc;
  const size_t es = dtype == VMCK_F64 ? 8 : 4;
  const cudaDataType dt = dtype == VMCK_F64 ? CUDA_R_64F : CUDA_R_32F;
  size_t dsize = 0, hsize = 0;
  VMCK_SOLVER(cusolverDnXpotrf_bufferSize(c->solver, c->params, CUBLAS_FILL_MODE_UPPER, n, dt, A,
                                          n, dt, &dsize, &hsize));
  const size_t fbytes = (size_t)n * n * es;
  const size_t off = (fbytes + 255) & ~size_t(255);
  if ((rc = grow(&c->dwork, &c->dwork_bytes, off + dsize + 256, st))) return rc;
  if ((rc = grow_host(c, hsize))) return rc;
  void *F = c->dwork;
  void *work = static_cast<char *>(c->dwork) + off;
  VMCK_CUDA(cudaMemcpyAsync(F, A, fbytes, cudaMemcpyDeviceToDevice, st));
  VMCK_CUDA(cudaMemcpyAsync(x, b, (size_t)n * es, cudaMemcpyDeviceToDevice, st));
  VMCK_SOLVER(cusolverDnXpotrf(c->solver, c->params, CUBLAS_FILL_MODE_UPPER, n, dt, F, n, dt, work,
                               dsize, c->hwork, hsize, c->d_info));
  VMCK_SOLVER(cusolverDnXpotrs(c->solver, c->params, CUBLAS_FILL_MODE_UPPER, n, 1, dt, F, n, dt, x,
                               n, c->d_info));
  if (dtype == VMCK_F64)
    solve_check_kernel<double><<<1, 1024, 0, st>>>(c->d_info, static_cast<const double *>(x),
                                                   static_cast<const double *>(b), n, status);
  else
    solve_check_kernel<float><<<1, 1024, 0, st>>>(c->d_info, static_cast<const float *>(x),
                                                  static_cast<const float *>(b), n, status);
  return check_launch("cholesky_solve check");
}

extern "C" int vmck_cholesky_solve_refined(vmck_ctx *c, vmck_stream s, const double *A64,
                                           float *A32, const double *b, double *x, int64_t n,
                                           int32_t max_iter, double tol, int32_t factor_mode,
                                           int32_t *status, double *residual_out) {
  VMCK_REQUIRE(c && A64 && A32 && b && x && n > 0 && max_iter >= 1, "refined solve arguments");
  VMCK_REQUIRE(factor_mode >= 0 && factor_mode <= 2, "factor_mode must be 0, 1 or 2");
  VMCK_REQUIRE(n < (1ll << 31), "refined solve size");
  cudaStream_t st = as_stream(s);
  int rc = bind(c, st);
  if (rc) return rc;
  const bool emulate = factor_mode != 0;
  VMCK_SOLVER(cusolverDnSetMathMode(c->solver, emulate ? CUSOLVER_FP32_EMULATED_BF16X9_MATH
                                                       : CUSOLVER_DEFAULT_MATH));
  if (emulate)
    VMCK_SOLVER(cusolverDnSetEmulationStrategy(c->solver, CUDA_EMULATION_STRATEGY_EAGER));
  size_t dsize = 0, hsize = 0;
  const int64_t fn = factor_mode == 2 ? std::min<int64_t>(n, CHOL_LEAF) : n;
  VMCK_SOLVER(cusolverDnXpotrf_bufferSize(c->solver, c->params, CUBLAS_FILL_MODE_UPPER, fn,
                                          CUDA_R_32F, A32, n, CUDA_R_32F, &dsize, &hsize));
  if ((rc = grow(&c->dwork, &c->dwork_bytes, dsize + 256, st))) return rc;
  if ((rc = grow_host(c, hsize))) return rc;
  // aux: r (n double), r32 (n float), two norms, symv slots (n_tiles x n double)
  const int64_t nt = (n + SY_T - 1) / SY_T;
  const size_t ws_off = (((size_t)n * 12 + 64) + 255) & ~size_t(255);
  const size_t need = ws_off + (size_t)nt * n * 8;
  if ((rc = grow(&c->aux, &c->aux_bytes, need, st))) return rc;
  double *r = static_cast<double *>(c->aux);
  float *r32 = reinterpret_cast<float *>(r + n);
  double *norms = reinterpret_cast<double *>(
      (reinterpret_cast<uintptr_t>(r32 + n) + 15) & ~uintptr_t(15));
  double *sws = reinterpret_cast<double *>(static_cast<char *>(c->aux) + ws_off);
  if (factor_mode == 2) {
    VMCK_BLAS(cublasSetMathMode(c->blas, CUBLAS_FP32_EMULATED_BF16X9_MATH));
    VMCK_BLAS(cublasSetEmulationStrategy(c->blas, CUBLAS_EMULATION_STRATEGY_EAGER));
    RecChol R{c, st, status, dsize, hsize};
    rc = chol_rec(R, A32, n, n);
    cublasSetMathMode(c->blas, CUBLAS_DEFAULT_MATH);
    cusolverDnSetMathMode(c->solver, CUSOLVER_DEFAULT_MATH);
    if (rc) return rc;
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
  VMCK_CUDA(cudaMemsetAsync(x, 0, (size_t)n * 8, st));
  const int blocks = ceil_div(n, 256);
  for (int it = 0; it < max_iter; ++it) {
    if (it == 0) {
      VMCK_CUDA(cudaMemcpyAsync(r, b, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
    } else if ((rc = symv_residual(st, A64, n, x, b, r, sws))) {
      return rc;
    }
    d2f_kernel<<<blocks, 256, 0, st>>>(r, r32, n);
    if ((rc = check_launch("refined solve cast"))) return rc;
    VMCK_SOLVER(cusolverDnXpotrs(c->solver, c->params, CUBLAS_FILL_MODE_UPPER, n, 1, CUDA_R_32F,
                                 A32, n, CUDA_R_32F, r32, n, c->d_info));
    axpy_f2d_kernel<<<blocks, 256, 0, st>>>(x, r32, n);
    if ((rc = check_launch("refined solve update"))) return rc;
  }
  if ((rc = symv_residual(st, A64, n, x, b, r, sws))) return rc;
  VMCK_BLAS(cublasSetPointerMode(c->blas, CUBLAS_POINTER_MODE_DEVICE));
  cublasStatus_t s1 = cublasDnrm2(c->blas, (int)n, r, 1, norms);
  cublasStatus_t s2 = cublasDnrm2(c->blas, (int)n, b, 1, norms + 1);
  cublasSetPointerMode(c->blas, CUBLAS_POINTER_MODE_HOST);
  if (s1 != CUBLAS_STATUS_SUCCESS || s2 != CUBLAS_STATUS_SUCCESS) {
    set_last_error("refined solve: cublasDnrm2 failed");
    return VMCK_ERR_LIBRARY;
  }
  refine_check_kernel<<<1, 1, 0, st>>>(norms, norms + 1, c->d_info, tol, status, residual_out);
  return check_launch("refined solve");
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

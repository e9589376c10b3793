// PauliStringsJax.get_conn_padded / n_conn (netket/operator/_pauli_strings/
// jax.py:240-269, 311-355) for spin-1/2 states.  A CTA per sample (grid-stride):
// the sample's down-spin bitmask in shared memory, one thread per slot for the
// matrix element (popcount parity per string), then the padded states written
// slot-major with consecutive threads on consecutive sites (coalesced).
#include <algorithm>

#include "common.cuh"
#include "pauli.cuh"

namespace vmck {

constexpr int PS_THREADS = 256;

static int sm_count() {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

__global__ void __launch_bounds__(PS_THREADS)
    get_conn_pauli_kernel(vmck_pauli_strings op, const int8_t *__restrict__ x, int64_t n,
                          int8_t *xp, double *mels, int32_t *n_conn) {
  extern __shared__ unsigned char smem_raw[];
  const int N = op.n_sites, W = op.n_words, F = op.n_flips;
  uint32_t *down = reinterpret_cast<uint32_t *>(smem_raw);
  int8_t *xs = reinterpret_cast<int8_t *>(down + W);
  uint8_t *keep = reinterpret_cast<uint8_t *>(xs + ((N + 15) & ~15));
  __shared__ int red[PS_THREADS / 32];
  for (int64_t b = blockIdx.x; b < n; b += gridDim.x) {
    for (int i = threadIdx.x; i < N; i += blockDim.x) xs[i] = x[b * N + i];
    __syncthreads();
    pauli_down_mask(xs, N, W, down, threadIdx.x, blockDim.x);
    __syncthreads();
    int cnt = 0;
    for (int f = threadIdx.x; f < F; f += blockDim.x) {
      const double m = pauli_mel(op, f, down);
      const bool k = fabs(m) > op.cutoff;
      keep[f] = k;
      mels[b * F + f] = k ? m : 0.0;
      cnt += k;
    }
    cnt = warp_sum(cnt);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0 && n_conn) {
      int t = 0;
      for (int w = 0; w < PS_THREADS / 32; ++w) t += red[w];
      n_conn[b] = t;
    }
    const int64_t FN = (int64_t)F * N;
    int8_t *out = xp + b * FN;
    for (int64_t idx = threadIdx.x; idx < FN; idx += blockDim.x) {
      const int f = (int)(idx / N), i = (int)(idx - (int64_t)f * N);
      const int8_t v = xs[i];
      const bool fl = keep[f] && ((op.flip_mask[(int64_t)f * W + (i >> 5)] >> (i & 31)) & 1u);
      out[idx] = fl ? (int8_t)(-v) : v;
    }
    __syncthreads();
  }
}

}  // namespace vmck

using namespace vmck;

extern "C" int vmck_get_conn_pauli(vmck_stream s, const vmck_pauli_strings *op, const int8_t *x,
                                   int64_t n, int8_t *xp, double *mels, int32_t *n_conn) {
  VMCK_REQUIRE(op && x && xp && mels && n >= 0, "get_conn_pauli arguments");
  int rc = validate_pauli(*op);
  if (rc) return rc;
  if (n == 0 || op->n_flips == 0) {
    if (n_conn && n > 0) VMCK_CUDA(cudaMemsetAsync(n_conn, 0, n * sizeof(int32_t), as_stream(s)));
    return VMCK_OK;
  }
  const size_t smem = 4 * (size_t)op->n_words + ((op->n_sites + 15) & ~15) + op->n_flips + 16;
  VMCK_REQUIRE(smem <= 200 * 1024, "get_conn_pauli: too many slots for shared memory");
  if (smem > 48 * 1024)
    VMCK_CUDA(cudaFuncSetAttribute(get_conn_pauli_kernel,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t grid = std::min<int64_t>(n, (int64_t)sm_count() * 16);
  get_conn_pauli_kernel<<<(unsigned)grid, PS_THREADS, smem, as_stream(s)>>>(*op, x, n, xp, mels,
                                                                           n_conn);
  return check_launch("get_conn_pauli");
}

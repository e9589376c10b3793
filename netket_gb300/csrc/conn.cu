// Connected elements (get_conn_padded) for the Ising and LocalOperator
// Hamiltonians, plus random spin states.
//
// Layout: x (n, N) int8; xp (n, K, N) int8; mels (n, K) FP64.  One CTA handles
// one sample: the per-slot change list is built in shared memory, then the
// K*N-byte output segment of the sample is streamed out with 16-byte stores on
// its 16-byte-aligned interior (the segment itself starts at an arbitrary byte
// offset when K*N is not a multiple of 16).  This kernel is HBM-write bound:
// n * (K*N + 8K) bytes out, n*N bytes in.
#include "common.cuh"
#include "localop.cuh"

namespace vmck {

// --------------------------------------------------------------- random states
// One thread per configuration.  Constrained draws place n_down down spins with
// a Fisher-Yates shuffle of the site list (N <= 4096).
__global__ void random_states_kernel(int8_t *out, int64_t n_batches, int N, int n_down,
                                     uint32_t k0, uint32_t k1, uint32_t sid) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= n_batches) return;
  int8_t *row = out + b * N;
  if (n_down < 0) {
    for (int base = 0; base < N; base += 128) {
      u32x4 r = philox4x32_10(u32x4{(uint32_t)b, (uint32_t)(b >> 32), (uint32_t)(base >> 7), sid},
                              k0, k1);
      uint32_t w[4] = {r.x, r.y, r.z, r.w};
      for (int i = base; i < N && i < base + 128; ++i) {
        int bit = (w[(i - base) >> 5] >> ((i - base) & 31)) & 1;
        row[i] = bit ? int8_t(-1) : int8_t(1);
      }
    }
    return;
  }
  for (int i = 0; i < N; ++i) row[i] = (i < n_down) ? int8_t(-1) : int8_t(1);
  // Fisher-Yates: for i = N-1..1 swap row[i] with row[j], j uniform in [0, i]
  u32x4 r{0, 0, 0, 0};
  for (int i = N - 1, q = 0; i > 0; --i, ++q) {
    if ((q & 3) == 0)
      r = philox4x32_10(u32x4{(uint32_t)b, (uint32_t)(b >> 32), (uint32_t)(q >> 2), sid ^ 0x80000000u},
                        k0, k1);
    uint32_t v = (q & 3) == 0 ? r.x : (q & 3) == 1 ? r.y : (q & 3) == 2 ? r.z : r.w;
    int j = (int)below(v, (uint32_t)(i + 1));
    int8_t t = row[i];
    row[i] = row[j];
    row[j] = t;
  }
}

// --------------------------------------------------------------- streaming out
// Write the K*N-byte segment of one sample.  slot_site[k*4 + c] / slot_val:
// up to 4 (site, new value) changes of slot k (site -1 = unused).
__device__ __forceinline__ int8_t conn_byte(const int8_t *xs, const int16_t *slot_site,
                                            const int8_t *slot_val, int k, int j) {
  int8_t v = xs[j];
  const int16_t *ss = slot_site + 4 * k;
#pragma unroll
  for (int c = 0; c < 4; ++c)
    if (ss[c] == j) v = slot_val[4 * k + c];
  return v;
}

__device__ void stream_out(int8_t *seg, int64_t K, int N, const int8_t *xs,
                           const int16_t *slot_site, const int8_t *slot_val) {
  const int64_t len = K * (int64_t)N;
  uintptr_t addr = reinterpret_cast<uintptr_t>(seg);
  int64_t head = (16 - (int64_t)(addr & 15)) & 15;
  if (head > len) head = len;
  for (int64_t o = threadIdx.x; o < head; o += blockDim.x)
    seg[o] = conn_byte(xs, slot_site, slot_val, (int)(o / N), (int)(o % N));
  const int64_t nvec = (len - head) >> 4;
  uint4 *vp = reinterpret_cast<uint4 *>(seg + head);
  for (int64_t v = threadIdx.x; v < nvec; v += blockDim.x) {
    int64_t o = head + v * 16;
    int k = (int)(o / N), j = (int)(o % N);
    union {
      uint4 u;
      int8_t b[16];
    } pk;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      pk.b[q] = conn_byte(xs, slot_site, slot_val, k, j);
      if (++j == N) {
        j = 0;
        ++k;
      }
    }
    vp[v] = pk.u;
  }
  for (int64_t o = head + nvec * 16 + threadIdx.x; o < len; o += blockDim.x)
    seg[o] = conn_byte(xs, slot_site, slot_val, (int)(o / N), (int)(o % N));
}

// --------------------------------------------------------------- Ising
__global__ void get_conn_ising_kernel(const int8_t *__restrict__ x, int64_t n, int N,
                                      const int32_t *__restrict__ edges, int n_edges,
                                      double h, double J, int h_zero, int8_t *xp,
                                      double *mels, int32_t *n_conn) {
  extern __shared__ unsigned char smem_raw[];
  const int K = h_zero ? 1 : N + 1;
  int8_t *xs = reinterpret_cast<int8_t *>(smem_raw);
  int16_t *slot_site = reinterpret_cast<int16_t *>(smem_raw + ((N + 15) & ~15));
  int8_t *slot_val = reinterpret_cast<int8_t *>(slot_site + 4 * K);
  __shared__ int red[32];
  for (int64_t b = blockIdx.x; b < n; b += gridDim.x) {
    const int8_t *xb = x + b * N;
    for (int i = threadIdx.x; i < N; i += blockDim.x) xs[i] = xb[i];
    __syncthreads();
    int same = 0;
    for (int e = threadIdx.x; e < n_edges; e += blockDim.x)
      same += (xs[edges[2 * e]] == xs[edges[2 * e + 1]]) ? 1 : -1;
    int tot = block_sum(same, red);
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
      slot_site[4 * k + 0] = (k == 0) ? int16_t(-1) : int16_t(k - 1);
      slot_site[4 * k + 1] = slot_site[4 * k + 2] = slot_site[4 * k + 3] = -1;
      slot_val[4 * k] = (k == 0) ? int8_t(0) : int8_t(-xs[k - 1]);
      mels[b * K + k] = (k == 0) ? J * (double)tot : -h;
    }
    if (n_conn && threadIdx.x == 0) n_conn[b] = (h_zero ? 0 : N) + ((J * (double)tot) != 0.0);
    __syncthreads();
    stream_out(xp + b * (int64_t)K * N, K, N, xs, slot_site, slot_val);
    __syncthreads();
  }
}

// --------------------------------------------------------------- LocalOperator
__global__ void get_conn_local_kernel(vmck_local_op op, const int8_t *__restrict__ x,
                                      int64_t n, int8_t *xp, double *mels,
                                      int32_t *n_conn) {
  extern __shared__ unsigned char smem_raw[];
  const int N = op.n_sites, K = op.max_conn_size;
  LocalConnShared sh = local_conn_shared_layout(smem_raw, op);
  int16_t *slot_site = reinterpret_cast<int16_t *>(sh.end);
  int8_t *slot_val = reinterpret_cast<int8_t *>(slot_site + 4 * K);
  for (int64_t b = blockIdx.x; b < n; b += gridDim.x) {
    const int8_t *xb = x + b * N;
    for (int i = threadIdx.x; i < N; i += blockDim.x) sh.xs[i] = xb[i];
    __syncthreads();
    int kept = local_conn_enumerate(op, sh);  // fills sh.slot_term/slot_col/slot_mel
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
      double mel = 0.0;
      int16_t s4[4] = {-1, -1, -1, -1};
      int8_t v4[4] = {0, 0, 0, 0};
      if (k < kept) {
        mel = sh.slot_mel[k];
        int t = sh.slot_term[k];
        if (t >= 0) {
          int c = sh.slot_col[k], row = sh.row[t], S = op.max_sites;
          int sz = op.acting_size[t];
          const int8_t *xpv = op.x_prime + (((int64_t)t * op.max_rows + row) * op.max_conns + c) * S;
          for (int q = 0; q < sz && q < 4; ++q) {
            s4[q] = (int16_t)op.acting_on[t * S + q];
            v4[q] = xpv[q];
          }
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        slot_site[4 * k + q] = s4[q];
        slot_val[4 * k + q] = v4[q];
      }
      mels[b * K + k] = mel;
    }
    if (n_conn && threadIdx.x == 0) n_conn[b] = kept;
    __syncthreads();
    stream_out(xp + b * (int64_t)K * N, K, N, sh.xs, slot_site, slot_val);
    __syncthreads();
  }
}

static int grid_for(int64_t n) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int64_t g = (int64_t)sms * 16;
  return (int)(n < g ? n : g);
}

}  // namespace vmck

using namespace vmck;

extern "C" int vmck_random_states(vmck_stream s, int8_t *out, int64_t n_batches, int32_t N,
                                  int32_t n_down, uint64_t seed, uint64_t stream_id) {
  VMCK_REQUIRE(out && N > 0 && n_batches >= 0 && n_down <= N, "random_states sizes");
  if (n_batches == 0) return VMCK_OK;
  int threads = 128;
  random_states_kernel<<<ceil_div(n_batches, threads), threads, 0, as_stream(s)>>>(
      out, n_batches, N, n_down, (uint32_t)seed, (uint32_t)(seed >> 32), (uint32_t)stream_id);
  return check_launch("random_states");
}

extern "C" int vmck_get_conn_ising(vmck_stream s, const int8_t *x, int64_t n, int32_t N,
                                   const int32_t *edges, int32_t n_edges, double h, double J,
                                   int32_t h_is_zero, int8_t *xp, double *mels,
                                   int32_t *n_conn) {
  VMCK_REQUIRE(x && xp && mels && N > 0 && N < 32768 && n >= 0, "get_conn_ising sizes");
  VMCK_REQUIRE(n_edges == 0 || edges, "edges");
  if (n == 0) return VMCK_OK;
  const int K = h_is_zero ? 1 : N + 1;
  size_t smem = ((N + 15) & ~15) + (size_t)K * 4 * sizeof(int16_t) + (size_t)K * 4;
  VMCK_REQUIRE(smem <= 200 * 1024, "N too large for get_conn_ising");
  if (smem > 48 * 1024)
    VMCK_CUDA(cudaFuncSetAttribute(get_conn_ising_kernel,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  get_conn_ising_kernel<<<grid_for(n), 256, smem, as_stream(s)>>>(
      x, n, N, edges, n_edges, h, J, h_is_zero, xp, mels, n_conn);
  return check_launch("get_conn_ising");
}

extern "C" int vmck_get_conn_local(vmck_stream s, const vmck_local_op *op, const int8_t *x,
                                   int64_t n, int8_t *xp, double *mels, int32_t *n_conn) {
  VMCK_REQUIRE(op && x && xp && mels && n >= 0, "get_conn_local pointers");
  int rc = validate_local_op(*op);
  if (rc) return rc;
  if (n == 0) return VMCK_OK;
  const int K = op->max_conn_size;
  size_t smem = local_conn_shared_bytes(*op) + (size_t)K * 4 * sizeof(int16_t) + (size_t)K * 4;
  VMCK_REQUIRE(smem <= 200 * 1024, "operator too large for get_conn_local");
  if (smem > 48 * 1024)
    VMCK_CUDA(cudaFuncSetAttribute(get_conn_local_kernel,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  get_conn_local_kernel<<<grid_for(n), 256, smem, as_stream(s)>>>(*op, x, n, xp, mels, n_conn);
  return check_launch("get_conn_local");
}

// RBM kernels: log-amplitude (theta GEMM with a log_cosh epilogue), local
// energies (plain reduction and the fused log-ratio form), O^T v and the dense
// centred Jacobian.
//
// Parameter layout (NetKet ravel order of the RBM pytree, netket/models/rbm.py):
//   params = [bias (M) | kernel W (N x M, row-major) | visible_bias (N)].
#include <algorithm>

#include "common.cuh"
#include "localop.cuh"
#include "pauli.cuh"

namespace vmck {

template <typename T>
struct RbmParams {
  const T *b, *W, *a;
  int N, M;
};

template <typename T>
__host__ __device__ inline RbmParams<T> rbm_view(const void *p, int N, int M) {
  const T *q = static_cast<const T *>(p);
  return RbmParams<T>{q, q + M, q + M + (int64_t)N * M, N, M};
}

// ============================================================ logpsi
// CTA: 64 rows x all M columns (in 64-column panels), K loop over N in chunks
// of 16.  256 threads, 4x4 register tile each.  Epilogue per panel:
// theta = acc + b, log_cosh summed per row (deterministic order: panel by
// panel, then a fixed shuffle tree), optional theta / tanh(theta) outputs.
constexpr int LP_BM = 64, LP_BN = 64, LP_BK = 16;

template <typename T>
__global__ void __launch_bounds__(256) logpsi_kernel(RbmParams<T> P, const int8_t *__restrict__ x,
                                                     int64_t n, T *__restrict__ logpsi,
                                                     T *__restrict__ theta_out,
                                                     T *__restrict__ tanh_out) {
  __shared__ T xs[LP_BK][LP_BM];
  __shared__ T ws[LP_BK][LP_BN];
  __shared__ T rowsum[16][LP_BM];
  const int N = P.N, M = P.M;
  const int tid = threadIdx.x;
  const int tr = tid >> 4, tc = tid & 15;  // 16 x 16 thread grid, 4 x 4 each
  const int64_t row0 = (int64_t)blockIdx.x * LP_BM;
  T lsum[4] = {0, 0, 0, 0};
  for (int c0 = 0; c0 < M; c0 += LP_BN) {
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = 0;
    for (int k0 = 0; k0 < N; k0 += LP_BK) {
      // x tile: 64 rows x 16 sites (transposed into xs[k][row])
      for (int e = tid; e < LP_BM * LP_BK; e += 256) {
        int r = e / LP_BK, k = e % LP_BK;
        int64_t gr = row0 + r;
        int gk = k0 + k;
        xs[k][r] = (gr < n && gk < N) ? (T)x[gr * N + gk] : T(0);
      }
      for (int e = tid; e < LP_BK * LP_BN; e += 256) {
        int k = e / LP_BN, c = e % LP_BN;
        int gk = k0 + k, gc = c0 + c;
        ws[k][c] = (gk < N && gc < M) ? P.W[(int64_t)gk * M + gc] : T(0);
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < LP_BK; ++k) {
        T xa[4], wb[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) xa[i] = xs[k][tr * 4 + i];
#pragma unroll
        for (int j = 0; j < 4; ++j) wb[j] = ws[k][tc * 4 + j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] += xa[i] * wb[j];
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int64_t gr = row0 + tr * 4 + i;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        int gc = c0 + tc * 4 + j;
        if (gr < n && gc < M) {
          T th = acc[i][j] + P.b[gc];
          lsum[i] += log_cosh(th);
          if (theta_out) theta_out[gr * M + gc] = th;
          if (tanh_out) tanh_out[gr * M + gc] = tanh(th);
        }
      }
    }
  }
  // reduce lsum over the 16 column-threads of each row
#pragma unroll
  for (int i = 0; i < 4; ++i) rowsum[tc][tr * 4 + i] = lsum[i];
  __syncthreads();
  if (tid < LP_BM) {
    int64_t gr = row0 + tid;
    if (gr < n) {
      T s = 0;
      for (int c = 0; c < 16; ++c) s += rowsum[c][tid];
      T v = 0;
      for (int i = 0; i < N; ++i) v += (T)x[gr * N + i] * P.a[i];
      logpsi[gr] = s + v;
    }
  }
}

// ============================================================ plain E_loc
template <typename T>
__global__ void eloc_reduce_kernel(const T *__restrict__ lp, const T *__restrict__ lpc,
                                   const double *__restrict__ mels, int64_t n, int K,
                                   double *eloc) {
  int64_t b = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (b >= n) return;
  double s = 0.0;
  T l0 = lp[b];
  for (int k = lane; k < K; k += 32)
    s += mels[b * K + k] * (double)exp(lpc[b * K + k] - l0);
  s = warp_sum(s);
  if (lane == 0) eloc[b] = s;
}

// ============================================================ fused E_loc
// One CTA (4 warps) per sample.  theta and log_cosh(theta) live in shared
// memory; every connected element changes at most 4 sites, so its log-ratio is
//   sum_j [log_cosh(theta_j + sum_s d_s W[site_s, j]) - log_cosh(theta_j)] + sum_s d_s a_site
// with d_s = x'_s - x_s.  Warps take connected elements round-robin; lanes split j.
constexpr int EL_THREADS = 128;

// block_sum over a thread group (same tree: warp shuffles, then the warp totals
// in one warp).  red: 32 elements of this group.
template <typename T>
__device__ inline T grp_sum(const Grp &g, T v, T *red) {
  const int lane = g.tid & 31, wid = g.tid >> 5, nw = g.size >> 5;
  v = warp_sum(v);
  grp_sync(g);
  if (lane == 0) red[wid] = v;
  grp_sync(g);
  T t = (lane < nw) ? red[lane] : T(0);
  return warp_sum(t);
}

template <typename T>
__device__ inline void theta_and_logpsi(const RbmParams<T> &P, const int8_t *xs, T *th, T *lc,
                                        T *red, T *logpsi_out, const Grp &g) {
  const int N = P.N, M = P.M;
  T part = 0;
  for (int j = g.tid; j < M; j += g.size) {
    T acc = P.b[j];
    for (int i = 0; i < N; ++i) acc += (T)xs[i] * P.W[(int64_t)i * M + j];
    th[j] = acc;
    T l = log_cosh_fast(acc);
    lc[j] = l;
    part += l;
  }
  for (int i = g.tid; i < N; i += g.size) part += (T)xs[i] * P.a[i];
  T tot = grp_sum(g, part, red);
  if (logpsi_out && g.tid == 0) *logpsi_out = tot;
}

template <typename T>
__device__ inline void theta_and_logpsi(const RbmParams<T> &P, const int8_t *xs, T *th, T *lc,
                                        T *red, T *logpsi_out) {
  theta_and_logpsi(P, xs, th, lc, red, logpsi_out, cta_grp());
}

// Log-ratio for NS sites with the W row pointers and the changes held in
// registers; a site with d = 0 adds an exact zero, so the result equals
// warp_log_ratio over the changed sites only.
template <typename T, int NS>
__device__ inline T warp_log_ratio_n(const RbmParams<T> &P, const T *th, const T *lc,
                                     const int (&site)[4], const T (&d)[4]) {
  const int lane = threadIdx.x & 31, M = P.M;
  const T *w[NS];
  T dd[NS];
#pragma unroll
  for (int q = 0; q < NS; ++q) {
    w[q] = P.W + (int64_t)site[q] * M;
    dd[q] = d[q];
  }
  T s = 0;
  for (int j = lane; j < M; j += 32) {
    T t = th[j];
#pragma unroll
    for (int q = 0; q < NS; ++q) t += dd[q] * w[q][j];
    s += log_cosh_fast(t) - lc[j];
  }
  s = warp_sum(s);
#pragma unroll
  for (int q = 0; q < NS; ++q) s += dd[q] * P.a[site[q]];
  return s;
}

template <typename T>
__device__ inline T warp_log_ratio(const RbmParams<T> &P, const T *th, const T *lc,
                                   const int *site, const T *d, int ns) {
  const int lane = threadIdx.x & 31, M = P.M;
  T s = 0;
  for (int j = lane; j < M; j += 32) {
    T t = th[j];
    for (int q = 0; q < ns; ++q) t += d[q] * P.W[(int64_t)site[q] * M + j];
    s += log_cosh_fast(t) - lc[j];
  }
  s = warp_sum(s);
  for (int q = 0; q < ns; ++q) s += d[q] * P.a[site[q]];
  return s;
}

// Local energy of one sample for the Ising Hamiltonian, by the whole CTA.
// xs must hold the configuration (visible to all threads); returns E_loc on
// every thread.
template <typename T>
__device__ double eloc_ising_sample(const RbmParams<T> &P, const int8_t *xs,
                                    const int32_t *__restrict__ edges, int n_edges, double h,
                                    double J, T *th, T *lc, T *red, double *redd, int *redi,
                                    T *logpsi_out) {
  const int N = P.N;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  theta_and_logpsi(P, xs, th, lc, red, logpsi_out);
  int same = 0;
  for (int e = threadIdx.x; e < n_edges; e += blockDim.x)
    same += (xs[edges[2 * e]] == xs[edges[2 * e + 1]]) ? 1 : -1;
  int tot = block_sum(same, redi);
  double acc = 0.0;
  if (h != 0.0) {
    for (int k = warp; k < N; k += nw) {
      int site = k;
      T d = (T)(-2 * xs[k]);
      T lr = warp_log_ratio(P, th, lc, &site, &d, 1);
      if (lane == 0) acc += -h * exp_ratio(lr);
    }
  }
  if (threadIdx.x == 0) acc += J * (double)tot;
  return block_sum(acc, redd);
}

template <typename T>
__global__ void __launch_bounds__(EL_THREADS) eloc_ising_kernel(
    RbmParams<T> P, const int8_t *__restrict__ x, int64_t n, const int32_t *__restrict__ edges,
    int n_edges, double h, double J, double *eloc, T *logpsi_out) {
  extern __shared__ unsigned char smem_raw[];
  const int N = P.N, M = P.M;
  T *th = reinterpret_cast<T *>(smem_raw);
  T *lc = th + M;
  int8_t *xs = reinterpret_cast<int8_t *>(lc + M);
  __shared__ T red[32];
  __shared__ double redd[32];
  __shared__ int redi[32];
  for (int64_t b = blockIdx.x; b < n; b += gridDim.x) {
    for (int i = threadIdx.x; i < N; i += blockDim.x) xs[i] = x[b * N + i];
    __syncthreads();
    double e = eloc_ising_sample(P, xs, edges, n_edges, h, J, th, lc, red, redd, redi,
                                 logpsi_out ? logpsi_out + b : nullptr);
    if (threadIdx.x == 0) eloc[b] = e;
    __syncthreads();
  }
}

template <typename T>
__global__ void __launch_bounds__(EL_THREADS) batched_eloc_ising_kernel(
    const vmck_batch_ising *__restrict__ inst, const int32_t *__restrict__ work, int n_items,
    int32_t *queue, int spi, int max_M) {
  extern __shared__ unsigned char smem_raw[];
  T *th = reinterpret_cast<T *>(smem_raw);
  T *lc = th + max_M;
  int8_t *xs = reinterpret_cast<int8_t *>(lc + max_M);
  __shared__ T red[32];
  __shared__ double redd[32];
  __shared__ int redi[32];
  __shared__ int item_s;
  while (true) {
    if (threadIdx.x == 0) item_s = atomicAdd(queue, 1);
    __syncthreads();
    const int item = item_s;
    __syncthreads();
    if (item >= n_items) break;
    const vmck_batch_ising I = inst[work[2 * item]];
    const RbmParams<T> P = rbm_view<T>(I.params, I.N, I.M);
    const int64_t first = work[2 * item + 1];
    for (int q = 0; q < spi; ++q) {
      const int64_t b = first + q;
      if (b >= I.n) break;  // uniform across the CTA
      for (int i = threadIdx.x; i < I.N; i += blockDim.x) xs[i] = I.x[b * I.N + i];
      __syncthreads();
      double e = eloc_ising_sample(P, xs, I.edges, I.n_edges, I.h, I.J, th, lc, red, redd, redi,
                                   (T *)nullptr);
      if (threadIdx.x == 0) I.eloc[b] = e;
      __syncthreads();
    }
  }
}

// Local energy of sample b by one 4-warp group g (the whole CTA in
// eloc_local_kernel): theta, enumeration of the connected elements, warps take
// them round-robin, lane 0 accumulates, the group's tree sums the warps.
template <typename T>
__device__ inline void eloc_local_sample(const RbmParams<T> &P, const int8_t *__restrict__ x,
                                         int64_t b, const vmck_local_op &op, double *eloc,
                                         T *logpsi_out, LocalConnShared &sh, T *th, T *lc, T *red,
                                         double *redd, const Grp &g) {
  const int N = P.N;
  const int warp = g.tid >> 5, lane = g.tid & 31, nw = g.size >> 5;
  const int S = op.max_sites;
  for (int i = g.tid; i < N; i += g.size) sh.xs[i] = x[b * N + i];
  grp_sync(g);
  theta_and_logpsi(P, sh.xs, th, lc, red, logpsi_out ? logpsi_out + b : nullptr, g);
  int kept = local_conn_enumerate(op, sh, g, sizeof(T) == 8);
  double acc = 0.0;
  for (int k = warp; k < kept; k += nw) {
    double mel = sh.slot_mel[k];
    int t = sh.slot_term[k];
    // sites of the term in slots 0..sz-1 (unchanged sites get d = 0)
    int site[4] = {0, 0, 0, 0};
    T d[4] = {0, 0, 0, 0};
    int ns = 0, sz = 0;
    if (t >= 0) {
      const int row = sh.row[t], c = sh.slot_col[k];
      sz = op.acting_size[t];
      const int8_t *xpv = op.x_prime + (((int64_t)t * op.max_rows + row) * op.max_conns + c) * S;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (q < sz) {
          const int st = op.acting_on[t * S + q];
          const int dv = (int)xpv[q] - (int)sh.xs[st];
          site[q] = st;
          d[q] = (T)dv;
          ns += dv != 0;
        }
      }
    }
    if (ns == 0) {
      if (lane == 0) acc += mel;
    } else {
      T lr;
      if (sz <= 1) lr = warp_log_ratio_n<T, 1>(P, th, lc, site, d);
      else if (sz == 2) lr = warp_log_ratio_n<T, 2>(P, th, lc, site, d);
      else if (sz == 3) lr = warp_log_ratio_n<T, 3>(P, th, lc, site, d);
      else lr = warp_log_ratio_n<T, 4>(P, th, lc, site, d);
      if (lane == 0) acc += mel * exp_ratio(lr);
    }
  }
  double e = grp_sum(g, acc, redd);
  if (g.tid == 0) eloc[b] = e;
  grp_sync(g);
}

template <typename T>
__global__ void __launch_bounds__(EL_THREADS) eloc_local_kernel(
    RbmParams<T> P, const int8_t *__restrict__ x, int64_t n, vmck_local_op op, double *eloc,
    T *logpsi_out) {
  extern __shared__ unsigned char smem_raw[];
  LocalConnShared sh = local_conn_shared_layout(smem_raw, op);
  T *th = reinterpret_cast<T *>(sh.end);
  T *lc = th + P.M;
  __shared__ T red[32];
  __shared__ double redd[32];
  const Grp g = cta_grp();
  for (int64_t b = blockIdx.x; b < n; b += gridDim.x)
    eloc_local_sample(P, x, b, op, eloc, logpsi_out, sh, th, lc, red, redd, g);
}

// Local energy for PauliStrings, one CTA per sample (grid-stride): theta and
// log_cosh(theta) in shared memory, the down-spin bitmask, then warps take
// slots round-robin.  Lanes split the slot's strings for its matrix element
// (a warp tree sum) and the hidden units for the log-ratio of flipping the
// slot's sites F: sum_j [log_cosh(theta_j - 2 sum_{i in F} x_i W_ij) -
// log_cosh(theta_j)] - 2 sum_{i in F} x_i a_i.
template <typename T>
__global__ void __launch_bounds__(EL_THREADS) eloc_pauli_kernel(
    RbmParams<T> P, const int8_t *__restrict__ x, int64_t n, vmck_pauli_strings op,
    double *eloc, T *logpsi_out) {
  extern __shared__ unsigned char smem_raw[];
  const int N = P.N, M = P.M;
  T *th = reinterpret_cast<T *>(smem_raw);
  T *lc = th + M;
  uint32_t *down = reinterpret_cast<uint32_t *>(lc + M);
  int8_t *xs = reinterpret_cast<int8_t *>(down + op.n_words);
  __shared__ T red[32];
  __shared__ double redd[32];
  const Grp g = cta_grp();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int64_t b = blockIdx.x; b < n; b += gridDim.x) {
    for (int i = threadIdx.x; i < N; i += blockDim.x) xs[i] = x[b * N + i];
    __syncthreads();
    pauli_down_mask(xs, N, op.n_words, down, threadIdx.x, blockDim.x);
    theta_and_logpsi(P, xs, th, lc, red, logpsi_out ? logpsi_out + b : nullptr, g);
    double acc = 0.0;
    for (int f = warp; f < op.n_flips; f += nw) {
      double m = 0.0;
      for (int s = op.string_offset[f] + lane; s < op.string_offset[f + 1]; s += 32)
        m += op.weight[s] * pauli_sign(op, s, down);
      m = warp_sum(m);
      if (!(fabs(m) > op.cutoff)) continue;
      const int q0 = op.flip_offset[f], q1 = op.flip_offset[f + 1];
      if (q0 == q1) {
        if (lane == 0) acc += m;
        continue;
      }
      T sl = 0;
      for (int j = lane; j < M; j += 32) {
        T t = th[j];
        for (int q = q0; q < q1; ++q) {
          const int i = op.flip_site[q];
          t += (T)(-2 * xs[i]) * P.W[(int64_t)i * M + j];
        }
        sl += log_cosh_fast(t) - lc[j];
      }
      sl = warp_sum(sl);
      for (int q = q0; q < q1; ++q) {
        const int i = op.flip_site[q];
        sl += (T)(-2 * xs[i]) * P.a[i];
      }
      if (lane == 0) acc += m * exp_ratio(sl);
    }
    const double e = grp_sum(g, acc, redd);
    if (threadIdx.x == 0) eloc[b] = e;
    __syncthreads();
  }
}

// ============================================================ O v
// One warp per sample: lanes take hidden units j, u_j = v_bias[j] + x_s . V[:, j]
// (FP64, V read through L1), then t_s . u + x_s . v_visible, a shuffle tree.
template <typename T>
__global__ void o_v_kernel(const T *__restrict__ t, const int8_t *__restrict__ x, int N, int M,
                           int64_t n, const double *__restrict__ v, double *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t s = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (s >= n) return;
  const int8_t *xs = x + s * N;
  const T *ts = t + s * M;
  const double *V = v + M;
  double acc = 0.0;
  for (int j = lane; j < M; j += 32) {
    double u = v[j];
    for (int i = 0; i < N; ++i) u += (double)xs[i] * __ldg(V + (int64_t)i * M + j);
    acc += (double)ts[j] * u;
  }
  const double *va = v + M + (int64_t)N * M;
  for (int i = lane; i < N; i += 32) acc += (double)xs[i] * va[i];
  acc = warp_sum(acc);
  if (lane == 0) out[s] = acc;
}

// ============================================================ O^T v
// grid (ceil(M/64), ceil(N/64), chunks).  Each CTA accumulates, over its chunk
// of samples, out[kernel_ij] for a 64 x 64 (i, j) tile (plus bias_j when
// blockIdx.y == 0 and visible_i when blockIdx.x == 0) and writes the partial to
// workspace[chunk][P]; a second kernel sums the chunks in a fixed order.
constexpr int OT_TJ = 64, OT_TI = 64, OT_SB = 32;

template <typename T>
__global__ void __launch_bounds__(256) ot_v_partial_kernel(const T *__restrict__ t,
                                                           const int8_t *__restrict__ x, int N,
                                                           int M, int64_t n, int64_t chunk,
                                                           const double *__restrict__ v,
                                                           double *__restrict__ ws) {
  __shared__ T tv[OT_SB][OT_TJ];
  __shared__ T xv[OT_SB][OT_TI];   // x * v (visible part)
  __shared__ int8_t xsm[OT_SB][OT_TI];
  const int tid = threadIdx.x;
  const int jj = tid & 63, ig = tid >> 6;  // 4 groups of i
  const int j0 = blockIdx.x * OT_TJ, i0 = blockIdx.y * OT_TI;
  const int64_t s0 = (int64_t)blockIdx.z * chunk;
  const int64_t s1 = (s0 + chunk < n) ? s0 + chunk : n;
  const int64_t P = (int64_t)M + (int64_t)N * M + N;
  T acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = 0;
  T accb = 0, accv = 0;
  for (int64_t sb = s0; sb < s1; sb += OT_SB) {
    for (int e = tid; e < OT_SB * OT_TJ; e += 256) {
      int r = e / OT_TJ, c = e % OT_TJ;
      int64_t s = sb + r;
      int j = j0 + c;
      tv[r][c] = (s < s1 && j < M) ? t[s * M + j] * (T)v[s] : T(0);
    }
    for (int e = tid; e < OT_SB * OT_TI; e += 256) {
      int r = e / OT_TI, c = e % OT_TI;
      int64_t s = sb + r;
      int i = i0 + c;
      int8_t xx = (s < s1 && i < N) ? x[s * N + i] : int8_t(0);
      xsm[r][c] = xx;
      xv[r][c] = (T)xx * ((s < s1) ? (T)v[s] : T(0));
    }
    __syncthreads();
    const int rows = (int)((s1 - sb) < OT_SB ? (s1 - sb) : OT_SB);
    for (int r = 0; r < rows; ++r) {
      T w = tv[r][jj];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        int8_t xx = xsm[r][ig + 4 * q];
        acc[q] += (xx > 0) ? w : ((xx < 0) ? -w : T(0));
      }
      if (ig == 0) accb += w;
      if (ig == 1) accv += xv[r][jj];
    }
    __syncthreads();
  }
  double *out = ws + (int64_t)blockIdx.z * P;
  const int j = j0 + jj;
  if (j < M) {
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      int i = i0 + ig + 4 * q;
      if (i < N) out[M + (int64_t)i * M + j] = (double)acc[q];
    }
    if (ig == 0 && blockIdx.y == 0) out[j] = (double)accb;
  }
  if (ig == 1 && blockIdx.x == 0) {
    int i = i0 + jj;
    if (i < N) out[M + (int64_t)N * M + i] = (double)accv;
  }
}

__global__ void reduce_chunks_kernel(const double *__restrict__ ws, int64_t P, int nchunk,
                                     double *__restrict__ out) {
  int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= P) return;
  double s = 0.0;
  for (int c = 0; c < nchunk; ++c) s += ws[(int64_t)c * P + p];
  out[p] = s;
}

// ============================================================ dense Jacobian
template <typename T, typename O>
__global__ void jacobian_kernel(const T *__restrict__ t, const int8_t *__restrict__ x, int N,
                                int M, int64_t n, const double *__restrict__ mean, double scale,
                                O *__restrict__ out) {
  const int64_t P = (int64_t)M + (int64_t)N * M + N;
  for (int64_t s = blockIdx.x; s < n; s += gridDim.x) {
    const T *ts = t + s * M;
    const int8_t *xs = x + s * N;
    O *row = out + s * P;
    for (int64_t p = threadIdx.x; p < P; p += blockDim.x) {
      double o;
      if (p < M)
        o = (double)ts[p];
      else if (p < M + (int64_t)N * M) {
        int64_t q = p - M;
        o = (double)xs[q / M] * (double)ts[q % M];
      } else
        o = (double)xs[p - M - (int64_t)N * M];
      row[p] = (O)((o - mean[p]) * scale);
    }
  }
}

static int num_sms() {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

template <typename T>
int launch_logpsi(cudaStream_t st, const void *params, int N, int M, const int8_t *x, int64_t n,
                  void *logpsi, void *theta, void *tanh_out) {
  RbmParams<T> P = rbm_view<T>(params, N, M);
  int64_t grid = (n + LP_BM - 1) / LP_BM;
  VMCK_REQUIRE(grid < (1ll << 31), "too many rows");
  logpsi_kernel<T><<<(unsigned)grid, 256, 0, st>>>(P, x, n, static_cast<T *>(logpsi),
                                                   static_cast<T *>(theta),
                                                   static_cast<T *>(tanh_out));
  return check_launch("rbm_logpsi");
}

template <typename T>
int launch_eloc_ising(cudaStream_t st, const void *params, int N, int M, const int8_t *x,
                      int64_t n, const int32_t *edges, int n_edges, double h, double J,
                      double *eloc, void *lp) {
  RbmParams<T> P = rbm_view<T>(params, N, M);
  size_t smem = 2 * sizeof(T) * (size_t)M + align16(N);
  VMCK_REQUIRE(smem <= 200 * 1024, "M too large for the fused local-energy kernel");
  if (smem > 48 * 1024)
    VMCK_CUDA(cudaFuncSetAttribute(eloc_ising_kernel<T>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t grid = std::min<int64_t>(n, (int64_t)num_sms() * 32);
  eloc_ising_kernel<T><<<(unsigned)grid, EL_THREADS, smem, st>>>(P, x, n, edges, n_edges, h, J,
                                                                 eloc, static_cast<T *>(lp));
  return check_launch("rbm_eloc_ising");
}

template <typename T>
int launch_eloc_local(cudaStream_t st, const void *params, int N, int M, const int8_t *x,
                      int64_t n, const vmck_local_op &op, double *eloc, void *lp) {
  RbmParams<T> P = rbm_view<T>(params, N, M);
  size_t smem = local_conn_shared_bytes(op) + 2 * sizeof(T) * (size_t)M + 16;
  VMCK_REQUIRE(smem <= 200 * 1024, "operator / M too large for the fused local-energy kernel");
  if (smem > 48 * 1024)
    VMCK_CUDA(cudaFuncSetAttribute(eloc_local_kernel<T>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t grid = std::min<int64_t>(n, (int64_t)num_sms() * 32);
  eloc_local_kernel<T><<<(unsigned)grid, EL_THREADS, smem, st>>>(P, x, n, op, eloc,
                                                                 static_cast<T *>(lp));
  return check_launch("rbm_eloc_local");
}

template <typename T>
int launch_eloc_pauli(cudaStream_t st, const void *params, int N, int M, const int8_t *x,
                      int64_t n, const vmck_pauli_strings &op, double *eloc, void *lp) {
  RbmParams<T> P = rbm_view<T>(params, N, M);
  const size_t smem = 2 * sizeof(T) * (size_t)M + 4 * (size_t)op.n_words + N + 16;
  VMCK_REQUIRE(smem <= 200 * 1024, "M too large for the fused local-energy kernel");
  if (smem > 48 * 1024)
    VMCK_CUDA(cudaFuncSetAttribute(eloc_pauli_kernel<T>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t grid = std::min<int64_t>(n, (int64_t)num_sms() * 32);
  eloc_pauli_kernel<T><<<(unsigned)grid, EL_THREADS, smem, st>>>(P, x, n, op, eloc,
                                                                 static_cast<T *>(lp));
  return check_launch("rbm_eloc_pauli");
}

}  // namespace vmck

using namespace vmck;

extern "C" int vmck_rbm_eloc_pauli(vmck_stream s, int32_t dtype, const void *params, int32_t N,
                                   int32_t M, const int8_t *x, int64_t n,
                                   const vmck_pauli_strings *op, double *eloc, void *logpsi_out) {
  VMCK_REQUIRE(params && x && op && eloc && N > 0 && M > 0 && n >= 0, "rbm_eloc_pauli arguments");
  int rc = validate_pauli(*op);
  if (rc) return rc;
  VMCK_REQUIRE(op->n_sites == N, "rbm_eloc_pauli: operator size differs from N");
  if (n == 0) return VMCK_OK;
  if (dtype == VMCK_F64)
    return launch_eloc_pauli<double>(as_stream(s), params, N, M, x, n, *op, eloc, logpsi_out);
  if (dtype == VMCK_F32)
    return launch_eloc_pauli<float>(as_stream(s), params, N, M, x, n, *op, eloc, logpsi_out);
  set_last_error("rbm_eloc_pauli: dtype %d unsupported", dtype);
  return VMCK_ERR_UNSUPPORTED;
}

extern "C" int vmck_rbm_o_v(vmck_stream s, int32_t dtype, const void *tanh_theta,
                            const int8_t *x, int32_t N, int32_t M, int64_t n, const double *v,
                            double *out) {
  VMCK_REQUIRE(tanh_theta && x && v && out && N > 0 && M > 0 && n >= 0, "rbm_o_v arguments");
  if (n == 0) return VMCK_OK;
  const unsigned grid = (unsigned)((n + 7) / 8);
  if (dtype == VMCK_F64)
    o_v_kernel<double><<<grid, 256, 0, as_stream(s)>>>(static_cast<const double *>(tanh_theta), x,
                                                        N, M, n, v, out);
  else if (dtype == VMCK_F32)
    o_v_kernel<float><<<grid, 256, 0, as_stream(s)>>>(static_cast<const float *>(tanh_theta), x,
                                                       N, M, n, v, out);
  else {
    set_last_error("rbm_o_v: dtype %d unsupported", dtype);
    return VMCK_ERR_UNSUPPORTED;
  }
  return check_launch("rbm_o_v");
}

extern "C" int vmck_rbm_logpsi(vmck_stream s, int32_t dtype, const void *params, int32_t N,
                               int32_t M, const int8_t *x, int64_t n, void *logpsi,
                               void *theta_out, void *tanh_out) {
  VMCK_REQUIRE(params && x && logpsi && N > 0 && M > 0 && n >= 0, "rbm_logpsi arguments");
  if (n == 0) return VMCK_OK;
  if (dtype == VMCK_F64)
    return launch_logpsi<double>(as_stream(s), params, N, M, x, n, logpsi, theta_out, tanh_out);
  if (dtype == VMCK_F32)
    return launch_logpsi<float>(as_stream(s), params, N, M, x, n, logpsi, theta_out, tanh_out);
  set_last_error("rbm_logpsi: dtype %d unsupported", dtype);
  return VMCK_ERR_UNSUPPORTED;
}

extern "C" int vmck_eloc_from_logpsi(vmck_stream s, int32_t dtype, const void *lp,
                                     const void *lp_conn, const double *mels, int64_t n,
                                     int32_t K, double *eloc) {
  VMCK_REQUIRE(lp && lp_conn && mels && eloc && n >= 0 && K > 0, "eloc_from_logpsi arguments");
  if (n == 0) return VMCK_OK;
  unsigned grid = (unsigned)((n + 7) / 8);
  if (dtype == VMCK_F64)
    eloc_reduce_kernel<double><<<grid, 256, 0, as_stream(s)>>>(
        static_cast<const double *>(lp), static_cast<const double *>(lp_conn), mels, n, K, eloc);
  else if (dtype == VMCK_F32)
    eloc_reduce_kernel<float><<<grid, 256, 0, as_stream(s)>>>(
        static_cast<const float *>(lp), static_cast<const float *>(lp_conn), mels, n, K, eloc);
  else {
    set_last_error("eloc_from_logpsi: dtype %d unsupported", dtype);
    return VMCK_ERR_UNSUPPORTED;
  }
  return check_launch("eloc_from_logpsi");
}

extern "C" int vmck_rbm_eloc_ising(vmck_stream s, int32_t dtype, const void *params, int32_t N,
                                   int32_t M, const int8_t *x, int64_t n, const int32_t *edges,
                                   int32_t n_edges, double h, double J, double *eloc,
                                   void *logpsi_out) {
  VMCK_REQUIRE(params && x && eloc && N > 0 && M > 0 && n >= 0, "rbm_eloc_ising arguments");
  VMCK_REQUIRE(n_edges == 0 || edges, "edges");
  if (n == 0) return VMCK_OK;
  if (dtype == VMCK_F64)
    return launch_eloc_ising<double>(as_stream(s), params, N, M, x, n, edges, n_edges, h, J,
                                     eloc, logpsi_out);
  if (dtype == VMCK_F32)
    return launch_eloc_ising<float>(as_stream(s), params, N, M, x, n, edges, n_edges, h, J, eloc,
                                    logpsi_out);
  set_last_error("rbm_eloc_ising: dtype %d unsupported", dtype);
  return VMCK_ERR_UNSUPPORTED;
}

extern "C" int vmck_rbm_eloc_local(vmck_stream s, int32_t dtype, const void *params, int32_t N,
                                   int32_t M, const int8_t *x, int64_t n, const vmck_local_op *op,
                                   double *eloc, void *logpsi_out) {
  VMCK_REQUIRE(params && x && eloc && op && N > 0 && M > 0 && n >= 0, "rbm_eloc_local arguments");
  int rc = validate_local_op(*op);
  if (rc) return rc;
  VMCK_REQUIRE(op->n_sites == N, "operator and model sizes differ");
  if (n == 0) return VMCK_OK;
  if (dtype == VMCK_F64)
    return launch_eloc_local<double>(as_stream(s), params, N, M, x, n, *op, eloc, logpsi_out);
  if (dtype == VMCK_F32)
    return launch_eloc_local<float>(as_stream(s), params, N, M, x, n, *op, eloc, logpsi_out);
  set_last_error("rbm_eloc_local: dtype %d unsupported", dtype);
  return VMCK_ERR_UNSUPPORTED;
}

static int64_t ot_chunk(int64_t n) { return 1024; }

extern "C" int64_t vmck_ot_v_workspace_size(int32_t N, int32_t M, int64_t n) {
  int64_t P = (int64_t)M + (int64_t)N * M + N;
  int64_t nchunk = (n + ot_chunk(n) - 1) / ot_chunk(n);
  if (nchunk < 1) nchunk = 1;
  return nchunk * P;
}

extern "C" int vmck_rbm_ot_v(vmck_stream s, int32_t dtype, const void *tanh_theta,
                             const int8_t *x, int32_t N, int32_t M, int64_t n, const double *v,
                             double *out, double *workspace, int64_t workspace_len) {
  VMCK_REQUIRE(tanh_theta && x && v && out && workspace && N > 0 && M > 0 && n > 0,
               "rbm_ot_v arguments");
  VMCK_REQUIRE(workspace_len >= vmck_ot_v_workspace_size(N, M, n), "rbm_ot_v workspace too small");
  const int64_t chunk = ot_chunk(n);
  const int nchunk = (int)((n + chunk - 1) / chunk);
  dim3 grid((M + OT_TJ - 1) / OT_TJ, (N + OT_TI - 1) / OT_TI, nchunk);
  cudaStream_t st = as_stream(s);
  if (dtype == VMCK_F64)
    ot_v_partial_kernel<double><<<grid, 256, 0, st>>>(static_cast<const double *>(tanh_theta), x,
                                                      N, M, n, chunk, v, workspace);
  else if (dtype == VMCK_F32)
    ot_v_partial_kernel<float><<<grid, 256, 0, st>>>(static_cast<const float *>(tanh_theta), x, N,
                                                     M, n, chunk, v, workspace);
  else {
    set_last_error("rbm_ot_v: dtype %d unsupported", dtype);
    return VMCK_ERR_UNSUPPORTED;
  }
  int rc = check_launch("rbm_ot_v partial");
  if (rc) return rc;
  const int64_t P = (int64_t)M + (int64_t)N * M + N;
  reduce_chunks_kernel<<<ceil_div(P, 256), 256, 0, st>>>(workspace, P, nchunk, out);
  return check_launch("rbm_ot_v reduce");
}

extern "C" int vmck_rbm_jacobian(vmck_stream s, int32_t dtype, const void *tanh_theta,
                                 const int8_t *x, int32_t N, int32_t M, int64_t n,
                                 const double *col_mean, double scale, int32_t out_dtype,
                                 void *O) {
  VMCK_REQUIRE(tanh_theta && x && col_mean && O && N > 0 && M > 0 && n > 0,
               "rbm_jacobian arguments");
  unsigned grid = (unsigned)std::min<int64_t>(n, (int64_t)num_sms() * 16);
  cudaStream_t st = as_stream(s);
  if (dtype == VMCK_F64 && out_dtype == VMCK_F64)
    jacobian_kernel<double, double><<<grid, 256, 0, st>>>(static_cast<const double *>(tanh_theta),
                                                          x, N, M, n, col_mean, scale,
                                                          static_cast<double *>(O));
  else if (dtype == VMCK_F32 && out_dtype == VMCK_F32)
    jacobian_kernel<float, float><<<grid, 256, 0, st>>>(static_cast<const float *>(tanh_theta), x,
                                                        N, M, n, col_mean, scale,
                                                        static_cast<float *>(O));
  else if (dtype == VMCK_F64 && out_dtype == VMCK_F32)
    jacobian_kernel<double, float><<<grid, 256, 0, st>>>(static_cast<const double *>(tanh_theta),
                                                         x, N, M, n, col_mean, scale,
                                                         static_cast<float *>(O));
  else {
    set_last_error("rbm_jacobian: dtype pair unsupported");
    return VMCK_ERR_UNSUPPORTED;
  }
  return check_launch("rbm_jacobian");
}

extern "C" int vmck_batched_eloc_ising(vmck_stream s, int32_t dtype, const vmck_batch_ising *inst,
                                       int32_t n_inst, const int32_t *work, int32_t n_items,
                                       int32_t samples_per_item, int32_t *queue, int32_t max_N,
                                       int32_t max_M, int32_t n_ctas) {
  VMCK_REQUIRE(inst && work && queue && n_inst > 0 && n_items >= 0 && samples_per_item > 0 &&
                   max_N > 0 && max_M > 0 && n_ctas > 0,
               "batched_eloc_ising arguments");
  cudaStream_t st = as_stream(s);
  VMCK_CUDA(cudaMemsetAsync(queue, 0, sizeof(int32_t), st));
  const size_t es = dtype == VMCK_F64 ? 8 : 4;
  const size_t smem = 2 * es * (size_t)max_M + align16(max_N);
  VMCK_REQUIRE(smem <= 200 * 1024, "batched_eloc_ising: max_M too large");
  if (dtype == VMCK_F32) {
    VMCK_CUDA(cudaFuncSetAttribute(batched_eloc_ising_kernel<float>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    batched_eloc_ising_kernel<float><<<n_ctas, EL_THREADS, smem, st>>>(
        inst, work, n_items, queue, samples_per_item, max_M);
  } else if (dtype == VMCK_F64) {
    VMCK_CUDA(cudaFuncSetAttribute(batched_eloc_ising_kernel<double>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    batched_eloc_ising_kernel<double><<<n_ctas, EL_THREADS, smem, st>>>(
        inst, work, n_items, queue, samples_per_item, max_M);
  } else {
    set_last_error("batched_eloc_ising: dtype %d unsupported", dtype);
    return VMCK_ERR_UNSUPPORTED;
  }
  return check_launch("batched_eloc_ising");
}

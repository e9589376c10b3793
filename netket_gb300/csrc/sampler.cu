// Metropolis sweeps for the RBM with Local and Exchange transition rules.
//
// One warp owns one chain for the whole launch (all discarded and kept
// sweeps).  Per chain the warp keeps in shared memory: the configuration
// x (N int8), theta = b + x W (M), log_cosh(theta) (M) and the proposal's
// theta' / log_cosh(theta') (2M).  A proposal changing sites {u (, v)} costs
// M log_cosh evaluations and 1-2 FMAs per hidden unit -- instead of the full
// N*M forward pass NetKet's sampler runs per proposal
// (netket/sampler/metropolis.py:438).  theta is recomputed exactly at the start
// of every sweep, so incremental rounding never builds up over more than one
// sweep.
//
// Acceptance follows netket/sampler/metropolis.py:440-450:
//   accept iff u < exp(2 Re[logpsi(x') - logpsi(x)] + corr).
// Exchange (netket/sampler/rules/exchange.py:143-184): pick uniformly among the
// clusters (u, v) with x_u != x_v, swap, corr = log #hoppable(x) - log #hoppable(x').
// With no hoppable cluster the proposal is x itself with a NaN correction in
// NetKet, which is never accepted; here it is rejected directly.
#include <algorithm>
#include <cstdlib>

#include "common.cuh"

namespace vmck {

template <typename T>
struct ChainSmem {
  T *th, *lc, *tn, *ln;
  int8_t *xs;
};

template <typename T>
__device__ inline void chain_recompute(const T *__restrict__ b, const T *__restrict__ W,
                                       const T *__restrict__ a, int N, int M, ChainSmem<T> c,
                                       T *logpsi) {
  const int lane = threadIdx.x & 31;
  T part = 0;
  for (int j = lane; j < M; j += 32) {
    T acc = b[j];
    for (int i = 0; i < N; ++i) acc += (T)c.xs[i] * W[(int64_t)i * M + j];
    c.th[j] = acc;
    T l = log_cosh_fast(acc);
    c.lc[j] = l;
    part += l;
  }
  for (int i = lane; i < N; i += 32) part += (T)c.xs[i] * a[i];
  part = warp_sum(part);
  *logpsi = part;
  __syncwarp();
}

// One chain, driven by one warp: n_discard + L sweeps of `sweep` proposals,
// the state after each of the last L sweeps written to samples_chain (L x N).
// b is the chain's index in its problem: it keys the Philox stream.
template <typename T, int RULE>
__device__ void run_chain(const T *__restrict__ params, int N, int M, int8_t *sigma_row,
                          double *log_prob_b, int64_t *n_accepted_b, int b, int sweep,
                          int n_discard, int L, int8_t *samples_chain, uint32_t k0, uint32_t k1,
                          uint64_t counter, const int16_t *cl, int C, ChainSmem<T> c) {
  const int lane = threadIdx.x & 31;
  const T *bvec = params, *W = params + M, *a = params + M + (int64_t)N * M;
  for (int i = lane; i < N; i += 32) c.xs[i] = sigma_row[i];
  __syncwarp();
  T logpsi;
  int hop = 0;
  if (RULE == 1) {
    for (int q0 = 0; q0 < C; q0 += 32) {
      int q = q0 + lane;
      bool h = q < C && c.xs[cl[2 * q]] != c.xs[cl[2 * q + 1]];
      hop += __popc(__ballot_sync(0xffffffffu, h));
    }
  }
  int64_t acc_count = 0;
  const int total = n_discard + L;
  for (int step = 0; step < total; ++step) {
    chain_recompute(bvec, W, a, N, M, c, &logpsi);
    for (int p = 0; p < sweep; ++p) {
      const uint64_t pidx = counter + (uint64_t)step * sweep + p;
      u32x4 r = philox4x32_10(u32x4{(uint32_t)pidx, (uint32_t)(pidx >> 32), (uint32_t)b, 0u}, k0, k1);
      int su, sv = -1;
      T du, dv = 0;
      T corr = 0;
      int hop_new = hop;
      if (RULE == 0) {
        su = (int)below(r.x, (uint32_t)N);
        du = (T)(-2 * c.xs[su]);
      } else {
        if (hop == 0) continue;  // no move possible: rejected (see header)
        int k = (int)below(r.x, (uint32_t)hop);
        int pick = -1;
        for (int q0 = 0; q0 < C && pick < 0; q0 += 32) {
          int q = q0 + lane;
          bool h = q < C && c.xs[cl[2 * q]] != c.xs[cl[2 * q + 1]];
          unsigned m = __ballot_sync(0xffffffffu, h);
          int pc = __popc(m);
          if (k < pc) {
            for (int z = 0; z < k; ++z) m &= m - 1;
            pick = q0 + __ffs(m) - 1;
          } else {
            k -= pc;
          }
        }
        if (pick < 0) continue;  // unreachable while hop is consistent; never index out of range
        su = cl[2 * pick];
        sv = cl[2 * pick + 1];
        const int8_t xu = c.xs[su], xv = c.xs[sv];
        du = (T)(xv - xu);
        dv = (T)(xu - xv);
        // hoppable count of the proposed configuration
        __syncwarp();
        if (lane == 0) {
          c.xs[su] = xv;
          c.xs[sv] = xu;
        }
        __syncwarp();
        hop_new = 0;
        for (int q0 = 0; q0 < C; q0 += 32) {
          int q = q0 + lane;
          bool h = q < C && c.xs[cl[2 * q]] != c.xs[cl[2 * q + 1]];
          hop_new += __popc(__ballot_sync(0xffffffffu, h));
        }
        __syncwarp();
        if (lane == 0) {
          c.xs[su] = xu;
          c.xs[sv] = xv;
        }
        __syncwarp();
        corr = log((T)hop) - log((T)hop_new);
      }
      // log-ratio of the RBM amplitude
      T s = 0;
      const T *Wu = W + (int64_t)su * M;
      const T *Wv = (sv >= 0) ? W + (int64_t)sv * M : Wu;
      for (int j = lane; j < M; j += 32) {
        T t = c.th[j] + du * Wu[j];
        if (RULE == 1) t += dv * Wv[j];
        T l = log_cosh_fast(t);
        c.tn[j] = t;
        c.ln[j] = l;
        s += l - c.lc[j];
      }
      s = warp_sum(s);
      s += du * a[su];
      if (RULE == 1) s += dv * a[sv];
      const T dlp = (T)2 * s;
      bool accept;
      if (sizeof(T) == 8) {
        double u = u01d(r.y, r.z);
        accept = u < exp((double)(dlp + corr));
      } else {
        float u = u01f(r.y);
        accept = u < expf((float)(dlp + corr));
      }
      if (accept) {
        for (int j = lane; j < M; j += 32) {
          c.th[j] = c.tn[j];
          c.lc[j] = c.ln[j];
        }
        __syncwarp();
        if (lane == 0) {
          c.xs[su] = (int8_t)(c.xs[su] + (int)du);
          if (RULE == 1) c.xs[sv] = (int8_t)(c.xs[sv] + (int)dv);
        }
        hop = hop_new;
        logpsi += s;
        ++acc_count;
      }
      __syncwarp();
    }
    if (step >= n_discard) {
      int8_t *dst = samples_chain + (int64_t)(step - n_discard) * N;
      for (int i = lane; i < N; i += 32) dst[i] = c.xs[i];
    }
  }
  chain_recompute(bvec, W, a, N, M, c, &logpsi);
  for (int i = lane; i < N; i += 32) sigma_row[i] = c.xs[i];
  if (lane == 0) {
    *log_prob_b = 2.0 * (double)logpsi;
    *n_accepted_b += acc_count;
  }
}

template <typename T, int RULE>
__global__ void metropolis_kernel(const T *__restrict__ params, int N, int M, int8_t *sigma,
                                  double *log_prob, int64_t *n_accepted, int B, int sweep,
                                  int n_discard, int L, int8_t *samples, uint32_t k0, uint32_t k1,
                                  uint64_t counter, const int32_t *__restrict__ clusters, int C,
                                  int wpb) {
  extern __shared__ unsigned char smem_raw[];
  int16_t *cl = reinterpret_cast<int16_t *>(smem_raw);
  unsigned char *base = smem_raw + ((4 * (size_t)C + 15) & ~size_t(15));
  const int warp = threadIdx.x >> 5;
  const size_t per_warp = 4 * (size_t)M * sizeof(T) + ((N + 15) & ~15);
  ChainSmem<T> c;
  c.th = reinterpret_cast<T *>(base + warp * per_warp);
  c.lc = c.th + M;
  c.tn = c.lc + M;
  c.ln = c.tn + M;
  c.xs = reinterpret_cast<int8_t *>(c.ln + M);
  if (RULE == 1)
    for (int q = threadIdx.x; q < 2 * C; q += blockDim.x) cl[q] = (int16_t)clusters[q];
  __syncthreads();
  const int b = blockIdx.x * wpb + warp;
  if (b >= B) return;
  run_chain<T, RULE>(params, N, M, sigma + (int64_t)b * N, log_prob + b, n_accepted + b, b, sweep,
                     n_discard, L, samples + (int64_t)b * L * N, k0, k1, counter, cl, C, c);
}

// Persistent batched sampler: CTAs pull (instance, first chain) items.
template <typename T>
__global__ void batched_metropolis_kernel(const vmck_batch_chains *__restrict__ inst,
                                          const int32_t *__restrict__ work, int n_items,
                                          int32_t *queue, int n_discard, int L, int max_N,
                                          int max_M) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ int item_s;
  const int warp = threadIdx.x >> 5;
  const size_t per_warp = 4 * (size_t)max_M * sizeof(T) + ((max_N + 15) & ~15);
  unsigned char *mine = smem_raw + warp * per_warp;
  while (true) {
    if (threadIdx.x == 0) item_s = atomicAdd(queue, 1);
    __syncthreads();
    const int item = item_s;
    __syncthreads();
    if (item >= n_items) break;
    const int i = work[2 * item];
    const vmck_batch_chains I = inst[i];
    const int b = work[2 * item + 1] + warp;
    if (b < I.n_chains) {
      ChainSmem<T> c;
      c.th = reinterpret_cast<T *>(mine);
      c.lc = c.th + I.M;
      c.tn = c.lc + I.M;
      c.ln = c.tn + I.M;
      c.xs = reinterpret_cast<int8_t *>(c.ln + I.M);
      run_chain<T, 0>(static_cast<const T *>(I.params), I.N, I.M, I.sigma + (int64_t)b * I.N,
                      I.log_prob + b, I.n_accepted + b, b, I.sweep_size, n_discard, L,
                      I.samples + (int64_t)b * L * I.N, (uint32_t)I.seed,
                      (uint32_t)(I.seed >> 32), I.counter, nullptr, 0, c);
    }
  }
}

__global__ void batch_advance_counters_kernel(vmck_batch_chains *inst, int n_inst, int steps) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_inst) inst[i].counter += (uint64_t)steps * (uint64_t)inst[i].sweep_size;
}

// ------------------------------------------------------------ Exchange, W in smem
// Exchange-rule sweeps for an FP32 RBM whose parameters fit in shared memory:
// the CTA stages W, b, a once; one warp drives one chain with theta and
// log_cosh(theta) in registers (lane l holds hidden units l + 32 r).  The set of
// hoppable clusters (x_u != x_v) is a per-chain bitmask in shared memory, so a
// proposal picks the k-th hoppable cluster with a warp scan of the word counts
// and updates the hoppable count from the clusters incident to the two swapped
// sites (incidence lists built in shared memory; sites with more than 16
// incident clusters fall back to a full recount).  Random stream, proposal
// order and every floating-point expression match metropolis_kernel<float, 1>,
// so the samples are identical.
constexpr int XS_MAXDEG = 16;

__device__ __forceinline__ int warp_sum_int(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

constexpr int XS_MAX_WARPS = 28;  // 896 threads: 73 registers per thread

// Position of the n-th (0-based) set bit of v, which has more than n set bits:
// a bisection on popcounts of the low half, quarter, ... of what is left.
__device__ __forceinline__ int nth_set_bit(uint32_t v, int n) {
  int pos = 0, c = __popc(v & 0xFFFFu);
  if (n >= c) { n -= c; pos += 16; v >>= 16; }
  c = __popc(v & 0xFFu);
  if (n >= c) { n -= c; pos += 8; v >>= 8; }
  c = __popc(v & 0xFu);
  if (n >= c) { n -= c; pos += 4; v >>= 4; }
  c = __popc(v & 0x3u);
  if (n >= c) { n -= c; pos += 2; v >>= 2; }
  if (n >= (int)(v & 1u)) pos += 1;
  return pos;
}

template <int R>
__global__ void __launch_bounds__(32 * XS_MAX_WARPS, 1) metropolis_exchange_smem_kernel(
    const float *__restrict__ params, int N, int M, int8_t *sigma, double *log_prob,
    int64_t *n_accepted, int B, int sweep, int n_discard, int L, int8_t *samples, uint32_t k0,
    uint32_t k1, uint64_t counter, const int32_t *__restrict__ clusters, int C, int wpb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nwords = (C + 31) >> 5;
  float *Ws = reinterpret_cast<float *>(smem_raw);                    // N x M
  float *bs = Ws + (size_t)N * M;                                     // M
  float *as = bs + M;                                                 // N
  float *logtab = as + N;                                             // C + 1
  int16_t *cl = reinterpret_cast<int16_t *>(logtab + C + 1);          // 2C
  int16_t *inc = cl + 2 * C;                                          // N x XS_MAXDEG
  int *deg = reinterpret_cast<int *>(                                 // N
      (reinterpret_cast<uintptr_t>(inc + (size_t)N * XS_MAXDEG) + 3) & ~uintptr_t(3));
  __shared__ int overflow;
  unsigned char *per_warp_base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(deg + N) + 15) & ~uintptr_t(15));
  const size_t per_warp = (((size_t)N + 15) & ~size_t(15)) + 4 * (size_t)nwords;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  {  // stage the parameters, clusters and incidence lists
    const float *Wg = params + M;
    for (int64_t e = tid; e < (int64_t)N * M; e += blockDim.x) Ws[e] = Wg[e];
    for (int j = tid; j < M; j += blockDim.x) bs[j] = params[j];
    for (int i = tid; i < N; i += blockDim.x) {
      as[i] = params[M + (int64_t)N * M + i];
      deg[i] = 0;
    }
    for (int k = tid; k <= C; k += blockDim.x) logtab[k] = logf((float)k);
    for (int q = tid; q < 2 * C; q += blockDim.x) cl[q] = (int16_t)clusters[q];
    if (tid == 0) overflow = 0;
    __syncthreads();
    for (int q = tid; q < C; q += blockDim.x) {
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int site = cl[2 * q + e];
        const int pos = atomicAdd(&deg[site], 1);
        if (pos < XS_MAXDEG) inc[site * XS_MAXDEG + pos] = (int16_t)q;
        else overflow = 1;
      }
    }
    __syncthreads();
  }
  const bool full_recount = overflow != 0;
  const int b = blockIdx.x * wpb + warp;
  if (b >= B) return;
  int8_t *xs = reinterpret_cast<int8_t *>(per_warp_base + warp * per_warp);
  uint32_t *mask = reinterpret_cast<uint32_t *>(xs + ((N + 15) & ~15));
  int8_t *sigma_row = sigma + (int64_t)b * N;
  for (int i = lane; i < N; i += 32) xs[i] = sigma_row[i];
  __syncwarp();
  // hoppable bitmask and count
  int hop = 0;
  for (int w = lane; w < nwords; w += 32) {
    uint32_t bits = 0u;
    for (int t = 0; t < 32; ++t) {
      const int q = 32 * w + t;
      if (q < C && xs[cl[2 * q]] != xs[cl[2 * q + 1]]) bits |= 1u << t;
    }
    mask[w] = bits;
    hop += __popc(bits);
  }
  hop = warp_sum_int(hop);
  __syncwarp();
  float th[R], lc[R];
  float logpsi = 0.0f;
  auto recompute = [&]() {
    float part = 0.0f;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int j = lane + 32 * r;
      if (j < M) {
        float acc = bs[j];
        for (int i = 0; i < N; ++i) acc += (float)xs[i] * Ws[i * M + j];
        th[r] = acc;
        const float l = log_cosh_fast(acc);
        lc[r] = l;
        part += l;
      }
    }
    for (int i = lane; i < N; i += 32) part += (float)xs[i] * as[i];
    logpsi = warp_sum(part);
    __syncwarp();
  };
  int64_t acc_count = 0;
  const int total = n_discard + L;
  for (int step = 0; step < total; ++step) {
    recompute();
    for (int p = 0; p < sweep; ++p) {
      const uint64_t pidx = counter + (uint64_t)step * sweep + p;
      u32x4 rr = philox4x32_10(u32x4{(uint32_t)pidx, (uint32_t)(pidx >> 32), (uint32_t)b, 0u}, k0, k1);
      if (hop == 0) continue;  // no move possible: rejected
      // the k-th hoppable cluster in cluster order
      int k = (int)below(rr.x, (uint32_t)hop);
      const uint32_t wbits = lane < nwords ? mask[lane] : 0u;
      const int cnt = __popc(wbits);
      int incl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      const int excl = incl - cnt;
      const bool owner = excl <= k && k < incl;
      const unsigned ob = __ballot_sync(0xffffffffu, owner);
      if (ob == 0u) continue;  // unreachable while hop matches the mask
      const int src = __ffs(ob) - 1;
      int pick = -1;
      if (owner) pick = 32 * lane + nth_set_bit(wbits, k - excl);
      pick = __shfl_sync(0xffffffffu, pick, src);
      if (pick < 0 || pick >= C) continue;  // likewise unreachable; never index out of range
      const int su = cl[2 * pick], sv = cl[2 * pick + 1];
      const int8_t xu = xs[su], xv = xs[sv];
      const float du = (float)(xv - xu), dv = (float)(xu - xv);
      // change of the hoppable count: clusters incident to su (lanes 0-15) or sv
      // (lanes 16-31, skipping those that also touch su)
      int q = -1, newh = 0;
      int hop_new;
      if (!full_recount) {
        const int site = lane < 16 ? su : sv, slot = lane & 15;
        if (slot < deg[site]) {
          q = inc[site * XS_MAXDEG + slot];
          const int a0 = cl[2 * q], a1 = cl[2 * q + 1];
          if (lane >= 16 && (a0 == su || a1 == su)) q = -1;
          if (q >= 0) {
            const int8_t x0 = a0 == su ? xv : (a0 == sv ? xu : xs[a0]);
            const int8_t x1 = a1 == su ? xv : (a1 == sv ? xu : xs[a1]);
            newh = x0 != x1;
          }
        }
        const int oldh = q >= 0 ? (int)((mask[q >> 5] >> (q & 31)) & 1u) : 0;
        hop_new = hop + warp_sum_int(q >= 0 ? newh - oldh : 0);
      } else {
        int h2 = 0;
        for (int q0 = 0; q0 < C; q0 += 32) {
          const int qq = q0 + lane;
          if (qq < C) {
            const int a0 = cl[2 * qq], a1 = cl[2 * qq + 1];
            const int8_t x0 = a0 == su ? xv : (a0 == sv ? xu : xs[a0]);
            const int8_t x1 = a1 == su ? xv : (a1 == sv ? xu : xs[a1]);
            h2 += x0 != x1;
          }
        }
        hop_new = warp_sum_int(h2);
      }
      const float corr = logtab[hop] - logtab[hop_new];
      // log-ratio of the RBM amplitude
      float sacc = 0.0f;
      const float *Wu = Ws + su * M, *Wv = Ws + sv * M;
      float ln[R];  // log_cosh of the proposal, kept for an accepted move
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int j = lane + 32 * r;
        ln[r] = 0.0f;
        if (j < M) {
          float t = th[r] + du * Wu[j];
          t += dv * Wv[j];
          const float l = log_cosh_fast(t);
          ln[r] = l;
          sacc += l - lc[r];
        }
      }
      float s = warp_sum(sacc);
      s += du * as[su];
      s += dv * as[sv];
      const float dlp = 2.0f * s;
      const float u = u01f(rr.y);
      if (u < expf(dlp + corr)) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int j = lane + 32 * r;
          if (j < M) {
            float t = th[r] + du * Wu[j];
            t += dv * Wv[j];
            th[r] = t;
            lc[r] = ln[r];
          }
        }
        __syncwarp();
        if (lane == 0) {
          xs[su] = (int8_t)(xu + (int)du);
          xs[sv] = (int8_t)(xv + (int)dv);
        }
        if (!full_recount) {
          if (q >= 0) {
            const uint32_t bit = 1u << (q & 31);
            if (newh) atomicOr(&mask[q >> 5], bit);
            else atomicAnd(&mask[q >> 5], ~bit);
          }
        } else {
          __syncwarp();
          for (int w = lane; w < nwords; w += 32) {
            uint32_t bits = 0u;
            for (int t = 0; t < 32; ++t) {
              const int qq = 32 * w + t;
              if (qq < C && xs[cl[2 * qq]] != xs[cl[2 * qq + 1]]) bits |= 1u << t;
            }
            mask[w] = bits;
          }
        }
        hop = hop_new;
        logpsi += s;
        ++acc_count;
      }
      __syncwarp();
    }
    if (step >= n_discard) {
      int8_t *dst = samples + ((int64_t)b * L + (step - n_discard)) * N;
      for (int i = lane; i < N; i += 32) dst[i] = xs[i];
    }
  }
  recompute();
  for (int i = lane; i < N; i += 32) sigma_row[i] = xs[i];
  if (lane == 0) {
    log_prob[b] = 2.0 * (double)logpsi;
    n_accepted[b] += acc_count;
  }
}

// ------------------------------------------------------------ Exchange, W in L2
// The same chain for hidden layers too wide for shared-memory weights (N M >
// ~48 K): W, b, a are read through L2 (2 MB for N = 256, M = 2048) and theta
// lives in the warp's shared memory (M floats); log_cosh(theta) is recomputed
// where it is needed instead of stored (the same function of the same value,
// so the same bits), and an accepted move recomputes theta'.  A chain then
// holds ~8.3 KB of shared memory and few registers: 24 chains per SM at
// M = 2048, where metropolis_kernel's four M-vectors leave 4 (a version with
// theta in registers, 64 per lane, was register-bound at 16 and stalled on the
// L2 loads of W: 25 % warps active).  Warps loop over chains (b += gridDim.x
// wpb).  Random stream, proposal order and every floating-point expression
// match metropolis_kernel<float, 1>, so the samples are identical.
constexpr int XL_WARPS = 24;

__global__ void __launch_bounds__(32 * XL_WARPS, 1) metropolis_exchange_l2_kernel(
    const float *__restrict__ params, int N, int M, int8_t *sigma, double *log_prob,
    int64_t *n_accepted, int B, int sweep, int n_discard, int L, int8_t *samples, uint32_t k0,
    uint32_t k1, uint64_t counter, const int32_t *__restrict__ clusters, int C) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nwords = (C + 31) >> 5;
  const float *Wg = params + M, *bg = params, *ag = params + M + (int64_t)N * M;
  float *logtab = reinterpret_cast<float *>(smem_raw);                // C + 1
  int16_t *cl = reinterpret_cast<int16_t *>(logtab + C + 1);          // 2C
  int16_t *inc = cl + 2 * C;                                          // N x XS_MAXDEG
  int *deg = reinterpret_cast<int *>(                                 // N
      (reinterpret_cast<uintptr_t>(inc + (size_t)N * XS_MAXDEG) + 3) & ~uintptr_t(3));
  __shared__ int overflow;
  unsigned char *per_warp_base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(deg + N) + 15) & ~uintptr_t(15));
  const size_t per_warp = 4 * (size_t)M + (((size_t)N + 15) & ~size_t(15)) + 4 * (size_t)nwords;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wpb = (int)(blockDim.x >> 5);
  {  // clusters and incidence lists
    for (int i = tid; i < N; i += blockDim.x) deg[i] = 0;
    for (int k = tid; k <= C; k += blockDim.x) logtab[k] = logf((float)k);
    for (int q = tid; q < 2 * C; q += blockDim.x) cl[q] = (int16_t)clusters[q];
    if (tid == 0) overflow = 0;
    __syncthreads();
    for (int q = tid; q < C; q += blockDim.x) {
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int site = cl[2 * q + e];
        const int pos = atomicAdd(&deg[site], 1);
        if (pos < XS_MAXDEG) inc[site * XS_MAXDEG + pos] = (int16_t)q;
        else overflow = 1;
      }
    }
    __syncthreads();
  }
  const bool full_recount = overflow != 0;
  float *ths = reinterpret_cast<float *>(per_warp_base + warp * per_warp);  // theta, M
  int8_t *xs = reinterpret_cast<int8_t *>(ths + M);
  uint32_t *mask = reinterpret_cast<uint32_t *>(xs + ((N + 15) & ~15));
  for (int b = blockIdx.x * wpb + warp; b < B; b += gridDim.x * wpb) {
    int8_t *sigma_row = sigma + (int64_t)b * N;
    __syncwarp();
    for (int i = lane; i < N; i += 32) xs[i] = sigma_row[i];
    __syncwarp();
    int hop = 0;
    for (int w = lane; w < nwords; w += 32) {
      uint32_t bits = 0u;
      for (int t = 0; t < 32; ++t) {
        const int q = 32 * w + t;
        if (q < C && xs[cl[2 * q]] != xs[cl[2 * q + 1]]) bits |= 1u << t;
      }
      mask[w] = bits;
      hop += __popc(bits);
    }
    hop = warp_sum_int(hop);
    __syncwarp();
    float logpsi = 0.0f;
    auto recompute = [&]() {
      float part = 0.0f;
      for (int j = lane; j < M; j += 32) {
        float acc = __ldg(bg + j);
        for (int i = 0; i < N; ++i) acc += (float)xs[i] * __ldg(Wg + (int64_t)i * M + j);
        ths[j] = acc;
        part += log_cosh_fast(acc);
      }
      for (int i = lane; i < N; i += 32) part += (float)xs[i] * __ldg(ag + i);
      logpsi = warp_sum(part);
      __syncwarp();
    };
    int64_t acc_count = 0;
    const int total = n_discard + L;
    for (int step = 0; step < total; ++step) {
      recompute();
      for (int p = 0; p < sweep; ++p) {
        const uint64_t pidx = counter + (uint64_t)step * sweep + p;
        u32x4 rr = philox4x32_10(u32x4{(uint32_t)pidx, (uint32_t)(pidx >> 32), (uint32_t)b, 0u},
                                 k0, k1);
        if (hop == 0) continue;  // no move possible: rejected
        int k = (int)below(rr.x, (uint32_t)hop);
        const uint32_t wbits = lane < nwords ? mask[lane] : 0u;
        const int cnt = __popc(wbits);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += v;
        }
        const int excl = incl - cnt;
        const bool owner = excl <= k && k < incl;
        const unsigned ob = __ballot_sync(0xffffffffu, owner);
        if (ob == 0u) continue;  // unreachable while hop matches the mask
        const int src = __ffs(ob) - 1;
        int pick = -1;
        if (owner) pick = 32 * lane + nth_set_bit(wbits, k - excl);
        pick = __shfl_sync(0xffffffffu, pick, src);
        if (pick < 0 || pick >= C) continue;  // likewise unreachable; never out of range
        const int su = cl[2 * pick], sv = cl[2 * pick + 1];
        const int8_t xu = xs[su], xv = xs[sv];
        const float du = (float)(xv - xu), dv = (float)(xu - xv);
        int q = -1, newh = 0;
        int hop_new;
        if (!full_recount) {
          const int site = lane < 16 ? su : sv, slot = lane & 15;
          if (slot < deg[site]) {
            q = inc[site * XS_MAXDEG + slot];
            const int a0 = cl[2 * q], a1 = cl[2 * q + 1];
            if (lane >= 16 && (a0 == su || a1 == su)) q = -1;
            if (q >= 0) {
              const int8_t x0 = a0 == su ? xv : (a0 == sv ? xu : xs[a0]);
              const int8_t x1 = a1 == su ? xv : (a1 == sv ? xu : xs[a1]);
              newh = x0 != x1;
            }
          }
          const int oldh = q >= 0 ? (int)((mask[q >> 5] >> (q & 31)) & 1u) : 0;
          hop_new = hop + warp_sum_int(q >= 0 ? newh - oldh : 0);
        } else {
          int h2 = 0;
          for (int q0 = 0; q0 < C; q0 += 32) {
            const int qq = q0 + lane;
            if (qq < C) {
              const int a0 = cl[2 * qq], a1 = cl[2 * qq + 1];
              const int8_t x0 = a0 == su ? xv : (a0 == sv ? xu : xs[a0]);
              const int8_t x1 = a1 == su ? xv : (a1 == sv ? xu : xs[a1]);
              h2 += x0 != x1;
            }
          }
          hop_new = warp_sum_int(h2);
        }
        const float corr = logtab[hop] - logtab[hop_new];
        float sacc = 0.0f;
        const float *Wu = Wg + (int64_t)su * M, *Wv = Wg + (int64_t)sv * M;
#pragma unroll 8
        for (int j = lane; j < M; j += 32) {
          const float th = ths[j];
          float t = th + du * __ldg(Wu + j);
          t += dv * __ldg(Wv + j);
          sacc += log_cosh_fast(t) - log_cosh_fast(th);
        }
        float s = warp_sum(sacc);
        s += du * __ldg(ag + su);
        s += dv * __ldg(ag + sv);
        const float dlp = 2.0f * s;
        const float u = u01f(rr.y);
        if (u < expf(dlp + corr)) {
#pragma unroll 8
          for (int j = lane; j < M; j += 32) {
            float t = ths[j] + du * __ldg(Wu + j);
            t += dv * __ldg(Wv + j);
            ths[j] = t;
          }
          __syncwarp();
          if (lane == 0) {
            xs[su] = (int8_t)(xu + (int)du);
            xs[sv] = (int8_t)(xv + (int)dv);
          }
          if (!full_recount) {
            if (q >= 0) {
              const uint32_t bit = 1u << (q & 31);
              if (newh) atomicOr(&mask[q >> 5], bit);
              else atomicAnd(&mask[q >> 5], ~bit);
            }
          } else {
            __syncwarp();
            for (int w = lane; w < nwords; w += 32) {
              uint32_t bits = 0u;
              for (int t = 0; t < 32; ++t) {
                const int qq = 32 * w + t;
                if (qq < C && xs[cl[2 * qq]] != xs[cl[2 * qq + 1]]) bits |= 1u << t;
              }
              mask[w] = bits;
            }
          }
          hop = hop_new;
          logpsi += s;
          ++acc_count;
        }
        __syncwarp();
      }
      if (step >= n_discard) {
        int8_t *dst = samples + ((int64_t)b * L + (step - n_discard)) * N;
        for (int i = lane; i < N; i += 32) dst[i] = xs[i];
      }
    }
    recompute();
    for (int i = lane; i < N; i += 32) sigma_row[i] = xs[i];
    if (lane == 0) {
      log_prob[b] = 2.0 * (double)logpsi;
      n_accepted[b] += acc_count;
    }
  }
}

static size_t exchange_l2_smem_bytes(int N, int M, int C, int wpb) {
  const int nwords = (C + 31) >> 5;
  size_t bytes = (size_t)(C + 1) * 4 + (size_t)C * 4 + (size_t)N * XS_MAXDEG * 2 + 4 +
                 (size_t)N * 4 + 16;
  bytes += (size_t)wpb * (4 * (size_t)M + (((size_t)N + 15) & ~size_t(15)) + 4 * (size_t)nwords);
  return bytes + 64;
}

// Dynamic shared memory a block may use on this GPU (227 KB on sm_100 / sm_103),
// less the kernel's static variable.
constexpr size_t XL_SMEM_MAX = 227 * 1024 - 64;

// Chains per block of the L2 kernel: as many as fit (at most XL_WARPS), 0 if
// fewer than 4 do.
static int exchange_l2_warps(int N, int M, int C) {
  int w = XL_WARPS;
  while (w >= 4 && exchange_l2_smem_bytes(N, M, C, w) > XL_SMEM_MAX) --w;
  return w >= 4 ? w : 0;
}

static int launch_exchange_l2(cudaStream_t st, const float *p, int N, int M, int8_t *sigma,
                              double *log_prob, int64_t *n_acc, int B, int sweep, int n_discard,
                              int L, int8_t *samples, uint32_t k0, uint32_t k1, uint64_t counter,
                              const int32_t *clusters, int C, int sms) {
  const int wpb = exchange_l2_warps(N, M, C);
  VMCK_REQUIRE(wpb >= 4, "exchange L2 kernel: M too large");
  const size_t smem = exchange_l2_smem_bytes(N, M, C, wpb);
  VMCK_CUDA(cudaFuncSetAttribute(metropolis_exchange_l2_kernel,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = (int)std::min<int64_t>(((int64_t)B + wpb - 1) / wpb, sms);
  metropolis_exchange_l2_kernel<<<grid, 32 * wpb, smem, st>>>(
      p, N, M, sigma, log_prob, n_acc, B, sweep, n_discard, L, samples, k0, k1, counter, clusters,
      C);
  return check_launch("metropolis_sample (exchange, weights through L2)");
}

static size_t exchange_smem_bytes(int N, int M, int C, int wpb) {
  const int nwords = (C + 31) >> 5;
  size_t bytes = (size_t)N * M * 4 + (size_t)M * 4 + (size_t)N * 4 + (size_t)(C + 1) * 4 +
                 (size_t)C * 4 + (size_t)N * XS_MAXDEG * 2 + 4 + (size_t)N * 4 + 16;
  bytes += (size_t)wpb * ((((size_t)N + 15) & ~size_t(15)) + 4 * (size_t)nwords);
  return bytes + 64;
}

template <int R>
static int launch_exchange_smem(cudaStream_t st, const float *p, int N, int M, int8_t *sigma,
                                double *log_prob, int64_t *n_acc, int B, int sweep, int n_discard,
                                int L, int8_t *samples, uint32_t k0, uint32_t k1, uint64_t counter,
                                const int32_t *clusters, int C, int sms) {
  int wpb = (B + sms - 1) / sms;
  if (wpb > XS_MAX_WARPS) wpb = XS_MAX_WARPS;
  const size_t smem = exchange_smem_bytes(N, M, C, wpb);
  VMCK_CUDA(cudaFuncSetAttribute(metropolis_exchange_smem_kernel<R>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = (B + wpb - 1) / wpb;
  metropolis_exchange_smem_kernel<R><<<grid, 32 * wpb, smem, st>>>(
      p, N, M, sigma, log_prob, n_acc, B, sweep, n_discard, L, samples, k0, k1, counter, clusters,
      C, wpb);
  return check_launch("metropolis_sample (exchange, shared-memory weights)");
}

template <typename T>
int launch_metropolis(cudaStream_t st, const void *params, int N, int M, int8_t *sigma,
                      double *log_prob, int64_t *n_acc, int B, int sweep, int n_discard, int L,
                      int8_t *samples, uint64_t seed, uint64_t counter, int rule,
                      const int32_t *clusters, int C) {
  const size_t per_warp = 4 * (size_t)M * sizeof(T) + ((N + 15) & ~15);
  const size_t cl_bytes = (rule == 1) ? ((4 * (size_t)C + 15) & ~size_t(15)) : 0;
  const size_t budget = 200 * 1024;
  VMCK_REQUIRE(cl_bytes + per_warp <= budget, "M too large for the Metropolis kernel");
  int wpb = (int)std::min<size_t>(4, (budget - cl_bytes) / per_warp);
  if (wpb < 1) wpb = 1;
  size_t smem = cl_bytes + wpb * per_warp;
  int grid = (B + wpb - 1) / wpb;
  const T *p = static_cast<const T *>(params);
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  // VMCK_EXCHANGE_GENERIC=1 routes the Exchange rule to metropolis_kernel<float, 1>
  // (read per call): the parity tests run both kernels on the same seeds.
  const char *generic = getenv("VMCK_EXCHANGE_GENERIC");
  const bool force_generic = generic && generic[0] == '1';
  if (sizeof(T) == 4 && rule == 1 && C <= 1024 && M <= 512 && !force_generic) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int wpb = std::min((B + sms - 1) / sms, XS_MAX_WARPS);
    if (exchange_smem_bytes(N, M, C, wpb) <= 200 * 1024) {
      const float *pf = reinterpret_cast<const float *>(params);
      if (M <= 128)
        return launch_exchange_smem<4>(st, pf, N, M, sigma, log_prob, n_acc, B, sweep, n_discard,
                                       L, samples, k0, k1, counter, clusters, C, sms);
      if (M <= 256)
        return launch_exchange_smem<8>(st, pf, N, M, sigma, log_prob, n_acc, B, sweep, n_discard,
                                       L, samples, k0, k1, counter, clusters, C, sms);
      if (M <= 416)
        return launch_exchange_smem<13>(st, pf, N, M, sigma, log_prob, n_acc, B, sweep, n_discard,
                                        L, samples, k0, k1, counter, clusters, C, sms);
      return launch_exchange_smem<16>(st, pf, N, M, sigma, log_prob, n_acc, B, sweep, n_discard,
                                      L, samples, k0, k1, counter, clusters, C, sms);
    }
  }
  if (sizeof(T) == 4 && rule == 1 && C <= 1024 && M > 512 && !force_generic &&
      exchange_l2_warps(N, M, C) > 0) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return launch_exchange_l2(st, reinterpret_cast<const float *>(params), N, M, sigma, log_prob,
                              n_acc, B, sweep, n_discard, L, samples, k0, k1, counter, clusters, C,
                              sms);
  }
  if (rule == 0) {
    if (smem > 48 * 1024)
      VMCK_CUDA(cudaFuncSetAttribute(metropolis_kernel<T, 0>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    metropolis_kernel<T, 0><<<grid, 32 * wpb, smem, st>>>(p, N, M, sigma, log_prob, n_acc, B, sweep,
                                                         n_discard, L, samples, k0, k1, counter,
                                                         clusters, 0, wpb);
  } else {
    if (smem > 48 * 1024)
      VMCK_CUDA(cudaFuncSetAttribute(metropolis_kernel<T, 1>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    metropolis_kernel<T, 1><<<grid, 32 * wpb, smem, st>>>(p, N, M, sigma, log_prob, n_acc, B, sweep,
                                                         n_discard, L, samples, k0, k1, counter,
                                                         clusters, C, wpb);
  }
  return check_launch("metropolis_sample");
}

}  // namespace vmck

using namespace vmck;

extern "C" int vmck_metropolis_sample(vmck_stream s, int32_t dtype, const void *params, int32_t N,
                                      int32_t M, int8_t *sigma, double *log_prob,
                                      int64_t *n_accepted, int32_t B, int32_t sweep_size,
                                      int32_t n_discard, int32_t chain_length, int8_t *samples,
                                      uint64_t seed, uint64_t counter, int32_t rule,
                                      const int32_t *clusters, int32_t n_clusters) {
  VMCK_REQUIRE(params && sigma && log_prob && n_accepted && N > 0 && N < 32768 && M > 0 && B > 0,
               "metropolis arguments");
  VMCK_REQUIRE(sweep_size >= 0 && n_discard >= 0 && chain_length >= 0, "metropolis lengths");
  VMCK_REQUIRE(chain_length == 0 || samples, "samples buffer");
  VMCK_REQUIRE(rule == 0 || rule == 1, "rule must be 0 (local) or 1 (exchange)");
  VMCK_REQUIRE(rule == 0 || (clusters && n_clusters > 0), "exchange clusters");
  cudaStream_t st = as_stream(s);
  if (dtype == VMCK_F64)
    return launch_metropolis<double>(st, params, N, M, sigma, log_prob, n_accepted, B, sweep_size,
                                     n_discard, chain_length, samples, seed, counter, rule,
                                     clusters, n_clusters);
  if (dtype == VMCK_F32)
    return launch_metropolis<float>(st, params, N, M, sigma, log_prob, n_accepted, B, sweep_size,
                                    n_discard, chain_length, samples, seed, counter, rule, clusters,
                                    n_clusters);
  set_last_error("metropolis_sample: dtype %d unsupported", dtype);
  return VMCK_ERR_UNSUPPORTED;
}

extern "C" int vmck_batched_metropolis_local(vmck_stream s, int32_t dtype, vmck_batch_chains *inst,
                                             int32_t n_inst, const int32_t *work, int32_t n_items,
                                             int32_t chains_per_item, int32_t *queue,
                                             int32_t n_discard, int32_t chain_length,
                                             int32_t max_N, int32_t max_M, int32_t n_ctas) {
  VMCK_REQUIRE(inst && work && queue && n_inst > 0 && n_items >= 0 && chains_per_item > 0 &&
                   chains_per_item <= 32 && max_N > 0 && max_N < 32768 && max_M > 0 && n_ctas > 0,
               "batched_metropolis arguments");
  VMCK_REQUIRE(n_discard >= 0 && chain_length >= 0, "batched_metropolis lengths");
  cudaStream_t st = as_stream(s);
  VMCK_CUDA(cudaMemsetAsync(queue, 0, sizeof(int32_t), st));
  const size_t es = dtype == VMCK_F64 ? 8 : 4;
  const size_t per_warp = 4 * (size_t)max_M * es + ((max_N + 15) & ~15);
  const size_t smem = per_warp * chains_per_item;
  VMCK_REQUIRE(smem <= 200 * 1024, "batched_metropolis: max_M too large");
  const int threads = 32 * chains_per_item;
  if (dtype == VMCK_F32) {
    VMCK_CUDA(cudaFuncSetAttribute(batched_metropolis_kernel<float>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    batched_metropolis_kernel<float><<<n_ctas, threads, smem, st>>>(inst, work, n_items, queue,
                                                                     n_discard, chain_length,
                                                                     max_N, max_M);
  } else if (dtype == VMCK_F64) {
    VMCK_CUDA(cudaFuncSetAttribute(batched_metropolis_kernel<double>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    batched_metropolis_kernel<double><<<n_ctas, threads, smem, st>>>(inst, work, n_items, queue,
                                                                      n_discard, chain_length,
                                                                      max_N, max_M);
  } else {
    set_last_error("batched_metropolis: dtype %d unsupported", dtype);
    return VMCK_ERR_UNSUPPORTED;
  }
  int rc = check_launch("batched_metropolis");
  if (rc) return rc;
  batch_advance_counters_kernel<<<ceil_div(n_inst, 128), 128, 0, st>>>(inst, n_inst,
                                                                      n_discard + chain_length);
  return check_launch("batched counters");
}

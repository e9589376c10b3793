// Metropolis sweeps with the Hamiltonian transition rule for the RBM
// (netket/sampler/rules/hamiltonian.py:99-127 numba form, 153-213 jax form):
// from x, propose uniformly one of the n(x) entries of x's row of the operator,
//   n(x) = [diagonal slot] + sum_t kept(t, row_t(x)),
// kept(t, r) = the stored off-diagonal columns of term t's row r with
// |mel| > mel_cutoff, and correct by log n(x) - log n(x').  The diagonal slot
// proposes x itself (accepted: the ratio and the correction are 1); it is
// counted whenever the operator has a diagonal (diag_rule 1: LocalOperator's
// n_conn, operator/_local_operator/jax.py:107-112 and numba.py:166) or only
// where the diagonal element is nonzero (diag_rule 2: IsingJax's n_conn,
// operator/_ising/jax.py:168-175).
//
// One warp owns one chain for the whole launch, as in sampler.cu: theta =
// b + x W and log_cosh(theta) stay in shared memory and a proposal costs one
// log_cosh per hidden unit plus one FMA per changed site (at most 4).  The
// per-term counts at the current x are kept in shared memory (cnt_cur); a
// proposal picks its term with a warp scan over them, then the counts at x'
// are formed into cnt_new (every term: the row index of each term is two to
// four shared-memory loads) and the two arrays swap on acceptance.
#include <algorithm>

#include "common.cuh"
#include "localop.cuh"
#include "pauli.cuh"

namespace vmck {

template <typename T>
struct HamSmem {
  T *th, *lc, *tn, *ln;
  int8_t *xs;
  uint8_t *cnt_cur, *cnt_new;
};

__device__ __forceinline__ int term_row(const vmck_local_op &op, const int8_t *xs, int t) {
  const int sz = op.acting_size[t];
  int r = 0;
  for (int q = 0; q < sz; ++q) r = (r << 1) | (xs[op.acting_on[t * op.max_sites + q]] < 0);
  return r;
}

__device__ __forceinline__ int term_kept(const vmck_local_op &op, int t, int r) {
  const int64_t tr = (int64_t)t * op.max_rows + r;
  const int nc = op.n_conns[tr];
  const double *m = op.mels + tr * op.max_conns;
  int k = 0;
  for (int c = 0; c < nc; ++c) k += fabs(m[c]) > op.mel_cutoff;
  return k;
}

// Counts of every term at the configuration in xs into cnt; returns n(x) and
// sets *diag to whether the diagonal slot is counted.  diag_rule 2 needs the
// diagonal element, constant + sum_t diag_mels[t, row_t] (a warp tree sum): it
// is tested against mel_cutoff, so a rounding residue of a sum of +-J that
// cancels exactly in the reference's J * sum(+-1) still counts as zero.
__device__ int ham_count(const vmck_local_op &op, const int8_t *xs, uint8_t *cnt, int diag_rule,
                         int *diag) {
  const int lane = threadIdx.x & 31;
  int tot = 0;
  double d = 0.0;
  for (int t = lane; t < op.n_terms; t += 32) {
    const int r = term_row(op, xs, t);
    const int k = term_kept(op, t, r);
    cnt[t] = (uint8_t)k;
    tot += k;
    if (diag_rule == 2) d += op.diag_mels[(int64_t)t * op.max_rows + r];
  }
  tot = warp_sum(tot);
  int slot = diag_rule == 1;
  if (diag_rule == 2) slot = fabs(op.constant + warp_sum(d)) > op.mel_cutoff;
  __syncwarp();
  *diag = slot;
  return tot + slot;
}

// theta = b + x W and log_cosh(theta) from scratch into th / lc (th, lc may be
// null for the final log-amplitude only); returns logpsi(x).
template <typename T>
__device__ T chain_theta(const T *__restrict__ params, int N, int M, const int8_t *xs, T *th,
                         T *lc) {
  const int lane = threadIdx.x & 31;
  const T *bvec = params, *W = params + M, *a = params + M + (int64_t)N * M;
  T part = 0;
  for (int j = lane; j < M; j += 32) {
    T acc = bvec[j];
    for (int i = 0; i < N; ++i) acc += (T)xs[i] * W[(int64_t)i * M + j];
    const T l = log_cosh_fast(acc);
    if (th) {
      th[j] = acc;
      lc[j] = l;
    }
    part += l;
  }
  for (int i = lane; i < N; i += 32) part += (T)xs[i] * a[i];
  const T r = warp_sum(part);
  __syncwarp();
  return r;
}

// Index of the entry holding the k-th unit of the counts cnt[0..n) (warp scan
// in chunks of 32); *kk = its offset inside that entry.  -1 if k >= sum(cnt).
__device__ inline int warp_pick_kth(const uint8_t *cnt, int n, int k, int *kk) {
  const int lane = threadIdx.x & 31;
  for (int t0 = 0; t0 < n; t0 += 32) {
    const int t = t0 + lane;
    const int v = t < n ? cnt[t] : 0;
    int inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    const int chunk = __shfl_sync(0xffffffffu, inc, 31);
    if (k < chunk) {
      const unsigned m = __ballot_sync(0xffffffffu, inc > k);
      const int l = __ffs(m) - 1;
      *kk = k - (__shfl_sync(0xffffffffu, inc, l) - __shfl_sync(0xffffffffu, v, l));
      return t0 + l;
    }
    k -= chunk;
  }
  return -1;
}

template <typename T>
__device__ void run_chain_ham(const T *__restrict__ params, int N, int M, const vmck_local_op &op,
                              int diag_rule, int8_t *sigma_row, double *log_prob_b,
                              int64_t *n_accepted_b, int b, int sweep, int n_discard, int L,
                              int8_t *samples_chain, uint32_t k0, uint32_t k1, uint64_t counter,
                              HamSmem<T> c, int *err) {
  const int lane = threadIdx.x & 31;
  const T *W = params + M, *a = params + M + (int64_t)N * M;
  const int S = op.max_sites;
  for (int i = lane; i < N; i += 32) c.xs[i] = sigma_row[i];
  __syncwarp();
  int has_diag = 0;
  int n_cur = ham_count(op, c.xs, c.cnt_cur, diag_rule, &has_diag);
  T logpsi = 0;
  int64_t acc_count = 0;
  const int total = n_discard + L;
  for (int step = 0; step < total; ++step) {
    // theta, log_cosh(theta) recomputed exactly once per sweep
    logpsi = chain_theta(params, N, M, c.xs, c.th, c.lc);
    for (int p = 0; p < sweep; ++p) {
      const uint64_t pidx = counter + (uint64_t)step * sweep + p;
      u32x4 r = philox4x32_10(u32x4{(uint32_t)pidx, (uint32_t)(pidx >> 32), (uint32_t)b, 0u}, k0, k1);
      if (n_cur <= 0) continue;  // no connected element: no move
      int k = (int)below(r.x, (uint32_t)n_cur);
      if (has_diag) {
        if (k == 0) {  // x' = x: ratio 1, correction 0, always accepted
          ++acc_count;
          continue;
        }
        --k;
      }
      // term holding the k-th kept entry: warp scan over the counts
      int kk = 0;
      const int t_sel = warp_pick_kth(c.cnt_cur, op.n_terms, k, &kk);
      if (t_sel < 0) {  // counts inconsistent with n_cur: flag it, never index out of range
        if (lane == 0) atomicOr(err, VMCK_DEV_INTERNAL);
        continue;
      }
      // column of the kk-th kept entry of the selected row, and the changed sites
      const int row = term_row(op, c.xs, t_sel);
      const int64_t tr = (int64_t)t_sel * op.max_rows + row;
      const double *mrow = op.mels + tr * op.max_conns;
      int col = -1;
      for (int cc = 0, seen = 0; cc < op.n_conns[tr]; ++cc) {
        if (fabs(mrow[cc]) > op.mel_cutoff) {
          if (seen == kk) {
            col = cc;
            break;
          }
          ++seen;
        }
      }
      if (col < 0) {
        if (lane == 0) atomicOr(err, VMCK_DEV_INTERNAL);
        continue;
      }
      const int8_t *xp = op.x_prime + (tr * op.max_conns + col) * S;
      const int sz = op.acting_size[t_sel];
      // the term's sites with their spin change (0 where x' agrees with x);
      // fixed-size unrolled loops keep site / dv in registers
      int site[4];
      T dv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        site[q] = 0;
        dv[q] = 0;
        if (q < sz) {
          site[q] = op.acting_on[t_sel * S + q];
          dv[q] = (T)(xp[q] - c.xs[site[q]]);
        }
      }
      // counts at x'
      __syncwarp();
      if (lane == 0)
#pragma unroll
        for (int q = 0; q < 4; ++q) c.xs[site[q]] = (int8_t)(c.xs[site[q]] + (int)dv[q]);
      __syncwarp();
      int has_diag_new = 0;
      const int n_new = ham_count(op, c.xs, c.cnt_new, diag_rule, &has_diag_new);
      __syncwarp();
      if (lane == 0)
#pragma unroll
        for (int q = 0; q < 4; ++q) c.xs[site[q]] = (int8_t)(c.xs[site[q]] - (int)dv[q]);
      __syncwarp();
      // RBM log-ratio of the changed sites
      T s = 0;
      const T *W0 = W + (int64_t)site[0] * M, *W1 = W + (int64_t)site[1] * M;
      const T *W2 = W + (int64_t)site[2] * M, *W3 = W + (int64_t)site[3] * M;
      for (int j = lane; j < M; j += 32) {
        T t = c.th[j] + dv[0] * W0[j];
        if (sz > 1) t += dv[1] * W1[j];
        if (sz > 2) t += dv[2] * W2[j];
        if (sz > 3) t += dv[3] * W3[j];
        const T l = log_cosh_fast(t);
        c.tn[j] = t;
        c.ln[j] = l;
        s += l - c.lc[j];
      }
      s = warp_sum(s);
#pragma unroll
      for (int q = 0; q < 4; ++q) s += dv[q] * a[site[q]];
      const T corr = log((T)n_cur) - log((T)n_new);
      bool accept;
      if (sizeof(T) == 8) {
        accept = u01d(r.y, r.z) < exp((double)(2 * s + corr));
      } else {
        accept = u01f(r.y) < expf((float)(2 * s + corr));
      }
      if (accept) {
        for (int j = lane; j < M; j += 32) {
          c.th[j] = c.tn[j];
          c.lc[j] = c.ln[j];
        }
        __syncwarp();
        if (lane == 0)
#pragma unroll
          for (int q = 0; q < 4; ++q) c.xs[site[q]] = (int8_t)(c.xs[site[q]] + (int)dv[q]);
        uint8_t *tmp = c.cnt_cur;
        c.cnt_cur = c.cnt_new;
        c.cnt_new = tmp;
        n_cur = n_new;
        has_diag = has_diag_new;
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
  // final log-amplitude from scratch
  logpsi = chain_theta<T>(params, N, M, c.xs, nullptr, nullptr);
  for (int i = lane; i < N; i += 32) sigma_row[i] = c.xs[i];
  if (lane == 0) {
    *log_prob_b = 2.0 * (double)logpsi;
    *n_accepted_b += acc_count;
  }
}

__host__ __device__ inline size_t ham_per_warp_bytes(int N, int M, int T_terms, size_t tsize) {
  return ((4 * (size_t)M * tsize + 15) & ~size_t(15)) + ((N + 15) & ~15) +
         2 * (((size_t)T_terms + 15) & ~size_t(15));
}

template <typename T>
__global__ void metropolis_hamiltonian_kernel(const T *__restrict__ params, int N, int M,
                                              vmck_local_op op, int diag_rule, int8_t *sigma,
                                              double *log_prob, int64_t *n_accepted, int B,
                                              int sweep, int n_discard, int L, int8_t *samples,
                                              uint32_t k0, uint32_t k1, uint64_t counter, int wpb,
                                              int *err) {
  extern __shared__ unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5;
  const int b = blockIdx.x * wpb + warp;
  if (b >= B) return;
  unsigned char *base = smem_raw + warp * ham_per_warp_bytes(N, M, op.n_terms, sizeof(T));
  HamSmem<T> c;
  c.th = reinterpret_cast<T *>(base);
  c.lc = c.th + M;
  c.tn = c.lc + M;
  c.ln = c.tn + M;
  unsigned char *p = base + ((4 * (size_t)M * sizeof(T) + 15) & ~size_t(15));
  c.xs = reinterpret_cast<int8_t *>(p);
  p += (N + 15) & ~15;
  c.cnt_cur = p;
  c.cnt_new = p + ((op.n_terms + 15) & ~15);
  run_chain_ham<T>(params, N, M, op, diag_rule, sigma + (int64_t)b * N, log_prob + b,
                   n_accepted + b, b, sweep, n_discard, L, samples + (int64_t)b * L * N, k0, k1,
                   counter, c, err);
}

template <typename T>
static int launch_ham(cudaStream_t st, const void *params, int N, int M, const vmck_local_op &op,
                      int diag_rule, int8_t *sigma, double *log_prob, int64_t *n_acc, int B,
                      int sweep, int n_discard, int L, int8_t *samples, uint64_t seed,
                      uint64_t counter, int *err) {
  const size_t per_warp = ham_per_warp_bytes(N, M, op.n_terms, sizeof(T));
  const size_t budget = 200 * 1024;
  VMCK_REQUIRE(per_warp <= budget, "metropolis_hamiltonian: M or the term count too large");
  const int wpb = (int)std::min<size_t>(4, budget / per_warp);
  const size_t smem = wpb * per_warp;
  if (smem > 48 * 1024)
    VMCK_CUDA(cudaFuncSetAttribute(metropolis_hamiltonian_kernel<T>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = (B + wpb - 1) / wpb;
  metropolis_hamiltonian_kernel<T><<<grid, 32 * wpb, smem, st>>>(
      static_cast<const T *>(params), N, M, op, diag_rule, sigma, log_prob, n_acc, B, sweep,
      n_discard, L, samples, (uint32_t)seed, (uint32_t)(seed >> 32), counter, wpb, err);
  return check_launch("metropolis_hamiltonian");
}

// ------------------------------------------------------------ PauliStrings
// The same rule for PauliStrings (PauliStringsJax.n_conn = the number of slots
// with |mel| > cutoff, _pauli_strings/jax.py:256-269, which is also the set the
// jax rule draws from).  Per chain: the keep flag of every slot at x (keep_cur)
// and the down-spin mask of x; a proposal takes the k-th kept slot, flips its
// sites, recounts the slots at x' with down(x') = down(x) ^ flip_mask, and
// forms the RBM log-ratio of the flipped sites.  A kept slot with an empty flip
// set proposes x itself (always accepted).
template <typename T>
struct PauliChainSmem {
  T *th, *lc, *tn, *ln;
  int8_t *xs;
  uint32_t *down, *down_new;
  uint8_t *keep_cur, *keep_new;
};

__device__ int pauli_count(const vmck_pauli_strings &op, const uint32_t *down, uint8_t *keep) {
  const int lane = threadIdx.x & 31;
  int tot = 0;
  for (int f = lane; f < op.n_flips; f += 32) {
    const int k = fabs(pauli_mel(op, f, down)) > op.cutoff;
    keep[f] = (uint8_t)k;
    tot += k;
  }
  tot = warp_sum(tot);
  __syncwarp();
  return tot;
}

template <typename T>
__device__ void run_chain_ham_pauli(const T *__restrict__ params, int N, int M,
                                    const vmck_pauli_strings &op, int8_t *sigma_row,
                                    double *log_prob_b, int64_t *n_accepted_b, int b, int sweep,
                                    int n_discard, int L, int8_t *samples_chain, uint32_t k0,
                                    uint32_t k1, uint64_t counter, PauliChainSmem<T> c,
                                    int *err) {
  const int lane = threadIdx.x & 31;
  const T *W = params + M, *a = params + M + (int64_t)N * M;
  const int Wd = op.n_words;
  for (int i = lane; i < N; i += 32) c.xs[i] = sigma_row[i];
  __syncwarp();
  pauli_down_mask(c.xs, N, Wd, c.down, lane, 32);
  __syncwarp();
  int n_cur = pauli_count(op, c.down, c.keep_cur);
  T logpsi = 0;
  int64_t acc_count = 0;
  const int total = n_discard + L;
  for (int step = 0; step < total; ++step) {
    logpsi = chain_theta(params, N, M, c.xs, c.th, c.lc);
    for (int p = 0; p < sweep; ++p) {
      const uint64_t pidx = counter + (uint64_t)step * sweep + p;
      u32x4 r = philox4x32_10(u32x4{(uint32_t)pidx, (uint32_t)(pidx >> 32), (uint32_t)b, 0u}, k0, k1);
      if (n_cur <= 0) continue;
      int kk = 0;
      const int f = warp_pick_kth(c.keep_cur, op.n_flips, (int)below(r.x, (uint32_t)n_cur), &kk);
      if (f < 0) {
        if (lane == 0) atomicOr(err, VMCK_DEV_INTERNAL);
        continue;
      }
      const int q0 = op.flip_offset[f], q1 = op.flip_offset[f + 1];
      if (q0 == q1) {  // x' = x
        ++acc_count;
        continue;
      }
      for (int w = lane; w < Wd; w += 32) c.down_new[w] = c.down[w] ^ op.flip_mask[(int64_t)f * Wd + w];
      __syncwarp();
      const int n_new = pauli_count(op, c.down_new, c.keep_new);
      T s = 0;
      for (int j = lane; j < M; j += 32) {
        T t = c.th[j];
        for (int q = q0; q < q1; ++q) {
          const int i = op.flip_site[q];
          t += (T)(-2 * c.xs[i]) * W[(int64_t)i * M + j];
        }
        const T l = log_cosh_fast(t);
        c.tn[j] = t;
        c.ln[j] = l;
        s += l - c.lc[j];
      }
      s = warp_sum(s);
      for (int q = q0; q < q1; ++q) {
        const int i = op.flip_site[q];
        s += (T)(-2 * c.xs[i]) * a[i];
      }
      const T corr = log((T)n_cur) - log((T)n_new);
      bool accept;
      if (sizeof(T) == 8) {
        accept = u01d(r.y, r.z) < exp((double)(2 * s + corr));
      } else {
        accept = u01f(r.y) < expf((float)(2 * s + corr));
      }
      if (accept) {
        for (int j = lane; j < M; j += 32) {
          c.th[j] = c.tn[j];
          c.lc[j] = c.ln[j];
        }
        __syncwarp();
        for (int q = q0 + lane; q < q1; q += 32) {
          const int i = op.flip_site[q];
          c.xs[i] = (int8_t)(-c.xs[i]);
        }
        uint8_t *tk = c.keep_cur;
        c.keep_cur = c.keep_new;
        c.keep_new = tk;
        uint32_t *td = c.down;
        c.down = c.down_new;
        c.down_new = td;
        n_cur = n_new;
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
  logpsi = chain_theta<T>(params, N, M, c.xs, nullptr, nullptr);
  for (int i = lane; i < N; i += 32) sigma_row[i] = c.xs[i];
  if (lane == 0) {
    *log_prob_b = 2.0 * (double)logpsi;
    *n_accepted_b += acc_count;
  }
}

__host__ __device__ inline size_t pauli_chain_bytes(int N, int M, int Wd, int F, size_t tsize) {
  return ((4 * (size_t)M * tsize + 15) & ~size_t(15)) + ((N + 15) & ~15) +
         2 * ((4 * (size_t)Wd + 15) & ~size_t(15)) + 2 * (((size_t)F + 15) & ~size_t(15));
}

template <typename T>
__global__ void metropolis_hamiltonian_pauli_kernel(const T *__restrict__ params, int N, int M,
                                                    vmck_pauli_strings op, int8_t *sigma,
                                                    double *log_prob, int64_t *n_accepted, int B,
                                                    int sweep, int n_discard, int L,
                                                    int8_t *samples, uint32_t k0, uint32_t k1,
                                                    uint64_t counter, int wpb, int *err) {
  extern __shared__ unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5;
  const int b = blockIdx.x * wpb + warp;
  if (b >= B) return;
  unsigned char *p =
      smem_raw + warp * pauli_chain_bytes(N, M, op.n_words, op.n_flips, sizeof(T));
  PauliChainSmem<T> c;
  c.th = reinterpret_cast<T *>(p);
  c.lc = c.th + M;
  c.tn = c.lc + M;
  c.ln = c.tn + M;
  p += (4 * (size_t)M * sizeof(T) + 15) & ~size_t(15);
  c.xs = reinterpret_cast<int8_t *>(p);
  p += (N + 15) & ~15;
  c.down = reinterpret_cast<uint32_t *>(p);
  p += (4 * (size_t)op.n_words + 15) & ~size_t(15);
  c.down_new = reinterpret_cast<uint32_t *>(p);
  p += (4 * (size_t)op.n_words + 15) & ~size_t(15);
  c.keep_cur = p;
  c.keep_new = p + ((op.n_flips + 15) & ~15);
  run_chain_ham_pauli<T>(params, N, M, op, sigma + (int64_t)b * N, log_prob + b, n_accepted + b,
                         b, sweep, n_discard, L, samples + (int64_t)b * L * N, k0, k1, counter, c,
                         err);
}

template <typename T>
static int launch_ham_pauli(cudaStream_t st, const void *params, int N, int M,
                            const vmck_pauli_strings &op, int8_t *sigma, double *log_prob,
                            int64_t *n_acc, int B, int sweep, int n_discard, int L,
                            int8_t *samples, uint64_t seed, uint64_t counter, int *err) {
  const size_t per_warp = pauli_chain_bytes(N, M, op.n_words, op.n_flips, sizeof(T));
  const size_t budget = 200 * 1024;
  VMCK_REQUIRE(per_warp <= budget, "metropolis_hamiltonian_pauli: M or the slot count too large");
  const int wpb = (int)std::min<size_t>(4, budget / per_warp);
  const size_t smem = wpb * per_warp;
  if (smem > 48 * 1024)
    VMCK_CUDA(cudaFuncSetAttribute(metropolis_hamiltonian_pauli_kernel<T>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = (B + wpb - 1) / wpb;
  metropolis_hamiltonian_pauli_kernel<T><<<grid, 32 * wpb, smem, st>>>(
      static_cast<const T *>(params), N, M, op, sigma, log_prob, n_acc, B, sweep, n_discard, L,
      samples, (uint32_t)seed, (uint32_t)(seed >> 32), counter, wpb, err);
  return check_launch("metropolis_hamiltonian_pauli");
}

}  // namespace vmck

using namespace vmck;

extern "C" int vmck_metropolis_hamiltonian_pauli(vmck_stream s, int32_t dtype, const void *params,
                                                 int32_t N, int32_t M,
                                                 const vmck_pauli_strings *op, int8_t *sigma,
                                                 double *log_prob, int64_t *n_accepted, int32_t B,
                                                 int32_t sweep_size, int32_t n_discard,
                                                 int32_t chain_length, int8_t *samples,
                                                 uint64_t seed, uint64_t counter,
                                                 int32_t *status) {
  VMCK_REQUIRE(params && op && sigma && log_prob && n_accepted && status && N > 0 && M > 0 &&
                   B > 0,
               "metropolis_hamiltonian_pauli arguments");
  VMCK_REQUIRE(sweep_size >= 0 && n_discard >= 0 && chain_length >= 0, "metropolis lengths");
  VMCK_REQUIRE(chain_length == 0 || samples, "samples buffer");
  int rc = validate_pauli(*op);
  if (rc) return rc;
  VMCK_REQUIRE(op->n_sites == N, "metropolis_hamiltonian_pauli: operator size differs from N");
  cudaStream_t st = as_stream(s);
  if (dtype == VMCK_F64)
    return launch_ham_pauli<double>(st, params, N, M, *op, sigma, log_prob, n_accepted, B,
                                    sweep_size, n_discard, chain_length, samples, seed, counter,
                                    status);
  if (dtype == VMCK_F32)
    return launch_ham_pauli<float>(st, params, N, M, *op, sigma, log_prob, n_accepted, B,
                                   sweep_size, n_discard, chain_length, samples, seed, counter,
                                   status);
  set_last_error("metropolis_hamiltonian_pauli: dtype %d unsupported", dtype);
  return VMCK_ERR_UNSUPPORTED;
}

extern "C" int vmck_metropolis_hamiltonian(vmck_stream s, int32_t dtype, const void *params,
                                           int32_t N, int32_t M, const vmck_local_op *op,
                                           int32_t diag_rule, int8_t *sigma, double *log_prob,
                                           int64_t *n_accepted, int32_t B, int32_t sweep_size,
                                           int32_t n_discard, int32_t chain_length,
                                           int8_t *samples, uint64_t seed, uint64_t counter,
                                           int32_t *status) {
  VMCK_REQUIRE(params && op && sigma && log_prob && n_accepted && status && N > 0 && M > 0 &&
                   B > 0,
               "metropolis_hamiltonian arguments");
  VMCK_REQUIRE(sweep_size >= 0 && n_discard >= 0 && chain_length >= 0, "metropolis lengths");
  VMCK_REQUIRE(chain_length == 0 || samples, "samples buffer");
  VMCK_REQUIRE(diag_rule >= 0 && diag_rule <= 2, "diag_rule must be 0, 1 or 2");
  int rc = validate_local_op(*op);
  if (rc) return rc;
  VMCK_REQUIRE(op->n_sites == N, "metropolis_hamiltonian: operator size differs from N");
  VMCK_REQUIRE(op->max_conns <= 255, "metropolis_hamiltonian: more than 255 columns per row");
  cudaStream_t st = as_stream(s);
  if (dtype == VMCK_F64)
    return launch_ham<double>(st, params, N, M, *op, diag_rule, sigma, log_prob, n_accepted, B,
                              sweep_size, n_discard, chain_length, samples, seed, counter, status);
  if (dtype == VMCK_F32)
    return launch_ham<float>(st, params, N, M, *op, diag_rule, sigma, log_prob, n_accepted, B,
                             sweep_size, n_discard, chain_length, samples, seed, counter, status);
  set_last_error("metropolis_hamiltonian: dtype %d unsupported", dtype);
  return VMCK_ERR_UNSUPPORTED;
}

// Enumeration of the connected elements of a packed spin-1/2 LocalOperator
// inside one CTA, shared by get_conn_local (which writes them out) and the
// fused local-energy kernel (which consumes them without materialising x').
//
// Order follows LocalOperatorJax (netket/operator/_local_operator/jax.py:74-201):
// [diagonal] then, per term in output order, the stored off-diagonal columns
// of the term's row; entries with |mel| <= mel_cutoff are dropped, the rest are
// compacted to the front.  The diagonal is
//   constant + sum_groups (sum_terms-in-group diag_mels[t, row_t]),
// summed sequentially in that order (one thread), so it reproduces NetKet's
// value bit for bit whenever the partial sums are exact (all couplings of the
// shipped Hamiltonians) and its sequential order otherwise.
#pragma once

#include "common.cuh"

namespace vmck {

struct LocalConnShared {
  int8_t *xs;         // [N] current configuration
  int32_t *row;       // [T] row index of each term
  int32_t *off;       // [T] exclusive offset of each term's kept entries
  int32_t *slot_term; // [K] term of slot k (-1 = diagonal)
  int32_t *slot_col;  // [K] stored column of slot k
  double *slot_mel;   // [K]
  int32_t *misc;      // [4]: kept count, base
  unsigned char *end;
};

__host__ __device__ inline size_t align16(size_t v) { return (v + 15) & ~size_t(15); }

__host__ __device__ inline size_t local_conn_shared_bytes(const vmck_local_op &op) {
  size_t b = align16(op.n_sites);
  b += align16(4 * (size_t)op.n_terms) * 2;
  b += align16(4 * (size_t)op.max_conn_size) * 2;
  b += align16(8 * (size_t)op.max_conn_size);
  b += 16;
  b += 32 * sizeof(int);  // scan scratch
  return align16(b);
}

__device__ inline LocalConnShared local_conn_shared_layout(unsigned char *p,
                                                           const vmck_local_op &op) {
  LocalConnShared s;
  s.xs = reinterpret_cast<int8_t *>(p);
  p += align16(op.n_sites);
  s.row = reinterpret_cast<int32_t *>(p);
  p += align16(4 * (size_t)op.n_terms);
  s.off = reinterpret_cast<int32_t *>(p);
  p += align16(4 * (size_t)op.n_terms);
  s.slot_term = reinterpret_cast<int32_t *>(p);
  p += align16(4 * (size_t)op.max_conn_size);
  s.slot_col = reinterpret_cast<int32_t *>(p);
  p += align16(4 * (size_t)op.max_conn_size);
  s.slot_mel = reinterpret_cast<double *>(p);
  p += align16(8 * (size_t)op.max_conn_size);
  s.misc = reinterpret_cast<int32_t *>(p);
  p += 16 + 32 * sizeof(int);
  s.end = reinterpret_cast<unsigned char *>(align16(reinterpret_cast<uintptr_t>(p)));
  return s;
}

// A group of threads that synchronise together: the whole CTA (bar == 0,
// __syncthreads) or a warp-aligned slice of it with its own named barrier.
struct Grp {
  int tid, size, bar;
};
__device__ inline Grp cta_grp() { return Grp{(int)threadIdx.x, (int)blockDim.x, 0}; }
__device__ inline void grp_sync(const Grp &g) {
  if (g.bar == 0)
    __syncthreads();
  else
    asm volatile("bar.sync %0, %1;" ::"r"(g.bar), "r"(g.size) : "memory");
}

// Group-wide exclusive scan of per-thread values; returns the prefix of this
// thread and writes the total to *total (all threads).  scratch: 32 ints.
__device__ inline int grp_exclusive_scan(const Grp &g, int v, int *scratch, int *total) {
  const int lane = g.tid & 31, wid = g.tid >> 5, nw = g.size >> 5;
  int inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  grp_sync(g);
  if (lane == 31) scratch[wid] = inc;
  grp_sync(g);
  if (wid == 0) {
    int w = (lane < nw) ? scratch[lane] : 0;
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < nw) scratch[lane] = wi - w;  // exclusive warp offsets
    if (lane == nw - 1) scratch[31] = wi;   // total
  }
  grp_sync(g);
  int res = scratch[wid] + inc - v;
  *total = scratch[31];
  grp_sync(g);
  return res;
}

__device__ inline int block_exclusive_scan(int v, int *scratch, int *total) {
  return grp_exclusive_scan(cta_grp(), v, scratch, total);
}

// Requires sh.xs to hold the configuration.  Returns the number of kept
// entries (<= max_conn_size); slots [0, kept) are filled.  seq_diag: sum the
// diagonal sequentially in NetKet's order on one thread (bit-exact parity
// path); otherwise warp 0 sums it with a shuffle tree (FP32 consumers).
__device__ inline int local_conn_enumerate(const vmck_local_op &op, LocalConnShared &sh,
                                           const Grp &g, bool seq_diag = true) {
  const int T = op.n_terms, S = op.max_sites, R = op.max_rows, C = op.max_conns;
  const int K = op.max_conn_size;
  const double cut = op.mel_cutoff;
  // contiguous chunk of terms per thread keeps the scan order equal to term order
  const int per = (T + g.size - 1) / g.size;
  const int t0 = g.tid * per, t1 = min(T, t0 + per);
  int mine = 0;
  for (int t = t0; t < t1; ++t) {
    const int sz = op.acting_size[t];
    int r = 0;
    for (int q = 0; q < sz; ++q) {
      int site = op.acting_on[t * S + q];
      r = (r << 1) | (sh.xs[site] < 0 ? 1 : 0);
    }
    sh.row[t] = r;
    const int nc = op.n_conns[(int64_t)t * R + r];
    const double *m = op.mels + ((int64_t)t * R + r) * C;
    int cnt = 0;
    for (int c = 0; c < nc; ++c) cnt += fabs(m[c]) > cut;
    mine += cnt;
  }
  int *scratch = reinterpret_cast<int *>(sh.misc + 4);
  int total = 0;
  int pre = grp_exclusive_scan(g, mine, scratch, &total);
  // rows are visible after the scan's barriers
  double dtree = 0.0;
  if (!seq_diag && op.nonzero_diagonal && g.tid < 32) {
    for (int t = g.tid; t < T; t += 32) dtree += op.diag_mels[(int64_t)t * R + sh.row[t]];
    dtree = warp_sum(dtree);
  }
  if (g.tid == 0) {
    int base = 0;
    if (op.nonzero_diagonal) {
      double tot = 0.0;
      if (seq_diag) {
        int t = 0;
        for (int gg = 0; gg < op.n_groups; ++gg) {
          double gs = 0.0;
          for (; t < op.group_end[gg]; ++t) gs += op.diag_mels[(int64_t)t * R + sh.row[t]];
          tot += gs;
        }
      } else {
        tot = dtree;
      }
      double d = op.constant + tot;
      if (fabs(d) > cut) {
        sh.slot_term[0] = -1;
        sh.slot_col[0] = 0;
        sh.slot_mel[0] = d;
        base = 1;
      }
    }
    sh.misc[0] = base;
  }
  grp_sync(g);
  const int base = sh.misc[0];
  int pos = base + pre;
  for (int t = t0; t < t1; ++t) {
    const int r = sh.row[t];
    const int nc = op.n_conns[(int64_t)t * R + r];
    const double *m = op.mels + ((int64_t)t * R + r) * C;
    for (int c = 0; c < nc; ++c) {
      double v = m[c];
      if (fabs(v) > cut) {
        if (pos < K) {
          sh.slot_term[pos] = t;
          sh.slot_col[pos] = c;
          sh.slot_mel[pos] = v;
        }
        ++pos;
      }
    }
  }
  grp_sync(g);
  int kept = base + total;
  return kept < K ? kept : K;
}

__device__ inline int local_conn_enumerate(const vmck_local_op &op, LocalConnShared &sh) {
  return local_conn_enumerate(op, sh, cta_grp());
}

inline int validate_local_op(const vmck_local_op &op) {
  if (op.n_sites <= 0 || op.n_terms < 0 || op.max_sites < 1 || op.max_sites > 4 ||
      op.max_rows != (1 << op.max_sites) || op.max_conns < 0 || op.max_conn_size < 0 ||
      op.n_groups < 0 || op.n_sites >= 32768) {
    set_last_error("vmck_local_op: inconsistent sizes");
    return VMCK_ERR_ARG;
  }
  if (op.n_terms > 0 && (!op.acting_on || !op.acting_size || !op.group_end ||
                         !op.diag_mels || !op.n_conns || (op.max_conns > 0 && (!op.mels || !op.x_prime)))) {
    set_last_error("vmck_local_op: null table pointer");
    return VMCK_ERR_ARG;
  }
  return VMCK_OK;
}

}  // namespace vmck

// PauliStrings on spin-1/2 states as bitmasks (PauliStringsJax,
// netket/operator/_pauli_strings/jax.py:50-269).  Slot f of a sample x is the
// state x with the sites of flip_mask[f] flipped; its matrix element is
//   mel_f(x) = sum_{s in slot f} weight[s] * (-1)^popcount(z_mask[s] & down(x)),
// down(x) = the sites with x_i = -1, summed over the slot's strings in order
// (the reference's einsum over the strings of one flip set).  Slots with
// |mel| <= cutoff are dropped (x' = x, mel 0).
#pragma once

#include "common.cuh"

namespace vmck {

// down(x) as n_words 32-bit words (bit i of word w: site 32 w + i is -1), by
// the threads [tid0, tid0 + nthreads) of the caller.
__device__ inline void pauli_down_mask(const int8_t *xs, int N, int W, uint32_t *down, int tid,
                                       int nthreads) {
  for (int w = tid; w < W; w += nthreads) {
    uint32_t v = 0;
    const int i0 = 32 * w;
    const int n = min(32, N - i0);
    for (int k = 0; k < n; ++k) v |= (uint32_t)(xs[i0 + k] < 0) << k;
    down[w] = v;
  }
}

// Sign (+1 / -1) of string s at the configuration given by down.
__device__ inline double pauli_sign(const vmck_pauli_strings &op, int s, const uint32_t *down) {
  const uint32_t *z = op.z_mask + (int64_t)s * op.n_words;
  int par = 0;
  for (int w = 0; w < op.n_words; ++w) par ^= __popc(z[w] & down[w]);
  return (par & 1) ? -1.0 : 1.0;
}

// mel_f(x), strings summed sequentially (one thread).
__device__ inline double pauli_mel(const vmck_pauli_strings &op, int f, const uint32_t *down) {
  double m = 0.0;
  for (int s = op.string_offset[f]; s < op.string_offset[f + 1]; ++s)
    m += op.weight[s] * pauli_sign(op, s, down);
  return m;
}

inline int validate_pauli(const vmck_pauli_strings &op) {
  if (op.n_sites <= 0 || op.n_sites >= 32768 || op.n_words != (op.n_sites + 31) / 32 ||
      op.n_flips < 0 || op.n_strings < 0) {
    set_last_error("vmck_pauli_strings: inconsistent sizes");
    return VMCK_ERR_ARG;
  }
  if (op.n_flips > 0 && (!op.flip_mask || !op.flip_offset || !op.flip_site ||
                         !op.string_offset || !op.z_mask || !op.weight)) {
    set_last_error("vmck_pauli_strings: null table pointer");
    return VMCK_ERR_ARG;
  }
  return VMCK_OK;
}

}  // namespace vmck

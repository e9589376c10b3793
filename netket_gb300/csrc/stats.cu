// Monte Carlo statistics in FP64: the blocking estimator of
// netket/stats/mc_stats_old.py:88-196 over data (n_chains B, chain_length L).
//
// Pass 1 (one CTA per chain): per-chain sum, the two half-chain sums used by
// split-R-hat and the block sums (block length max(1, L / 32)), written to the
// workspace.  Pass 2 (one CTA): mean, two-pass population variance, variance of
// chain means, of block means and of half-chain means, then NetKet's choice of
// error estimate and R-hat.  Every reduction runs in a fixed order, so results
// are bit-reproducible run to run.
#include <mutex>

#include "common.cuh"

namespace vmck {

struct StatsLayout {
  int B, L, l_block, nb, h;
  int64_t chain_off, half_off, block_off, total;
};

__host__ __device__ inline StatsLayout stats_layout(int B, int L) {
  StatsLayout s;
  s.B = B;
  s.L = L;
  s.l_block = L / 32 > 1 ? L / 32 : 1;
  s.nb = L / s.l_block;
  s.h = L / 2;
  s.chain_off = 0;
  s.half_off = B;
  s.block_off = 3 * (int64_t)B;
  s.total = 3 * (int64_t)B + (int64_t)B * s.nb;
  return s;
}

__global__ void stats_pass1(const double *__restrict__ data, StatsLayout lay, double *ws) {
  __shared__ double red[32];
  const int b = blockIdx.x;
  const double *row = data + (int64_t)b * lay.L;
  double s = 0, s0 = 0, s1 = 0;
  for (int l = threadIdx.x; l < lay.L; l += blockDim.x) {
    double v = row[l];
    s += v;
    if (l < lay.h)
      s0 += v;
    else if (l < 2 * lay.h)
      s1 += v;
  }
  s = block_sum(s, red);
  s0 = block_sum(s0, red);
  s1 = block_sum(s1, red);
  if (threadIdx.x == 0) {
    ws[lay.chain_off + b] = s;
    ws[lay.half_off + 2 * b] = s0;
    ws[lay.half_off + 2 * b + 1] = s1;
  }
  // block sums: one thread per block (blocks are short: l_block = L/32)
  for (int k = threadIdx.x; k < lay.nb; k += blockDim.x) {
    double t = 0;
    for (int q = 0; q < lay.l_block; ++q) t += row[k * lay.l_block + q];
    ws[lay.block_off + (int64_t)b * lay.nb + k] = t;
  }
}

// population variance of v[i] * scale over count entries (two-pass)
__device__ double pop_var(const double *v, int64_t count, double scale, double *red) {
  double s = 0;
  for (int64_t i = threadIdx.x; i < count; i += blockDim.x) s += v[i] * scale;
  double mean = block_sum(s, red) / (double)count;
  double q = 0;
  for (int64_t i = threadIdx.x; i < count; i += blockDim.x) {
    double d = v[i] * scale - mean;
    q += d * d;
  }
  return block_sum(q, red) / (double)count;
}

__global__ void stats_pass2(const double *__restrict__ data, StatsLayout lay, int plain_rhat,
                            const double *ws, double *out5) {
  __shared__ double red[32];
  const int64_t ts = (int64_t)lay.B * lay.L;
  double s = 0;
  for (int b = threadIdx.x; b < lay.B; b += blockDim.x) s += ws[lay.chain_off + b];
  const double mean = block_sum(s, red) / (double)ts;
  double q = 0;
  for (int64_t i = threadIdx.x; i < ts; i += blockDim.x) {
    double d = data[i] - mean;
    q += d * d;
  }
  const double variance = block_sum(q, red) / (double)ts;
  double batch_var = pop_var(ws + lay.chain_off, lay.B, 1.0 / lay.L, red);
  const int n_batches = lay.B;
  const int64_t n_blocks = (int64_t)lay.B * lay.nb;
  double block_var = n_blocks > 0 ? pop_var(ws + lay.block_off, n_blocks, 1.0 / lay.l_block, red)
                                  : nan("");
  double split_var = 0;
  if (!plain_rhat && n_batches > 1 && lay.h > 0)
    split_var = pop_var(ws + lay.half_off, 2 * (int64_t)lay.B, 1.0 / lay.h, red);
  if (threadIdx.x == 0) {
    const int batch_size = 32;
    double tau_batch = (((double)ts / n_batches) * batch_var / variance - 1) * 0.5;
    double tau_block = (((double)ts / (double)n_blocks) * block_var / variance - 1) * 0.5;
    bool batch_good = (tau_batch < 6.0 * lay.L) && (n_batches >= batch_size);
    bool block_good = (tau_block < 6.0 * lay.l_block) && (n_blocks >= batch_size);
    double err, tau;
    if (batch_good) {
      err = sqrt(batch_var / n_batches);
      tau = tau_batch < 0 ? 0.0 : tau_batch;
    } else if (block_good) {
      err = sqrt(block_var / (double)n_blocks);
      tau = tau_block < 0 ? 0.0 : tau_block;
    } else {
      err = nan("");
      tau = nan("");
    }
    double rhat = nan("");
    if (n_batches > 1) {
      double bv = plain_rhat ? batch_var : (lay.h > 0 ? split_var : nan(""));
      rhat = sqrt((double)(lay.L - 1) / lay.L + bv / variance);
    }
    out5[0] = mean;
    out5[1] = err;
    out5[2] = variance;
    out5[3] = tau;
    out5[4] = rhat;
  }
}

// ------------------------------------------------------------ online accumulator
// One warp per chain (netket/_src/stats/online_stats/kernels.py:123-190).
// Welford: the batch mean and the batch sum of squared deviations (two passes
// over the chain's row), then the merge into (count, mean, M2) after the decay.
// ACF: lane l owns the lags k = l, l + 32, ...; for each it walks the batch once
// for the pairs (x_j, x_{j-k}) with j >= k and once for the pairs whose older
// member is in the rolling buffer (j < k, k - j <= buf_len).  In every
// iteration all lanes read the same x_j (a broadcast) and neighbouring x_{j-k}
// (one coalesced line), so the row is read from L1 after its first touch.
// The within-batch and cross-batch sums are formed separately and added to the
// (decayed) accumulator as (within + cross), the reference's association.
// Finally the buffer keeps the newest max_lag samples: a forward in-place shift
// by n_batch in 32-wide chunks (each chunk's reads are at higher addresses than
// every write so far) followed by the batch's tail.
constexpr int OS_WARPS = 4;

__global__ void __launch_bounds__(OS_WARPS * 32)
    online_stats_update_kernel(const double *__restrict__ data, int C, int nb, int L,
                               int old_len, double decay, int mean_f32, vmck_online_stats st) {
  const int lane = threadIdx.x & 31;
  const int c = blockIdx.x * OS_WARPS + (threadIdx.x >> 5);
  if (c >= C) return;
  const double *x = data + (int64_t)c * nb;

  double s = 0.0;
  for (int j = lane; j < nb; j += 32) s += x[j];
  const double c_mean = warp_sum(s) / nb;
  double q = 0.0;
  for (int j = lane; j < nb; j += 32) {
    const double d = x[j] - c_mean;
    q += d * d;
  }
  q = warp_sum(q);
  if (lane == 0) {
    const double cnt = st.count[c] * decay;
    const double M2 = st.M2[c] * decay;
    const double mu = st.mean[c];
    const double cnt_new = cnt + nb;
    const double safe = cnt_new > 0.0 ? cnt_new : 1.0;
    const double delta = c_mean - mu;
    double mu_new = mu + delta * ((double)nb / safe);
    if (mean_f32) mu_new = (double)(float)mu_new;
    st.mean[c] = mu_new;
    st.M2[c] = M2 + q + delta * delta * (cnt * nb / safe);
    st.count[c] = cnt_new;
  }
  if (L <= 0) return;

  const int64_t arow = (int64_t)c * (L + 1);
  double *buf = st.buf + (int64_t)c * L;
  for (int k = lane; k <= L; k += 32) {
    double cw = 0.0, m1w = 0.0, m2w = 0.0;
    for (int j = k; j < nb; ++j) {
      const double cur = x[j], lag = x[j - k];
      cw = fma(cur, lag, cw);
      m1w += lag;
      m2w += cur;
    }
    const double nw = nb > k ? (double)(nb - k) : 0.0;
    double cc = 0.0, m1c = 0.0, m2c = 0.0;
    const int jlo = k - old_len > 0 ? k - old_len : 0;
    const int jhi = k < nb ? k : nb;
    for (int j = jlo; j < jhi; ++j) {
      const double cur = x[j], lag = buf[L - (k - j)];
      cc = fma(cur, lag, cc);
      m1c += lag;
      m2c += cur;
    }
    const double nc = jhi > jlo ? (double)(jhi - jlo) : 0.0;
    st.cross[arow + k] = st.cross[arow + k] * decay + (cw + cc);
    st.m1[arow + k] = st.m1[arow + k] * decay + (m1w + m1c);
    st.m2[arow + k] = st.m2[arow + k] * decay + (m2w + m2c);
    st.pair[arow + k] = st.pair[arow + k] * decay + (nw + nc);
  }
  __syncwarp();
  if (nb >= L) {
    for (int i = lane; i < L; i += 32) buf[i] = x[nb - L + i];
  } else {
    const int keep = L - nb;
    for (int base = 0; base < keep; base += 32) {
      const int i = base + lane;
      const double v = i < keep ? buf[i + nb] : 0.0;
      __syncwarp();
      if (i < keep) buf[i] = v;
      __syncwarp();
    }
    for (int i = lane; i < nb; i += 32) buf[keep + i] = x[i];
  }
}

}  // namespace vmck

using namespace vmck;

extern "C" int vmck_online_stats_update(vmck_stream s, const double *data, int32_t n_chains,
                                        int32_t n_batch, int32_t max_lag, int32_t buf_len,
                                        double decay, int32_t mean_f32,
                                        const vmck_online_stats *state) {
  VMCK_REQUIRE(data && state && n_chains > 0 && n_batch > 0, "online_stats_update arguments");
  VMCK_REQUIRE(max_lag >= 0 && max_lag <= VMCK_ONLINE_STATS_MAX_LAG,
               "online_stats_update: max_lag out of range");
  VMCK_REQUIRE(buf_len >= 0 && buf_len <= max_lag, "online_stats_update: buf_len out of range");
  VMCK_REQUIRE(decay >= 0.0 && decay <= 1.0, "online_stats_update: decay must lie in [0, 1]");
  VMCK_REQUIRE(state->count && state->mean && state->M2, "online_stats_update: state");
  VMCK_REQUIRE(max_lag == 0 || (state->cross && state->m1 && state->m2 && state->pair &&
                                state->buf),
               "online_stats_update: ACF state");
  const int blocks = (n_chains + OS_WARPS - 1) / OS_WARPS;
  online_stats_update_kernel<<<blocks, OS_WARPS * 32, 0, as_stream(s)>>>(
      data, n_chains, n_batch, max_lag, buf_len, decay, mean_f32 ? 1 : 0, *state);
  return check_launch("online_stats_update");
}

// ------------------------------------------------------------ allocation-free variant
// Scratch for vmck_stats_f64_noalloc: a fixed array that lives in every device's
// global memory from library load until process exit, so the entry point never
// allocates.  Host code cannot use the symbol itself as a pointer (on the host
// it only names a shadow variable); the device address is fetched once per
// device with cudaGetSymbolAddress while that device is current.
static __device__ __align__(256) double g_stats_scratch[VMCK_STATS_NOALLOC_MAX_DOUBLES];

namespace {
std::mutex g_scratch_mutex;
double *g_scratch_ptr[64] = {nullptr};
}  // namespace

static int stats_scratch_for_current_device(double **out) {
  int dev = 0;
  VMCK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_last_error("stats_f64_noalloc: device ordinal %d out of range", dev);
    return VMCK_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_stats_scratch);
    if (e != cudaSuccess || !p) {
      set_last_error("stats_f64_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return VMCK_ERR_CUDA;
    }
    g_scratch_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_scratch_ptr[dev];
  return VMCK_OK;
}

extern "C" int vmck_stats_f64_noalloc(vmck_stream s, const double *data, int32_t n_chains,
                                      int32_t chain_length, int32_t plain_rhat, double *out5) {
  VMCK_REQUIRE(data && out5 && n_chains > 0 && chain_length > 0, "stats_noalloc arguments");
  StatsLayout lay = stats_layout(n_chains, chain_length);
  if (lay.total > VMCK_STATS_NOALLOC_MAX_DOUBLES) {
    set_last_error("stats_f64_noalloc: %d chains x %d samples need %lld scratch doubles, more "
                   "than the fixed %d; use vmck_stats_f64 with a caller workspace",
                   n_chains, chain_length, (long long)lay.total, VMCK_STATS_NOALLOC_MAX_DOUBLES);
    return VMCK_ERR_ARG;
  }
  double *scratch = nullptr;
  int rc = stats_scratch_for_current_device(&scratch);
  if (rc) return rc;
  // Pass 1 overwrites every scratch element pass 2 reads, so the contents left
  // by an earlier call need no clearing.
  cudaStream_t st = as_stream(s);
  stats_pass1<<<n_chains, 128, 0, st>>>(data, lay, scratch);
  rc = check_launch("stats_noalloc pass 1");
  if (rc) return rc;
  stats_pass2<<<1, 1024, 0, st>>>(data, lay, plain_rhat, scratch, out5);
  return check_launch("stats_noalloc pass 2");
}

extern "C" int64_t vmck_stats_workspace_size(int32_t n_chains, int32_t chain_length) {
  if (n_chains <= 0 || chain_length <= 0) return 0;
  return stats_layout(n_chains, chain_length).total;
}

extern "C" int vmck_stats_f64(vmck_stream s, const double *data, int32_t n_chains,
                              int32_t chain_length, int32_t plain_rhat, double *out5,
                              double *workspace, int64_t workspace_len) {
  VMCK_REQUIRE(data && out5 && workspace && n_chains > 0 && chain_length > 0, "stats arguments");
  StatsLayout lay = stats_layout(n_chains, chain_length);
  VMCK_REQUIRE(workspace_len >= lay.total, "stats workspace too small");
  cudaStream_t st = as_stream(s);
  stats_pass1<<<n_chains, 128, 0, st>>>(data, lay, workspace);
  int rc = check_launch("stats pass 1");
  if (rc) return rc;
  stats_pass2<<<1, 1024, 0, st>>>(data, lay, plain_rhat, workspace, out5);
  return check_launch("stats pass 2");
}

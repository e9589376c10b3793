// Blocked Cholesky factorisation of an FP32 matrix on the tcgen05 tensor cores
// (factor_mode 4 of vmck_cholesky_solve_refined): the factor of the FP32 copy
// of T that iterative refinement against the FP64 matrix turns into an
// FP64-accurate solve.  It replaces jax.scipy.linalg.cho_factor in
// netket/optimizer/solver/solvers.py:266-268.
//
// Storage: the matrix is column-major with its UPPER triangle valid (row-major
// lower triangle, the library's convention); the factor U (A = U^T U) replaces
// it in place.
//
// Algorithm: right-looking, 512-row block rows, each factored in 128-row inner
// panels:
//   leaf   chol_leaf_kernel: one CTA factors the 128 x 128 diagonal block in
//          shared memory and forms its inverse X = U_pp^-1;
//   panel  U[r0:r1, r1:n] = X^T A[r0:r1, r1:n]  (a GEMM with K = 128);
//   inner  A[r1:k1, r1:n] -= U[r0:r1, r1:k1]^T U[r0:r1, r1:n]  (K = 128), the
//          rest of the block row;
//   bulk   A[k1:n, k1:n] -= U[k0:k1, k1:n]^T U[k0:k1, k1:n]  (K = 512), once per
//          block row.
// Every GEMM runs in tc_gemm_kernel.  Its operands are FP32 values split into
// two FP16 terms, t * s = hi + lo with s a power of two that keeps the operand
// inside FP16's normal range (|t| s < 2^13), and it accumulates hi_a hi_b +
// hi_a lo_b + lo_a hi_b in FP32 in tensor memory: 22 significant bits per
// operand, so each product carries ~2^-21 relative error (lo_a lo_b, ~2^-22, is
// dropped) - FP32-GEMM class, at three half-precision MMAs where a BF16 split
// needs six.  Each GEMM's epilogue also writes the split form of the values the
// next GEMM consumes (the panel rows), so no separate conversion pass runs.
//
// Scales: for SPD A every trailing-matrix entry is bounded by max_i A_ii and
// every factor entry by sqrt(max_i A_ii); the leaf measures max |X| itself.
// A matrix that is not SPD reports VMCK_DEV_NOT_SPD from the leaf (the pivot is
// replaced by 1 so the run stays finite); the caller falls back.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "chol_tc.cuh"
#include "tc_common.cuh"

namespace vmck {

// scales[0] = s(max diag A), scales[1] = s(sqrt(max diag A)); status gets
// NONFINITE for a non-finite diagonal.  One block.
__global__ void __launch_bounds__(256) chol_bounds_kernel(const float *__restrict__ A, int64_t n,
                                                          float *scales, int32_t *status) {
  __shared__ float red[8];
  float m = 0.0f;
  bool bad = false;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const float d = A[i + i * n];
    bad |= !isfinite(d);
    m = fmaxf(m, fabsf(d));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  bad = __syncthreads_or(bad);
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < 8; ++w) t = fmaxf(t, red[w]);
    scales[0] = split_scale(t);
    scales[1] = split_scale(sqrtf(t));
    if (bad && status) atomicOr(status, VMCK_DEV_NONFINITE);
  }
}

// B operand of the first panel GEMM: out[j * ldo + i] = split(A(r0 + i, c0 + j))
// for i < rows (column-major A), zero for i in [rows, ldo).
__global__ void chol_split_rows_kernel(const float *__restrict__ A, int64_t n, int64_t r0,
                                       int64_t c0, int rows, int64_t cols, int ldo,
                                       const float *scales, __half *oh, __half *ol) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= cols * ldo) return;
  const int64_t j = e / ldo;
  const int i = (int)(e - j * ldo);
  __half hi = __float2half_rn(0.0f), lo = hi;
  if (i < rows) split_f16(A[(r0 + i) + (c0 + j) * n], scales[0], hi, lo);
  oh[e] = hi;
  ol[e] = lo;
}

// ------------------------------------------------------------ the GEMM
// C[m + nn ldc] = alpha (A_op B_op^T)(m, nn) / (sa sb) + beta C[m + nn ldc]
// with A_op (M x K) and B_op (N x K) given as split FP16 pairs whose rows are
// K-contiguous (TMA tensors: x = K, y = row).  tri: only m <= nn is written and
// tiles wholly below the diagonal are skipped.  Optional split output of the
// result: oh/ol[(nn - o_col0) ldo + m] = split(value * so) for m < o_rows,
// nn >= o_col0.
//
// Launched with programmatic dependent launch: the prologue (tensor-memory
// allocation, barriers, descriptor prefetch) overlaps the previous kernel of the
// stream.  Persistent and warp-specialised: warp 0 streams 64-wide K slabs of the four
// operand tiles with TMA (128-byte swizzle) into a 2-stage ring; warp 1 issues
// the tcgen05.mma (kind::f16, M = 128, N = 256) from one thread; warps 2-17 hold
// the tile's FP32 sums in registers (64 per thread).
//
// Accumulation.  The tensor core adds each MMA's products into its FP32
// accumulator with a truncating alignment, an error of up to an ulp of the
// running sum per MMA that does not average out: over K = 512 (96 MMAs) it left
// the factor's backward error at ~4e-6 and refinement converging by only ~0.08
// per pass.  Here the large hi * hi products accumulate in tensor memory for one
// 64-wide slab only (4 MMAs, region D1), and the epilogue adds each slab's sum
// to its registers with round-to-nearest FP32 additions; the small cross terms
// hi * lo + lo * hi (2^-11 of the sum) accumulate over the whole tile in region
// D2 (with lolo also lo * lo: the result is then the exact product of the split
// operands up to FP32 summation, so a Gram matrix stays positive semidefinite;
// without it the missing 2^-22 part is a positive semidefinite matrix taken
// away).  The MMA thread issues a slab's cross terms first, so the epilogue drains
// D1 of the previous slab meanwhile.  With beta != 0 the register sums start
// from the old C values, loaded while the tile's first slab runs, so the
// write-out only stores.  Waits for work are bounded by the library's wait limit; a wait that
// runs out sets VMCK_DEV_TIMEOUT and the CTA winds down.
constexpr int G_BM = 128, G_BN = 256, G_BK = 64, G_STAGES = 2;
constexpr int G_EPI_WARPS = 16;  // four per tensor-memory lane quarter, 64 columns each
constexpr int G_THREADS = 32 * (2 + G_EPI_WARPS);
constexpr int G_TMEM_COLS = 2 * G_BN;  // D1 (hi * hi, one slab), D2 (cross terms, one tile)
constexpr int G_COLS = G_BN / 4;       // columns per epilogue warp
constexpr int G_A_BYTES = G_BM * G_BK * 2;  // 16 KB (one of hi / lo)
constexpr int G_B_BYTES = G_BN * G_BK * 2;  // 32 KB
constexpr int G_STAGE_BYTES = 2 * G_A_BYTES + 2 * G_B_BYTES;
constexpr int G_UMMA_K = 16;
constexpr int G_CHUNK = 8;  // epilogue columns per tensor-memory load
constexpr int G_NCH = G_COLS / G_CHUNK;

struct GemmParams {
  int M, N, K;
  int a_row0, b_row0, k_off;  // TMA coordinates of A_op row 0, B_op row 0, first K
  float *C;
  int64_t ldc;
  float alpha, beta;
  const float *sa, *sb;
  int tri;
  int lolo;  // also lo * lo (a Gram matrix of the split operand stays one)
  // split K: tile t of kz * base_tiles covers K range [z kchunk, +kchunk) of
  // output tile t % base_tiles, z = t / base_tiles, into C + z zstride
  int kz, kchunk;
  int64_t zstride, base_tiles;
  __half *oh, *ol;
  int64_t ldo;
  int o_rows, o_col0;
  const float *so;
  int32_t *status;
  unsigned long long wait_ns;
  int mt, nt;
  int64_t tiles;
};

// Tile t -> (mi, ni).  Upper-triangular launches (BN = 2 BM, common origin):
// column tile ni holds row tiles 0 .. min(mt, 2 ni + 2) - 1.
__device__ __forceinline__ int64_t tri_cum(int64_t ni, int64_t mt) {
  const int64_t h = mt / 2;
  return ni <= h ? ni * (ni + 1) : h * (h + 1) + (ni - h) * mt;
}
__device__ __forceinline__ void gemm_tile(const GemmParams &g, int64_t t, int &mi, int &ni) {
  if (!g.tri) {
    mi = (int)(t % g.mt);
    ni = (int)(t / g.mt);
    return;
  }
  int lo = 0, hi = g.nt - 1;  // largest ni with tri_cum(ni) <= t
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tri_cum(mid, g.mt) <= t) lo = mid;
    else hi = mid - 1;
  }
  ni = lo;
  mi = (int)(t - tri_cum(lo, g.mt));
}

// Tile t -> (mi, ni), its K slab range [kb0, kb0 + nkb) and output C.
__device__ __forceinline__ void gemm_work(const GemmParams &g, int64_t t, int &mi, int &ni,
                                          int &kb0, int &nkb, float *&C) {
  if (g.kz == 1) {  // no split: skip the 64-bit division
    gemm_tile(g, t, mi, ni);
    kb0 = 0;
    nkb = (g.K + G_BK - 1) / G_BK;
    C = g.C;
    return;
  }
  const int64_t z = t / g.base_tiles;
  gemm_tile(g, t - z * g.base_tiles, mi, ni);
  const int k0 = (int)z * g.kchunk;
  const int k1 = min(g.K, k0 + g.kchunk);
  kb0 = k0 / G_BK;
  nkb = (k1 - k0 + G_BK - 1) / G_BK;
  C = g.C + z * g.zstride;
}

__global__ void __launch_bounds__(G_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap mAh, const __grid_constant__ CUtensorMap mAl,
                   const __grid_constant__ CUtensorMap mBh, const __grid_constant__ CUtensorMap mBl,
                   GemmParams g) {
  extern __shared__ __align__(1024) unsigned char g_smem_raw[];
  unsigned char *smem = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(g_smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + G_STAGES * G_STAGE_BYTES);
  uint64_t *empty = full + G_STAGES;
  uint64_t *d1_full = empty + G_STAGES;
  uint64_t *d1_empty = d1_full + 1;
  uint64_t *d2_full = d1_empty + 1;
  uint64_t *d2_empty = d2_full + 1;
  uint64_t *drain = d2_empty + 1;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(drain + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0)
    *abort_flag =
        (g.status && (*reinterpret_cast<volatile int32_t *>(g.status) & VMCK_DEV_TIMEOUT)) ? 1 : 0;
  __syncthreads();
  if (*abort_flag) return;
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(G_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < G_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(d1_full, 1);
    mbar_init(d1_empty, G_EPI_WARPS);
    mbar_init(d2_full, 1);
    mbar_init(d2_empty, G_EPI_WARPS);
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mAh)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mAl)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mBh)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mBl)) : "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;
  // the prologue above overlaps the previous kernel of the stream; its output
  // (operands, C) is read only from here on
  pdl_wait();
  pdl_trigger();

  auto fail = [&]() {
    if (g.status) atomicOr(g.status, VMCK_DEV_TIMEOUT);
    *abort_flag = 1;
  };

  if (warp == 0) {
    // ---------------- TMA producer
    if (lane == 0) {
      int64_t it = 0;
      for (int64_t tile = blockIdx.x; tile < g.tiles && !*abort_flag; tile += gridDim.x) {
        int mi, ni, kb0, num_kb;
        float *Ct;
        gemm_work(g, tile, mi, ni, kb0, num_kb, Ct);
        const int ya = g.a_row0 + mi * G_BM, yb = g.b_row0 + ni * G_BN;
        for (int kb = 0; kb < num_kb; ++kb, ++it) {
          const int s = (int)(it % G_STAGES);
          if (it >= G_STAGES &&
              !mbar_wait(&empty[s], (uint32_t)(((it / G_STAGES) - 1) & 1), g.wait_ns)) {
            fail();
            break;
          }
          if (*abort_flag) break;
          unsigned char *st = smem + s * G_STAGE_BYTES;
          const int x = g.k_off + (kb0 + kb) * G_BK;
          mbar_expect_tx(&full[s], G_STAGE_BYTES);
          tma_load_2d(st, &mAh, &full[s], x, ya);
          tma_load_2d(st + G_A_BYTES, &mAl, &full[s], x, ya);
          tma_load_2d(st + 2 * G_A_BYTES, &mBh, &full[s], x, yb);
          tma_load_2d(st + 2 * G_A_BYTES + G_B_BYTES / 2, &mBh, &full[s], x, yb + G_BN / 2);
          tma_load_2d(st + 2 * G_A_BYTES + G_B_BYTES, &mBl, &full[s], x, yb);
          tma_load_2d(st + 2 * G_A_BYTES + G_B_BYTES + G_B_BYTES / 2, &mBl, &full[s], x,
                      yb + G_BN / 2);
        }
      }
      // every copy issued must land before the CTA may exit
      const int64_t first = it > G_STAGES ? it - G_STAGES : 0;
      for (int64_t q = first; q < it; ++q)
        mbar_wait(&full[q % G_STAGES], (uint32_t)((q / G_STAGES) & 1));
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc = umma_idesc_f16(G_BM, G_BN);
      const uint32_t d1 = tmem_base, d2 = tmem_base + G_BN;
      int64_t it = 0, slab = 0, tcount = 0;
      bool issued_any = false, ok = true;
      for (int64_t tile = blockIdx.x; tile < g.tiles && ok && !*abort_flag;
           tile += gridDim.x, ++tcount) {
        if (tcount > 0 && !mbar_wait(d2_empty, (uint32_t)((tcount - 1) & 1), g.wait_ns)) {
          fail();
          break;
        }
        tc_fence_after();
        int mi, ni, kb0, num_kb;
        float *Ct;
        gemm_work(g, tile, mi, ni, kb0, num_kb, Ct);
        for (int kb = 0; kb < num_kb; ++kb, ++it, ++slab) {
          const int s = (int)(it % G_STAGES);
          if (!mbar_wait(&full[s], (uint32_t)((it / G_STAGES) & 1), g.wait_ns)) {
            fail();
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t ah = smem_u32(smem + s * G_STAGE_BYTES);
          const uint32_t al = ah + G_A_BYTES, bh = ah + 2 * G_A_BYTES, bl = bh + G_B_BYTES;
          // cross terms of this slab into D2 (accumulates over the tile)
#pragma unroll
          for (int k = 0; k < G_BK / G_UMMA_K; ++k) {
            const uint32_t off = k * G_UMMA_K * 2;
            umma_f16(d2, umma_desc_sw128(ah + off), umma_desc_sw128(bl + off), idesc,
                     (kb == 0 && k == 0) ? 0u : 1u);
            umma_f16(d2, umma_desc_sw128(al + off), umma_desc_sw128(bh + off), idesc, 1u);
            if (g.lolo)
              umma_f16(d2, umma_desc_sw128(al + off), umma_desc_sw128(bl + off), idesc, 1u);
          }
          // hi * hi of this slab into D1 once the epilogue has read the last slab
          if (slab > 0 && !mbar_wait(d1_empty, (uint32_t)((slab - 1) & 1), g.wait_ns)) {
            fail();
            ok = false;
            issued_any = true;
            break;
          }
          tc_fence_after();
#pragma unroll
          for (int k = 0; k < G_BK / G_UMMA_K; ++k) {
            const uint32_t off = k * G_UMMA_K * 2;
            umma_f16(d1, umma_desc_sw128(ah + off), umma_desc_sw128(bh + off), idesc,
                     k == 0 ? 0u : 1u);
          }
          umma_commit(&empty[s]);
          umma_commit(d1_full);
          issued_any = true;
        }
        if (!ok) break;
        umma_commit(d2_full);
      }
      if (issued_any) {
        umma_commit(drain);
        mbar_wait(drain, 0);
      }
    }
  } else {
    // ---------------- epilogue: warp e reads TMEM lane quarter (warp & 3),
    // columns [64 * (e >> 2), +64) of the 256-column tile
    const int e = warp - 2, quarter = warp & 3, part = e >> 2;
    const float inv_s = 1.0f / ((g.sa ? *g.sa : 1.0f) * (g.sb ? *g.sb : 1.0f));
    const float alpha = g.alpha * inv_s;  // a power of two times +-1: exact scaling
    const float cscale = g.beta / alpha;  // old C in units of the sums
    const float so = g.so ? *g.so : 1.0f;
    const uint32_t lane_off = static_cast<uint32_t>(quarter * 32) << 16;
    const uint32_t t1 = tmem_base + lane_off + (uint32_t)(part * G_COLS);
    const uint32_t t2 = t1 + G_BN;
    int64_t tcount = 0, slab = 0;
    bool alive = true;
    for (int64_t tile = blockIdx.x; tile < g.tiles && alive; tile += gridDim.x, ++tcount) {
      int mi, ni, kb0, num_kb;
      float *Ct;
      gemm_work(g, tile, mi, ni, kb0, num_kb, Ct);
      const int m = mi * G_BM + quarter * 32 + lane;
      const int nbase = ni * G_BN + part * G_COLS;
      const bool row_ok = m < g.M;
      float *Crow = Ct + m;
      // the sums start from the old C values (loaded while the first slab's MMAs
      // run), so the write-out only stores
      float acc[G_COLS];
      if (g.beta != 0.0f) {
        const float *cp = Crow + (int64_t)nbase * g.ldc;
#pragma unroll
        for (int i = 0; i < G_COLS; ++i) {
          const int nn = nbase + i;
          acc[i] = (row_ok && nn < g.N && (!g.tri || m <= nn)) ? *cp * cscale : 0.0f;
          cp += g.ldc;
        }
      } else {
#pragma unroll
        for (int i = 0; i < G_COLS; ++i) acc[i] = 0.0f;
      }
      for (int kb = 0; kb < num_kb; ++kb, ++slab) {
        if (!mbar_wait(d1_full, (uint32_t)(slab & 1), g.wait_ns)) {
          fail();
          alive = false;
          break;
        }
        tc_fence_after();
#pragma unroll
        for (int ch = 0; ch < G_NCH; ++ch) {
          float v[G_CHUNK];
          tmem_ld_8cols(t1 + ch * G_CHUNK, v);
          tmem_wait_ld();
#pragma unroll
          for (int j = 0; j < G_CHUNK; ++j) acc[ch * G_CHUNK + j] += v[j];
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(d1_empty);
      }
      if (!alive) break;
      if (!mbar_wait(d2_full, (uint32_t)(tcount & 1), g.wait_ns)) {
        fail();
        break;
      }
      tc_fence_after();
#pragma unroll
      for (int ch = 0; ch < G_NCH; ++ch) {
        float v[G_CHUNK];
        tmem_ld_8cols(t2 + ch * G_CHUNK, v);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < G_CHUNK; ++j) acc[ch * G_CHUNK + j] += v[j];
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(d2_empty);
      // write-out (stores only)
      float *cp = Crow + (int64_t)nbase * g.ldc;
      const bool split_row = g.oh && row_ok && m < g.o_rows;
#pragma unroll
      for (int i = 0; i < G_COLS; ++i) {
        const int nn = nbase + i;
        if (row_ok && nn < g.N && (!g.tri || m <= nn)) {
          const float val = alpha * acc[i];
          *cp = val;
          if (split_row && nn >= g.o_col0) {
            __half hi, lo;
            split_f16(val, so, hi, lo);
            const int64_t o = (int64_t)(nn - g.o_col0) * g.ldo + m;
            g.oh[o] = hi;
            g.ol[o] = lo;
          }
        }
        cp += g.ldc;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "r"(G_TMEM_COLS)
                 : "memory");
  }
}

// ------------------------------------------------------------ the leaf
// One CTA factors the mp x mp (mp <= 128) diagonal block at (r0, r0) of the
// column-major upper A in shared memory and forms X = U^-1.  Per 32-wide
// sub-panel p:
//   (a) warp 0 factors the 32 x 32 diagonal block, lane l holding column l in
//       registers: per pivot one shuffle and one FMA per row, the rows shifted
//       down one register per step so the step loop has a single compact body
//       (entries below the diagonal are updated too and never read);
//   (b) the panel row U_pp^-T A_p,j by forward substitution, two threads per
//       column j (even / odd rows), fully unrolled;
//   (c) the rank-32 update of the trailing block in 4 x 4 register tiles.
// Then warps 0-3 invert the four 32 x 32 diagonal blocks and all threads form
// the off-diagonal blocks of X by block back substitution, four outputs per
// thread at a time.
// Writes U in place, X split into K-contiguous rows (xh/xl[m * 128 + k] = X(k, m),
// scale from max |X| into *scale_x) and Y = X^T zero-padded column-major
// 128 x 128 (the refinement's triangular solves).  Rows / columns past mp are
// the identity.  A non-positive or NaN pivot raises VMCK_DEV_NOT_SPD and is
// replaced by 1.
constexpr int LB = 128, LLD = LB + 1, LEAF_T = 256;
constexpr int LPAD = 64;  // zeros after S: the diagonal inverse reads up to 31 floats past it
constexpr size_t CHOL_LEAF_SMEM = (size_t)(2 * LB * LLD + LPAD + LB + 3 * 32 * 33) * sizeof(float);

__global__ void __launch_bounds__(LEAF_T, 1) chol_leaf_kernel(float *__restrict__ A, int64_t n,
                                                           int64_t r0, int mp,
                                                           __half *__restrict__ xh,
                                                           __half *__restrict__ xl,
                                                           float *scale_x, float *__restrict__ yinv,
                                                           int32_t *status) {
  extern __shared__ float lsm[];
  float *S = lsm;             // S[i * LLD + j] = U(i, j), i <= j; zero below
  float *X = lsm + LB * LLD + LPAD;  // X[i * LLD + j] = U^-1(i, j), blocks I <= J only
  float *rd = X + LB * LLD;          // rd[i] = 1 / U(i, i)
  float *Tb = rd + LB;        // 3 x [32][33] temporaries of the inverse
  __shared__ float red[LEAF_T / 32];
  __shared__ int not_spd;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) not_spd = 0;
  if (tid < LPAD) S[LB * LLD + tid] = 0.0f;
  pdl_wait();  // the block was written by the previous kernel of the stream
  pdl_trigger();
  if (tid < LB) S[tid * LLD + LB] = 0.0f;  // each row's padding column
  {
    // all 64 of a thread's loads in flight at once
    float v[LB * LB / LEAF_T];
#pragma unroll
    for (int u = 0; u < LB * LB / LEAF_T; ++u) {
      const int e = u * LEAF_T + tid;
      const int j = e / LB, i = e - j * LB;
      v[u] = 0.0f;
      if (i <= j) {
        if (j < mp) v[u] = A[(r0 + i) + (r0 + j) * n];
        else if (i == j) v[u] = 1.0f;
      }
    }
#pragma unroll
    for (int u = 0; u < LB * LB / LEAF_T; ++u) {
      const int e = u * LEAF_T + tid;
      const int j = e / LB, i = e - j * LB;
      S[i * LLD + j] = v[u];
    }
  }
  __syncthreads();
#pragma unroll 1
  for (int p = 0; p < 4; ++p) {
    const int P = 32 * p;
    if (warp == 0) {
      // (a) at step k, c[i] holds row k + i of column P + lane
      float c[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) c[i] = S[(P + i) * LLD + P + lane];
      bool bad = false;
      float d = __shfl_sync(0xffffffffu, c[0], 0);
#pragma unroll 1
      for (int k = 0; k < 32; ++k) {
        if (!(d > 0.0f)) {
          bad = true;
          d = 1.0f;
        }
        const float inv = rsqrtf(d);
        const float u = (lane == k) ? d * inv : (lane > k ? c[0] * inv : 0.0f);  // U(k, lane)
        S[(P + k) * LLD + P + lane] = u;
        if (lane == 0) rd[P + k] = inv;
        // the next pivot's row first and its diagonal broadcast at once: the
        // dependency from one pivot to the next is then these two steps, and
        // the other 30 row updates issue while the broadcast is in flight
        c[0] = fmaf(-__shfl_sync(0xffffffffu, u, (k + 1) & 31), u, c[1]);
        const float dn = __shfl_sync(0xffffffffu, c[0], (k + 1) & 31);
#pragma unroll
        for (int i = 2; i < 32; ++i)
          c[i - 1] = fmaf(-__shfl_sync(0xffffffffu, u, (k + i) & 31), u, c[i]);
        c[31] = 0.0f;
        d = dn;
      }
      if (bad && lane == 0) not_spd = 1;
    }
    __syncthreads();
    const int ncols = LB - P - 32;
    if (ncols > 0) {
      // (b) thread pair (2 jj, 2 jj + 1): column j, rows P + g + 2 r
      if (tid < 2 * ncols) {
        const int g = tid & 1, j = P + 32 + (tid >> 1);
        float y[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) y[r] = S[(P + g + 2 * r) * LLD + j];
#pragma unroll
        for (int k = 0; k < 32; ++k) {
          const float mine = (g == (k & 1)) ? y[k >> 1] * rd[P + k] : 0.0f;
          const float yk = __shfl_sync(0xffffffffu, mine, (lane & ~1) | (k & 1));
          if (g == (k & 1)) y[k >> 1] = yk;
          const float *urow = S + (P + k) * LLD + P + g;  // U(k, P + g + 2 r) = urow[2 r]
#pragma unroll
          for (int r = 0; r < 16; ++r)
            if (2 * r + 1 > k && 2 * r + g > k) y[r] = fmaf(-urow[2 * r], yk, y[r]);
        }
#pragma unroll
        for (int r = 0; r < 16; ++r) S[(P + g + 2 * r) * LLD + j] = y[r];
      }
      __syncthreads();
      // (c) trailing update of the upper triangle [P+32, 128)^2 in 4 x 4 tiles
      const int T = ncols / 4, ntl = T * (T + 1) / 2;
      const int base = P + 32;
#pragma unroll 1
      for (int t = tid; t < ntl; t += LEAF_T) {
        int tj = (int)((sqrtf(8.0f * t + 1.0f) - 1.0f) * 0.5f);
        while (tj * (tj + 1) / 2 > t) --tj;
        while ((tj + 1) * (tj + 2) / 2 <= t) ++tj;
        const int ti = t - tj * (tj + 1) / 2;
        const int i0 = base + 4 * ti, j0 = base + 4 * tj;
        float acc[4][4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[r][q] = S[(i0 + r) * LLD + j0 + q];
#pragma unroll 4
        for (int k = 0; k < 32; ++k) {
          const float *row = S + (P + k) * LLD;
          float a[4], bq[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) a[r] = row[i0 + r];
#pragma unroll
          for (int q = 0; q < 4; ++q) bq[q] = row[j0 + q];
#pragma unroll
          for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[r][q] = fmaf(-a[r], bq[q], acc[r][q]);
        }
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (i0 + r <= j0 + q) S[(i0 + r) * LLD + j0 + q] = acc[r][q];
      }
      __syncthreads();
    }
  }
  // diagonal blocks of X: warp p inverts U_pp; lane l solves U x = e_l from the
  // bottom row up, x[q] holding row i + 1 + q at step s (i = 31 - s); rows past
  // the block hold 0, so their products with the entries read past the block's
  // last column (finite: later S entries, the zeroed padding column of each row
  // or the zero pad after S) vanish
  float am = 0.0f;  // max |X| over the valid block (this thread's writes)
  if (warp < 4) {
    const int P = 32 * warp;
    float x[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) x[i] = 0.0f;
#pragma unroll 1
    for (int s2 = 0; s2 < 32; ++s2) {
      const int i = 31 - s2;
      const float *urow = S + (P + i) * LLD + P + i + 1;  // U(i, i + 1 + q) = urow[q]
      float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
#pragma unroll
      for (int q = 0; q < 32; q += 4) {
        a0 = fmaf(urow[q], x[q], a0);
        a1 = fmaf(urow[q + 1], x[q + 1], a1);
        a2 = fmaf(urow[q + 2], x[q + 2], a2);
        a3 = fmaf(urow[q + 3], x[q + 3], a3);
      }
      const float ri = rd[P + i];
      const float xi = (i == lane) ? ri : (i < lane ? -((a0 + a1) + (a2 + a3)) * ri : 0.0f);
      X[(P + i) * LLD + P + lane] = xi;
      if (P + lane < mp) am = fmaxf(am, fabsf(xi));
#pragma unroll
      for (int q = 31; q > 0; --q) x[q] = x[q - 1];
      x[0] = xi;
    }
  }
  __syncthreads();
  // off-diagonal blocks of X: X_IJ = -X_II sum_{K=I+1..J} U_IK X_KJ, by distance d
  // (I = blk, J = blk + d), each thread a 4 x 4 tile of one block (64 per block)
  // in registers.  X below the block diagonal is never read.
#pragma unroll 1
  for (int d = 1; d < 4; ++d) {
    const int ntile = (4 - d) * 64;
    const int blk = tid >> 6, r0t = 4 * ((tid >> 3) & 7), c0t = 4 * (tid & 7);
    const bool act = tid < ntile;
    float acc[4][4];
    if (act) {
      // phase 1: Tb[blk] = sum_K U_IK X_KJ over the 32 d columns right of block I
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[r][q] = 0.0f;
      const float *ur = S + (32 * blk + r0t) * LLD + 32 * (blk + 1);
      const float *xc = X + 32 * (blk + 1) * LLD + 32 * (blk + d) + c0t;
#pragma unroll 4
      for (int k = 0; k < 32 * d; ++k) {
        float a[4], bq[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) a[r] = ur[r * LLD + k];
#pragma unroll
        for (int q = 0; q < 4; ++q) bq[q] = xc[k * LLD + q];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[r][q] = fmaf(a[r], bq[q], acc[r][q]);
      }
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) Tb[blk * 32 * 33 + (r0t + r) * 33 + c0t + q] = acc[r][q];
    }
    __syncthreads();
    if (act) {
      // phase 2: X_IJ = -X_II Tb[blk]
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[r][q] = 0.0f;
      const float *xr = X + (32 * blk + r0t) * LLD + 32 * blk;
      const float *tc = Tb + blk * 32 * 33 + c0t;
#pragma unroll 4
      for (int k = 0; k < 32; ++k) {
        float a[4], bq[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) a[r] = xr[r * LLD + k];
#pragma unroll
        for (int q = 0; q < 4; ++q) bq[q] = tc[k * 33 + q];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[r][q] = fmaf(a[r], bq[q], acc[r][q]);
      }
      const int row0 = 32 * blk + r0t, col0 = 32 * (blk + d) + c0t;
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          X[(row0 + r) * LLD + col0 + q] = -acc[r][q];
          if (col0 + q < mp) am = fmaxf(am, fabsf(acc[r][q]));
        }
    }
    __syncthreads();
  }
  // max |X| over the valid block -> split scale
  for (int o = 16; o > 0; o >>= 1) am = fmaxf(am, __shfl_xor_sync(0xffffffffu, am, o));
  if (lane == 0) red[warp] = am;
  __syncthreads();
  float amax = 0.0f;
#pragma unroll
  for (int w = 0; w < LEAF_T / 32; ++w) amax = fmaxf(amax, red[w]);
  const float sx = split_scale(amax);
  if (tid == 0) {
    *scale_x = sx;
    if (not_spd && status) atomicOr(status, VMCK_DEV_NOT_SPD);
  }
  // outputs
  for (int j = warp; j < mp; j += LEAF_T / 32)
    for (int i = lane; i <= j; i += 32) A[(r0 + i) + (r0 + j) * n] = S[i * LLD + j];
  for (int e = 2 * tid; e < LB * LB; e += 2 * LEAF_T) {
    const int m = e / LB, k = e - m * LB;  // row m of the split operand = column m of X
    __half h0 = __float2half_rn(0.0f), l0 = h0, h1 = h0, l1 = h0;
    if (m < mp && k <= m) split_f16(X[k * LLD + m], sx, h0, l0);
    if (m < mp && k + 1 <= m) split_f16(X[(k + 1) * LLD + m], sx, h1, l1);
    reinterpret_cast<__half2 *>(xh)[e >> 1] = __halves2half2(h0, h1);
    reinterpret_cast<__half2 *>(xl)[e >> 1] = __halves2half2(l0, l1);
  }
  for (int e = tid; e < LB * LB; e += LEAF_T) {
    const int c = e / LB, r = e - c * LB;  // Y(r, c) = X(c, r)
    yinv[e] = (r < mp && c <= r) ? X[c * LLD + r] : 0.0f;
  }
}

// ------------------------------------------------------------ host side
static int make_f16_map(CUtensorMap *map, const __half *base, int64_t kdim, int64_t rows,
                        int64_t ld) {
  auto fn = encode_fn();
  if (!fn) {
    set_last_error("cuTensorMapEncodeTiled is unavailable");
    return VMCK_ERR_CUDA;
  }
  cuuint64_t dims[2] = {(cuuint64_t)kdim, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
  cuuint32_t box[2] = {(cuuint32_t)G_BK, (cuuint32_t)G_BM};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<__half *>(base), dims,
                  strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_last_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return VMCK_ERR_CUDA;
  }
  return VMCK_OK;
}


static int num_sms_dev() {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

static size_t gemm_smem_bytes() { return 1024 + G_STAGES * G_STAGE_BYTES + 8 * 16 + 64; }

int tc_gemm(cudaStream_t st, const SplitOperand &a, int a_row0, const SplitOperand &b, int b_row0,
            int k_off, int M, int N, int K, float *C, int64_t ldc, float alpha, float beta,
            const float *sa, const float *sb, int tri, __half *oh, __half *ol, int64_t ldo,
            int o_rows, int o_col0, const float *so, int32_t *status, int max_ctas, int lolo,
            int kchunk, int64_t zstride) {
  if (M <= 0 || N <= 0 || K <= 0) return VMCK_OK;
  if (kchunk <= 0 || kchunk >= K) kchunk = K;
  if (kchunk < K && (kchunk % G_BK != 0 || tri || oh || beta != 0.0f)) {
    set_last_error("tc_gemm: split K needs kchunk %% %d == 0, no tri / split output / beta", G_BK);
    return VMCK_ERR_ARG;
  }
  CUtensorMap mAh, mAl, mBh, mBl;
  int rc;
  if ((rc = make_f16_map(&mAh, a.hi, a.kdim, a.rows, a.ld))) return rc;
  if ((rc = make_f16_map(&mAl, a.lo, a.kdim, a.rows, a.ld))) return rc;
  if ((rc = make_f16_map(&mBh, b.hi, b.kdim, b.rows, b.ld))) return rc;
  if ((rc = make_f16_map(&mBl, b.lo, b.kdim, b.rows, b.ld))) return rc;
  GemmParams g{};
  g.M = M;
  g.N = N;
  g.K = K;
  g.a_row0 = a_row0;
  g.b_row0 = b_row0;
  g.k_off = k_off;
  g.C = C;
  g.ldc = ldc;
  g.alpha = alpha;
  g.beta = beta;
  g.sa = sa;
  g.sb = sb;
  g.tri = tri;
  g.lolo = lolo;
  g.oh = oh;
  g.ol = ol;
  g.ldo = ldo;
  g.o_rows = o_rows;
  g.o_col0 = o_col0;
  g.so = so;
  g.status = status;
  g.wait_ns = wait_limit_ns();
  g.mt = (M + G_BM - 1) / G_BM;
  g.nt = (N + G_BN - 1) / G_BN;
  if (tri) {
    const int64_t h = g.mt / 2;
    g.base_tiles = g.nt <= h ? (int64_t)g.nt * (g.nt + 1) : h * (h + 1) + (int64_t)(g.nt - h) * g.mt;
  } else {
    g.base_tiles = (int64_t)g.mt * g.nt;
  }
  g.kchunk = kchunk;
  g.kz = (K + kchunk - 1) / kchunk;
  g.zstride = zstride;
  g.tiles = g.base_tiles * g.kz;
  const size_t smem = gemm_smem_bytes();
  VMCK_CUDA(cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
  const int sms = max_ctas > 0 ? max_ctas : num_sms_dev();
  const unsigned grid = (unsigned)std::min<int64_t>(g.tiles, sms);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(G_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  VMCK_CUDA(cudaLaunchKernelEx(&cfg, tc_gemm_kernel, mAh, mAl, mBh, mBl, g));
  return check_launch("tc_gemm");
}

int chol_block_rows(int64_t n) {
  static const int forced = [] {
    const char *v = getenv("VMCK_CHOL_BLOCK");
    const int r = v ? atoi(v) : 0;
    return (r == 128 || r == 256 || r == 512 || r == 1024 || r == 2048 || r == 4096) ? r : 0;
  }();
  if (forced) return forced;
  // measured on GB300 (factor + refinement): n = 16,384: 18.5 / 18.2 / 19.7 ms
  // for 512 / 1024 / 2048 rows; 32,768: 86 / 68 / 71 ms; 65,536: 609 / 440 /
  // 385 / 412 ms (4096)
  return n >= 3 * CHOL_BIG_N / 2 ? 2048 : (n >= CHOL_BIG_N / 2 ? 1024 : CHOL_BLOCK);
}

int64_t chol_tc_workspace_bytes(int64_t n) {
  const int64_t nb = (n + LB - 1) / LB;
  int64_t b = 0;
  b += 4 * (int64_t)chol_block_rows(n) * n * 2;  // Ph hi / lo, two buffers (K = block rows)
  b += 2 * (int64_t)LB * n * 2;          // Bs hi / lo
  b += 2 * (int64_t)LB * LB * 2;         // Xs hi / lo
  b += 64;                               // scales
  b += nb * LB * LB * 4;                 // Yinv
  return b + 8 * 1024;                   // alignment
}

int chol_events_needed(int64_t n) {
  const int64_t blk = chol_block_rows(n);
  return (int)(3 * ((n + blk - 1) / blk) + 2 + 2 * ((n + LB - 1) / LB));
}

// Trailing-update CTAs of the side stream: every SM but a reserve that stays
// free for the chain's kernels: 48 below n = CHOL_BIG_N, 24 from there on
// (measured: the chain's share of the work shrinks with n; n = 65,536: 385 /
// 366 / 371 ms with 48 / 24 / 12), unless VMCK_CHOL_RESERVE (read once per
// process) sets it.
static int side_ctas(int sms, int64_t n) {
  static const int forced = [] {
    const char *v = getenv("VMCK_CHOL_RESERVE");
    return v ? std::max(0, atoi(v)) : -1;
  }();
  const int reserve = forced >= 0 ? forced : (n >= CHOL_BIG_N ? 24 : 48);
  return std::max(8, sms - reserve);
}

static char *align_up(char *p, size_t a) {
  return reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(p) + a - 1) & ~uintptr_t(a - 1));
}

int chol_tc_factor(cudaStream_t st, float *A, int64_t n, void *ws, int32_t *status,
                   float **yinv_out, const CholStreams *ls) {
  if (n <= 0) return VMCK_OK;
  if (n >= (1ll << 30)) {
    set_last_error("chol_tc: n must be below 2^30");
    return VMCK_ERR_UNSUPPORTED;
  }
  const int64_t blk = chol_block_rows(n);
  char *p = align_up(static_cast<char *>(ws), 1024);
  __half *ph_hi[2], *ph_lo[2];
  for (int q = 0; q < 2; ++q) {
    ph_hi[q] = reinterpret_cast<__half *>(p);
    p = align_up(p + (size_t)blk * n * 2, 1024);
    ph_lo[q] = reinterpret_cast<__half *>(p);
    p = align_up(p + (size_t)blk * n * 2, 1024);
  }
  __half *bs_hi = reinterpret_cast<__half *>(p);
  p = align_up(p + (size_t)LB * n * 2, 1024);
  __half *bs_lo = reinterpret_cast<__half *>(p);
  p = align_up(p + (size_t)LB * n * 2, 1024);
  __half *xs_hi = reinterpret_cast<__half *>(p);
  p = align_up(p + (size_t)LB * LB * 2, 1024);
  __half *xs_lo = reinterpret_cast<__half *>(p);
  p = align_up(p + (size_t)LB * LB * 2, 1024);
  float *scales = reinterpret_cast<float *>(p);  // [0] A entries, [1] U entries, [2] X
  p = align_up(p + 64, 1024);
  float *yinv = reinterpret_cast<float *>(p);
  if (yinv_out) *yinv_out = yinv;

  const int nblocks = (int)((n + blk - 1) / blk);
  // look-ahead: the chain stream factors block row b and updates block row b + 1
  // (LA); the side stream updates rows b + 2 .. with block row b, first block row
  // b + 2 (event E[b]: LA(b + 1) waits for it), then the rest (event G[b]: block
  // row b + 2 reuses block row b's split-panel buffer).  F[b]: block row b's
  // panel is complete.
  const bool two = ls && ls->chain && ls->side && ls->n_events >= 3 * nblocks + 2;
  cudaStream_t chain = two ? ls->chain : st, side = two ? ls->side : st;
  cudaEvent_t *F = two ? ls->events : nullptr, *E = F ? F + nblocks : nullptr;
  cudaEvent_t *G = E ? E + nblocks : nullptr;
  // split block-row updates: PA[p] panel p's rows are written (chain), PB[p] the
  // update of the rows below panel p + 1 by panel p is done (chain2)
  const int npanels = (int)((n + LB - 1) / LB);
  const bool split = two && ls->chain2 && ls->n_events >= 3 * nblocks + 2 + 2 * npanels;
  cudaEvent_t *PA = split ? G + nblocks + 2 : nullptr, *PB = split ? PA + npanels : nullptr;
  int rc;
  if (two) {
    VMCK_CUDA(cudaEventRecord(ls->events[3 * nblocks], st));
    VMCK_CUDA(cudaStreamWaitEvent(chain, ls->events[3 * nblocks], 0));
    VMCK_CUDA(cudaStreamWaitEvent(side, ls->events[3 * nblocks], 0));
    if (split) VMCK_CUDA(cudaStreamWaitEvent(ls->chain2, ls->events[3 * nblocks], 0));
  }
  const int side_grid = two ? side_ctas(num_sms_dev(), n) : 0;
  VMCK_CUDA(cudaFuncSetAttribute(chol_leaf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)CHOL_LEAF_SMEM));
  chol_bounds_kernel<<<1, 256, 0, chain>>>(A, n, scales, status);
  if ((rc = check_launch("chol_tc bounds"))) return rc;
  {
    const int rows = (int)std::min<int64_t>(LB, n);
    const int64_t cols = n - rows;
    if (cols > 0) {
      chol_split_rows_kernel<<<ceil_div(cols * LB, 256), 256, 0, chain>>>(
          A, n, 0, rows, rows, cols, LB, scales, bs_hi, bs_lo);
      if ((rc = check_launch("chol_tc split"))) return rc;
    }
  }
  for (int b = 0; b < nblocks; ++b) {
    const int64_t k0 = b * blk;
    const int64_t k1 = std::min<int64_t>(n, k0 + blk), w = k1 - k0;
    const int64_t k2 = std::min<int64_t>(n, k1 + blk), k3 = std::min<int64_t>(n, k2 + blk);
    __half *qh = ph_hi[two ? (b & 1) : 0], *ql = ph_lo[two ? (b & 1) : 0];
    // the block row's split panel: row (c - k0) holds U(k0 .. k1, c) (K = w)
    const SplitOperand ph{qh, ql, blk, w, n - k0};
    if (two && b >= 2)
      VMCK_CUDA(cudaStreamWaitEvent(chain, G[b - 2], 0));  // side is done with this buffer
    bool pb_pending = false;  // PB[pi - 1] recorded in this block row
    for (int64_t r0 = k0; r0 < k1; r0 += LB) {
      const int64_t r1 = std::min<int64_t>(k1, r0 + LB);
      const int mp = (int)(r1 - r0), pp = (int)((r0 - k0) / LB);
      const int pi = (int)(r0 / LB);
      {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(1);
        cfg.blockDim = dim3(LEAF_T);
        cfg.dynamicSmemBytes = CHOL_LEAF_SMEM;
        cfg.stream = chain;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        VMCK_CUDA(cudaLaunchKernelEx(&cfg, chol_leaf_kernel, A, n, r0, mp, xs_hi, xs_lo,
                                     scales + 2, yinv + (r0 / LB) * LB * LB, status));
        if ((rc = check_launch("chol_tc leaf"))) return rc;
      }
      if (r1 == n) break;
      const SplitOperand xop{xs_hi, xs_lo, LB, mp, mp};
      const SplitOperand bop{bs_hi, bs_lo, LB, mp, n - r1};
      // panel: U[r0:r1, r1:n] = X^T A[r0:r1, r1:n], split copy into Ph
      if ((rc = tc_gemm(chain, xop, 0, bop, 0, 0, mp, (int)(n - r1), mp, A + r0 + r1 * n, n,
                        1.0f, 0.0f, scales + 2, scales + 0, 0,
                        qh + (r1 - k0) * blk + pp * LB, ql + (r1 - k0) * blk + pp * LB, blk,
                        mp, 0, scales + 1,
                        status, 0)))
        return rc;
      if (r1 < k1) {
        // rest of the block row; rows [r1, r1 + next) feed the next panel (split)
        const int next = (int)std::min<int64_t>(LB, k1 - r1);
        const SplitOperand pk{qh, ql, blk, pp * LB + mp, n - k0};
        if (!split) {
          if ((rc = tc_gemm(chain, pk, (int)(r1 - k0), pk, (int)(r1 - k0), pp * LB,
                            (int)(k1 - r1), (int)(n - r1), mp, A + r1 + r1 * n, n, -1.0f, 1.0f,
                            scales + 1, scales + 1, 1, bs_hi, bs_lo, LB, next, next,
                            scales + 0, status, 0)))
            return rc;
        } else {
          // the next panel's rows on the chain (after the previous panel's update
          // of the same rows on chain2), the rows below them on chain2
          const int64_t r2 = r1 + next;
          if (r2 < k1) VMCK_CUDA(cudaEventRecord(PA[pi], chain));
          if (pb_pending) VMCK_CUDA(cudaStreamWaitEvent(chain, PB[pi - 1], 0));
          pb_pending = false;
          if ((rc = tc_gemm(chain, pk, (int)(r1 - k0), pk, (int)(r1 - k0), pp * LB, next,
                            (int)(n - r1), mp, A + r1 + r1 * n, n, -1.0f, 1.0f, scales + 1,
                            scales + 1, 1, bs_hi, bs_lo, LB, next, next, scales + 0, status, 0)))
            return rc;
          if (r2 < k1) {
            VMCK_CUDA(cudaStreamWaitEvent(ls->chain2, PA[pi], 0));
            if ((rc = tc_gemm(ls->chain2, pk, (int)(r2 - k0), pk, (int)(r2 - k0), pp * LB,
                              (int)(k1 - r2), (int)(n - r2), mp, A + r2 + r2 * n, n, -1.0f,
                              1.0f, scales + 1, scales + 1, 1, nullptr, nullptr, 0, 0, 0,
                              nullptr, status, 0)))
              return rc;
            VMCK_CUDA(cudaEventRecord(PB[pi], ls->chain2));
            pb_pending = true;
          }
        }
      }
    }
    if (k1 == n) break;
    const int next = (int)std::min<int64_t>(LB, n - k1);
    if (!two) {
      // trailing matrix by the whole block row; rows [k1, k1 + next) feed the
      // next block row's first panel (split)
      if ((rc = tc_gemm(st, ph, (int)w, ph, (int)w, 0, (int)(n - k1), (int)(n - k1), (int)w,
                        A + k1 + k1 * n, n, -1.0f, 1.0f, scales + 1, scales + 1, 1, bs_hi, bs_lo,
                        LB, next, next, scales + 0, status, 0)))
        return rc;
      continue;
    }
    VMCK_CUDA(cudaEventRecord(F[b], chain));
    // LA(b): block row b + 1 by this block row, once the side stream has applied
    // the previous block row to it
    if (b >= 1) VMCK_CUDA(cudaStreamWaitEvent(chain, E[b - 1], 0));
    if ((rc = tc_gemm(chain, ph, (int)w, ph, (int)w, 0, (int)(k2 - k1), (int)(n - k1), (int)w,
                      A + k1 + k1 * n, n, -1.0f, 1.0f, scales + 1, scales + 1, 1, bs_hi, bs_lo,
                      LB, next, next, scales + 0, status, 0)))
      return rc;
    // side: block row b + 2, then the rest
    VMCK_CUDA(cudaStreamWaitEvent(side, F[b], 0));
    if (k2 < n) {
      const int off2 = (int)(k2 - k0);
      if ((rc = tc_gemm(side, ph, off2, ph, off2, 0, (int)(k3 - k2), (int)(n - k2), (int)w,
                        A + k2 + k2 * n, n, -1.0f, 1.0f, scales + 1, scales + 1, 1, nullptr,
                        nullptr, 0, 0, 0, nullptr, status, side_grid)))
        return rc;
    }
    VMCK_CUDA(cudaEventRecord(E[b], side));
    if (k3 < n) {
      const int off3 = (int)(k3 - k0);
      if ((rc = tc_gemm(side, ph, off3, ph, off3, 0, (int)(n - k3), (int)(n - k3), (int)w,
                        A + k3 + k3 * n, n, -1.0f, 1.0f, scales + 1, scales + 1, 1, nullptr,
                        nullptr, 0, 0, 0, nullptr, status, side_grid)))
        return rc;
    }
    VMCK_CUDA(cudaEventRecord(G[b], side));
  }
  if (two) {
    VMCK_CUDA(cudaEventRecord(ls->events[3 * nblocks], chain));
    VMCK_CUDA(cudaStreamWaitEvent(st, ls->events[3 * nblocks], 0));
    VMCK_CUDA(cudaEventRecord(ls->events[3 * nblocks + 1], side));
    VMCK_CUDA(cudaStreamWaitEvent(st, ls->events[3 * nblocks + 1], 0));
    if (split) {  // (already ordered through the chain; kept explicit)
      VMCK_CUDA(cudaEventRecord(ls->events[3 * nblocks], ls->chain2));
      VMCK_CUDA(cudaStreamWaitEvent(st, ls->events[3 * nblocks], 0));
    }
  }
  return VMCK_OK;
}

}  // namespace vmck

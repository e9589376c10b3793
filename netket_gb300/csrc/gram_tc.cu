// Tensor-core form of the structured minSR Gram matrix (sm_103a: tcgen05 + TMA).
//
// T = (A o (1 + B) + B - g 1^T - 1 g^T + c 1 1^T) / n + diag_shift I with
// A = t t^T (t = tanh theta, n x M) and B = x x^T (exact, popcount).  A runs on
// the 5th-generation tensor cores in a persistent, warp-specialised kernel: one
// CTA per SM walks the 128 x 128 lower-triangular tiles of T; warp 0 streams
// K-slabs of the two operand panels with TMA (cp.async.bulk.tensor, 128-byte
// swizzle) into a 4-stage shared-memory ring, warp 1 issues tcgen05.mma
// (kind::f16, BF16 in, FP32 accumulate in tensor memory) from one thread, and
// eight epilogue warps read the accumulators back with tcgen05.ld, form T in
// double-float FP32 and write it with coalesced row segments staged through
// shared memory.  Tensor memory holds two tile buffers, so the epilogue of one
// tile overlaps the MMAs of the next.
//
// Precision: t arrives rounded to hi + lo (two BF16 terms) or to one BF16; the
// operand panels [hi | hi | lo | lo] and [hi | lo | hi | lo] (each segment
// padded to a multiple of 64) make one GEMM form all four products, i.e. t t^T
// exactly up to FP32 accumulation.  The hi * hi segment and the three small
// cross segments accumulate in separate tensor-memory regions (single-BF16 mode:
// alternate K-slabs), which keeps the tensor core's accumulation error on the
// large part from growing with the number of steps; the epilogue adds the
// regions in double-float.  Every other ingredient of T (column means, g) is
// computed from the same rounded t, so T is the Gram matrix of a slightly
// perturbed Jacobian.
//
// Every mbarrier wait is bounded by wall time (2 s, %globaltimer); a wait that
// runs out sets VMCK_DEV_TIMEOUT in the status word and an abort flag in shared
// memory; every role then leaves its loop, the producer waits (bounded) for the
// TMA copies it issued, the MMA thread for its last commit, and the CTA frees
// its tensor memory and exits.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "gram_tc.cuh"
#include "tc_common.cuh"

namespace vmck {

constexpr int TC_BM = 128;     // tile rows (UMMA M)
constexpr int TC_BN = 128;     // tile cols (UMMA N)
constexpr int TC_BK = 64;      // K slab: 64 bf16 = 128 bytes = one swizzle row
constexpr int TC_STAGES = 4;
constexpr int TC_UMMA_K = 16;  // K per tcgen05.mma for 16-bit inputs
constexpr int TC_TMEM_COLS = 512;  // 2 buffers x 2 regions x TC_BN columns
constexpr int TC_EPI_WARPS = 8;    // two per tensor-memory lane quarter, 64 columns each
constexpr int TC_THREADS = 32 * (2 + TC_EPI_WARPS);
constexpr int TC_CHUNK = 16;       // epilogue columns per tcgen05.ld
constexpr int TC_STG_LD = TC_CHUNK + 1;

// ------------------------------------------------------------ operand panels
// Input t is already rounded (exactly hi + lo, or exactly one BF16), so
//   split:  L = [hi | hi | lo | lo], R = [hi | lo | hi | lo]  ->  L R^T = t t^T,
//   single: L = R = [bf16(t)]                                 ->  L R^T = t t^T,
// exactly up to the FP32 accumulation.  Each segment is Mp = M rounded up to a
// multiple of 64 long (zero padded), so a K-slab never straddles two segments.
__global__ void tc_split_kernel(const float *__restrict__ t, int64_t n, int M, int Mp, int Kp,
                                int split, __nv_bfloat16 *__restrict__ L,
                                __nv_bfloat16 *__restrict__ R) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= n * Kp) return;
  const int64_t s = e / Kp;
  const int k = (int)(e % Kp);
  __nv_bfloat16 lv = __float2bfloat16(0.0f), rv = lv;
  const int seg = k / Mp, j = k % Mp;
  if (j < M) {
    if (!split) {
      lv = rv = __float2bfloat16(t[s * M + j]);
    } else {
      const float v = t[s * M + j];
      const __nv_bfloat16 hi = __float2bfloat16(v);
      const __nv_bfloat16 lo = __float2bfloat16(v - __bfloat162float(hi));
      lv = (seg < 2) ? hi : lo;
      rv = (seg & 1) ? lo : hi;
    }
  }
  L[e] = lv;
  R[e] = rv;
}

// ------------------------------------------------------------ the Gram kernel
struct TcEpilogue {
  const uint32_t *bits;
  int words, N;
  int64_t n;
  const float2 *h, *w, *s0sq;
  float inv_n;
  double diag_shift;
  double *T64;
  float *T32;
  int32_t *status;
  unsigned long long wait_ns;  // limit of the waits for work
};

__device__ inline void tc_tri_tile(int64_t bid, int64_t &I, int64_t &J) {
  int64_t i = (int64_t)((sqrt(8.0 * (double)bid + 1.0) - 1.0) * 0.5);
  while (i * (i + 1) / 2 > bid) --i;
  while ((i + 1) * (i + 2) / 2 <= bid) ++i;
  I = i;
  J = bid - i * (i + 1) / 2;
}

// num_kb K-slabs per tile; kb_hi: slabs of the hi * hi segment (split mode), or 0
// (single mode: slabs alternate between the two regions).
__global__ void __launch_bounds__(TC_THREADS, 1)
    gram_tc_kernel(const __grid_constant__ CUtensorMap mapL,
                   const __grid_constant__ CUtensorMap mapR, int num_kb, int kb_hi,
                   int64_t n_tiles, TcEpilogue ep) {
  extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
  unsigned char *smem = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
  constexpr int SLAB = TC_BM * TC_BK * 2;  // 16 KB
  unsigned char *slabA = smem;
  unsigned char *slabB = smem + TC_STAGES * SLAB;
  // per epilogue warp: the chunk being written, as (hi, lo) pairs [32][TC_STG_LD]
  float2 *stg = reinterpret_cast<float2 *>(smem + 2 * TC_STAGES * SLAB);
  // per epilogue warp: its 64 columns' sign bits (N <= 128), w and h pairs
  uint4 *cbits = reinterpret_cast<uint4 *>(stg + TC_EPI_WARPS * 32 * TC_STG_LD);
  float4 *cwh = reinterpret_cast<float4 *>(cbits + TC_EPI_WARPS * 64);
  uint64_t *full = reinterpret_cast<uint64_t *>(cwh + TC_EPI_WARPS * 64);
  uint64_t *empty = full + TC_STAGES;
  uint64_t *tfull = empty + TC_STAGES;  // [2]
  uint64_t *tempty = tfull + 2;         // [2]
  uint64_t *drain = tempty + 2;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(drain + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0)
    *abort_flag =
        (ep.status && (*reinterpret_cast<volatile int32_t *>(ep.status) & VMCK_DEV_TIMEOUT)) ? 1 : 0;
  __syncthreads();
  if (*abort_flag) return;  // an earlier CTA timed out: do no work
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], TC_EPI_WARPS);
    }
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapL)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapR)) : "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  auto fail = [&]() {
    if (ep.status) atomicOr(ep.status, VMCK_DEV_TIMEOUT);
    *abort_flag = 1;
  };

  if (warp == 0) {
    // ---------------- TMA producer
    if (lane == 0) {
      int64_t it = 0;
      for (int64_t tile = blockIdx.x; tile < n_tiles && !*abort_flag; tile += gridDim.x) {
        int64_t I, J;
        tc_tri_tile(tile, I, J);
        for (int kb = 0; kb < num_kb; ++kb, ++it) {
          const int s = (int)(it % TC_STAGES);
          if (it >= TC_STAGES &&
              !mbar_wait(&empty[s], (uint32_t)(((it / TC_STAGES) - 1) & 1), ep.wait_ns)) {
            fail();
            break;
          }
          if (*abort_flag) break;
          mbar_expect_tx(&full[s], 2 * SLAB);
          tma_load_2d(slabA + s * SLAB, &mapL, &full[s], kb * TC_BK, (int)(I * TC_BM));
          tma_load_2d(slabB + s * SLAB, &mapR, &full[s], kb * TC_BK, (int)(J * TC_BN));
        }
      }
      // every copy issued must land before the CTA may exit: wait for the last
      // TC_STAGES fills (bounded)
      const int64_t first = it > TC_STAGES ? it - TC_STAGES : 0;
      for (int64_t q = first; q < it; ++q)
        mbar_wait(&full[q % TC_STAGES], (uint32_t)((q / TC_STAGES) & 1));
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc = umma_idesc_bf16(TC_BM, TC_BN);
      int64_t it = 0, tcount = 0;
      bool issued_any = false;
      for (int64_t tile = blockIdx.x; tile < n_tiles && !*abort_flag; tile += gridDim.x, ++tcount) {
        const int b = (int)(tcount & 1);
        if (tcount >= 2 &&
            !mbar_wait(&tempty[b], (uint32_t)(((tcount >> 1) - 1) & 1), ep.wait_ns)) {
          fail();
          break;
        }
        tc_fence_after();
        bool ok = true;
        for (int kb = 0; kb < num_kb; ++kb, ++it) {
          const int s = (int)(it % TC_STAGES);
          if (!mbar_wait(&full[s], (uint32_t)((it / TC_STAGES) & 1), ep.wait_ns)) {
            fail();
            ok = false;
            break;
          }
          tc_fence_after();
          const int region = kb_hi ? (kb < kb_hi ? 0 : 1) : (kb & 1);
          const bool first = kb_hi ? (kb == 0 || kb == kb_hi) : (kb < 2);
          const uint32_t dacc = tmem_base + (uint32_t)(b * 2 * TC_BN + region * TC_BN);
          const uint32_t a0 = smem_u32(slabA + s * SLAB), b0 = smem_u32(slabB + s * SLAB);
#pragma unroll
          for (int k = 0; k < TC_BK / TC_UMMA_K; ++k) {
            const uint32_t off = k * TC_UMMA_K * 2;  // bytes along the swizzled row
            umma_f16(dacc, umma_desc_sw128(a0 + off), umma_desc_sw128(b0 + off), idesc,
                      (first && k == 0) ? 0u : 1u);
          }
          umma_commit(&empty[s]);
          issued_any = true;
        }
        if (!ok) break;
        umma_commit(&tfull[b]);
      }
      // wait for every MMA issued to complete before the tensor memory is freed
      if (issued_any) {
        umma_commit(drain);
        mbar_wait(drain, 0);
      }
    }
  } else {
    // ---------------- epilogue: warp e = warp - 2 reads TMEM lane quarter (warp & 3),
    // columns [64 * (e >> 2), +64)
    const int e = warp - 2, quarter = warp & 3, half = e >> 2;
    const int r = quarter * 32 + lane;  // tile row of this thread
    float2 *st = stg + e * 32 * TC_STG_LD;
    uint4 *wb = cbits + e * 64;
    float4 *wwh = cwh + e * 64;
    const df32 shift = df_from(ep.diag_shift);
    const df32 s0sq = {ep.s0sq->x, ep.s0sq->y};
    const bool two = kb_hi ? (num_kb > kb_hi) : (num_kb > 1);
    const bool narrow = ep.words <= 4;  // sign bits of a column fit one uint4
    int64_t tcount = 0;
    for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x, ++tcount) {
      const int b = (int)(tcount & 1);
      int64_t I, J;
      tc_tri_tile(tile, I, J);
      const int64_t r0 = I * TC_BM, c0 = J * TC_BN;
      // column-side inputs of this warp's 64 columns (independent of the MMAs)
      __syncwarp();
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int cc = lane + 32 * u;
        const int64_t scol = c0 + half * 64 + cc;
        uint4 bw = make_uint4(0u, 0u, 0u, 0u);
        float4 v4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (scol < ep.n) {
          if (narrow) {
            const uint32_t *bp = ep.bits + scol * ep.words;
            bw.x = bp[0];
            if (ep.words > 1) bw.y = bp[1];
            if (ep.words > 2) bw.z = bp[2];
            if (ep.words > 3) bw.w = bp[3];
          }
          const float2 cw = ep.w[scol], ch = ep.h[scol];
          v4 = make_float4(cw.x, cw.y, ch.x, ch.y);
        }
        wb[cc] = bw;
        wwh[cc] = v4;
      }
      const int64_t srow = r0 + r;
      uint32_t rb[9];
      float2 hrow = make_float2(0.0f, 0.0f), wrow = hrow;
#pragma unroll
      for (int w = 0; w < 9; ++w) rb[w] = 0u;
      if (srow < ep.n) {
#pragma unroll
        for (int w = 0; w < 9; ++w)
          if (w < ep.words) rb[w] = ep.bits[srow * ep.words + w];
        hrow = ep.h[srow];
        wrow = ep.w[srow];
      }
      const df32 wr_s0 = df_add(df32{wrow.x, wrow.y}, s0sq);
      const df32 nh_row = {-hrow.x, -hrow.y};
      __syncwarp();
      if (!mbar_wait(&tfull[b], (uint32_t)((tcount >> 1) & 1), ep.wait_ns)) {
        fail();
        break;
      }
      if (*abort_flag) break;
      tc_fence_after();
      const uint32_t taddr = tmem_base + (static_cast<uint32_t>(quarter * 32) << 16) +
                             (uint32_t)(b * 2 * TC_BN + half * 64);
#pragma unroll 1
      for (int ch = 0; ch < 64 / TC_CHUNK; ++ch) {
        float a0[TC_CHUNK], a1[TC_CHUNK];
        tmem_ld_16cols(taddr + ch * TC_CHUNK, a0);
        if (two) tmem_ld_16cols(taddr + TC_BN + ch * TC_CHUNK, a1);
        tmem_wait_ld();
        if (ch == 64 / TC_CHUNK - 1) {
          // all of this warp's reads of buffer b are done: release it to the MMA warp
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&tempty[b]);
        }
#pragma unroll
        for (int j = 0; j < TC_CHUNK; ++j) {
          const int cl = ch * TC_CHUNK + j;  // column within the warp's 64
          int diff = 0;
          if (narrow) {
            const uint4 bw = wb[cl];
            diff = __popc(rb[0] ^ bw.x) + __popc(rb[1] ^ bw.y) + __popc(rb[2] ^ bw.z) +
                   __popc(rb[3] ^ bw.w);
          } else {
            const int64_t scol = c0 + half * 64 + cl;
            if (scol < ep.n) {
#pragma unroll
              for (int w = 0; w < 9; ++w)
                if (w < ep.words) diff += __popc(rb[w] ^ __ldg(ep.bits + scol * ep.words + w));
            }
          }
          const int B = ep.N - 2 * diff;
          const float4 cv = wwh[cl];
          const df32 acc = two ? df_two_sum(a0[j], a1[j]) : df32{a0[j], 0.0f};
          const df32 a = df_add(df_add(wr_s0, df32{cv.x, cv.y}), acc);
          df32 v = df_mul(a, (float)(1 + B));
          v = df_add(v, (float)B);
          v = df_add(v, df_add(nh_row, df32{-cv.z, -cv.w}));
          v = df_mul(v, ep.inv_n);
          if (c0 + half * 64 + cl == srow) v = df_add(v, shift);
          st[lane * TC_STG_LD + j] = make_float2(v.hi, v.lo);
        }
        __syncwarp();
        // coalesced write-out: half-warps take rows, lanes 16 consecutive columns
        const int cb = half * 64 + ch * TC_CHUNK;
#pragma unroll 4
        for (int q = 0; q < 16; ++q) {
          const int rr = 2 * q + (lane >> 4), cc = lane & 15;
          const int64_t orow = r0 + quarter * 32 + rr, ocol = c0 + cb + cc;
          if (orow < ep.n && ocol <= orow) {
            const float2 v = st[rr * TC_STG_LD + cc];
            ep.T32[orow * ep.n + ocol] = v.x + v.y;
            if (ep.T64) ep.T64[orow * ep.n + ocol] = df_to_double(df32{v.x, v.y});
          }
        }
        __syncwarp();
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "r"(TC_TMEM_COLS)
                 : "memory");
  }
}

// ------------------------------------------------------------ host side
static int make_map(CUtensorMap *map, const void *base, int64_t rows, int64_t Kp) {
  auto fn = encode_fn();
  if (!fn) {
    set_last_error("cuTensorMapEncodeTiled is unavailable");
    return VMCK_ERR_CUDA;
  }
  cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(Kp * 2)};
  cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)TC_BM};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_last_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return VMCK_ERR_CUDA;
  }
  return VMCK_OK;
}

static int tc_mp(int M) { return (M + TC_BK - 1) / TC_BK * TC_BK; }
static int64_t tc_kp(int M, bool split) { return (split ? 4 : 1) * (int64_t)tc_mp(M); }

int64_t gram_tc_workspace_doubles(int M, int64_t n) {
  // two bf16 panels of n x Kp (split layout, the larger one), plus alignment
  return (2 * n * tc_kp(M, true) * 2 + 1024) / 8 + 1;
}

static size_t tc_smem_bytes() {
  return 1024 /*align*/ + 2 * TC_STAGES * TC_BM * TC_BK * 2 +
         TC_EPI_WARPS * 32 * TC_STG_LD * 8 + TC_EPI_WARPS * 64 * (16 + 16) +
         8 * (2 * TC_STAGES + 5) + 16 + 256 /*margin*/;
}

int gram_tc_launch(vmck_ctx *ctx, cudaStream_t st, const float *tanh_theta, const uint32_t *bits,
                   int words, int N, int M, int64_t n, const float2 *h, const float2 *w,
                   const float2 *s0sq, double inv_n, double diag_shift, double *T64, float *T32,
                   double *ws, int split, int32_t *status) {
  (void)ctx;
  if (words > 9) {
    set_last_error("rbm_gram tensor-core mode supports N <= 288");
    return VMCK_ERR_UNSUPPORTED;
  }
  if (n >= (1ll << 31) / TC_BM) {
    set_last_error("rbm_gram tensor-core mode: n too large");
    return VMCK_ERR_UNSUPPORTED;
  }
  const int64_t Kp = tc_kp(M, split != 0);
  __nv_bfloat16 *L = reinterpret_cast<__nv_bfloat16 *>(
      (reinterpret_cast<uintptr_t>(ws) + 1023) & ~uintptr_t(1023));
  __nv_bfloat16 *R = L + n * Kp;  // n * Kp * 2 bytes: a multiple of 128, so 16-byte aligned
  tc_split_kernel<<<ceil_div(n * Kp, 256), 256, 0, st>>>(tanh_theta, n, M, tc_mp(M), (int)Kp,
                                                          split, L, R);
  int rc = check_launch("gram_tc split");
  if (rc) return rc;
  CUtensorMap mL, mR;
  if ((rc = make_map(&mL, L, n, Kp))) return rc;
  if ((rc = make_map(&mR, R, n, Kp))) return rc;
  const size_t smem = tc_smem_bytes();
  VMCK_CUDA(cudaFuncSetAttribute(gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
  const int64_t nt = (n + TC_BM - 1) / TC_BM, tiles = nt * (nt + 1) / 2;
  TcEpilogue ep{bits, words, N, n, h, w, s0sq, (float)inv_n, diag_shift, T64, T32, status,
                wait_limit_ns()};
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned grid = (unsigned)std::min<int64_t>(tiles, sms);
  const int kb_hi = split ? tc_mp(M) / TC_BK : 0;
  gram_tc_kernel<<<grid, TC_THREADS, smem, st>>>(mL, mR, (int)(Kp / TC_BK), kb_hi, tiles, ep);
  return check_launch("gram_tc");
}

}  // namespace vmck

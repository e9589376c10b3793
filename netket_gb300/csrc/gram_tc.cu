// Tensor-core form of the structured minSR Gram matrix (sm_103a: tcgen05 + TMA).
//
// T = (A o (1 + B) + B - g 1^T - 1 g^T + c 1 1^T) / n + diag_shift I with
// A = t t^T (t = tanh theta, n x M) and B = x x^T (exact, popcount).  A runs on
// the 5th-generation tensor cores: each CTA owns one 128 x 128 lower-triangular
// tile of T, streams K-slabs of the two operand panels with TMA
// (cp.async.bulk.tensor, 128-byte swizzle) into a 4-stage shared-memory ring
// guarded by mbarriers, issues tcgen05.mma (kind::f16, BF16 in, FP32
// accumulate in tensor memory) from one thread, and the four warps read the
// accumulator back with tcgen05.ld for the fused epilogue that writes T64 / T32.
//
// Precision: t arrives rounded to hi + lo (two BF16 terms) or to one BF16; the
// operand panels [hi | hi | lo | lo] and [hi | lo | hi | lo] make one GEMM form
// all four products, i.e. t t^T exactly up to FP32 accumulation.  Every other
// ingredient of T (column means, g) is computed from the same rounded t, so T
// is the exact Gram matrix of a slightly perturbed Jacobian and keeps its
// positive definiteness.  The epilogue works in double-float FP32.
//
// Every mbarrier wait is bounded by wall time (2 s, %globaltimer); a wait that
// runs out sets VMCK_DEV_TIMEOUT in the status word and the CTA winds down
// (waiting, again bounded, for its own TMA copies) instead of hanging.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "gram_tc.cuh"

namespace vmck {

constexpr int TC_BM = 128;     // tile rows (UMMA M)
constexpr int TC_BN = 128;     // tile cols (UMMA N)
constexpr int TC_BK = 64;      // K slab: 64 bf16 = 128 bytes = one swizzle row
constexpr int TC_STAGES = 4;
constexpr int TC_UMMA_K = 16;  // K per tcgen05.mma for 16-bit inputs
constexpr int TC_ACC = 4;           // accumulators the K-blocks rotate over
constexpr int TC_TMEM_COLS = 512;  // TC_ACC x TC_BN columns: all of tensor memory
constexpr unsigned long long TC_WAIT_NS = 2000000000ull;
constexpr int TC_THREADS = 128;

// ------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: true on completion, false when TC_WAIT_NS elapsed.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > TC_WAIT_NS) return false;
  }
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar,
                                            int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

// UMMA shared-memory descriptor, K-major operand with 128-byte swizzle:
// start address >> 4 (bits 0-13), leading byte offset (unused for swizzled
// K-major, 16 B) (bits 16-29), stride byte offset 1024 B between 8-row groups
// (bits 32-45), descriptor version 1 (bits 46-47), layout SWIZZLE_128B = 2
// (bits 61-63).
__device__ __forceinline__ uint64_t umma_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFF);
  d |= static_cast<uint64_t>(1) << 16;
  d |= static_cast<uint64_t>(1024 >> 4) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  d |= static_cast<uint64_t>(2) << 61;
  return d;
}

// Instruction descriptor for kind::f16: FP32 accumulate (bits 4-5 = 1), A and B
// BF16 (bits 7-9 = 1, bits 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
         (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld_32cols(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// ------------------------------------------------------------ operand panels
// Input t is already rounded (exactly hi + lo, or exactly one BF16), so
//   split:  L = [hi | hi | lo | lo], R = [hi | lo | hi | lo]  ->  L R^T = t t^T,
//   single: L = R = [bf16(t)]                                 ->  L R^T = t t^T,
// exactly up to the FP32 accumulation: T is then the exact Gram matrix of the
// rounded Jacobian and stays positive semidefinite.  Rows are Kp long
// (zero padding to a multiple of 64).
__global__ void tc_split_kernel(const float *__restrict__ t, int64_t n, int M, int Kp, int split,
                                __nv_bfloat16 *__restrict__ L, __nv_bfloat16 *__restrict__ R) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= n * Kp) return;
  const int64_t s = e / Kp;
  const int k = (int)(e % Kp);
  __nv_bfloat16 lv = __float2bfloat16(0.0f), rv = lv;
  const int seg = k / M, j = k % M;
  if (!split) {
    if (seg == 0) lv = rv = __float2bfloat16(t[s * M + j]);
  } else if (seg < 4) {
    const float v = t[s * M + j];
    const __nv_bfloat16 hi = __float2bfloat16(v);
    const __nv_bfloat16 lo = __float2bfloat16(v - __bfloat162float(hi));
    lv = (seg < 2) ? hi : lo;
    rv = (seg & 1) ? lo : hi;
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
};

__device__ inline void tc_tri_tile(int64_t bid, int64_t &I, int64_t &J) {
  int64_t i = (int64_t)((sqrt(8.0 * (double)bid + 1.0) - 1.0) * 0.5);
  while (i * (i + 1) / 2 > bid) --i;
  while ((i + 1) * (i + 2) / 2 <= bid) ++i;
  I = i;
  J = bid - i * (i + 1) / 2;
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    gram_tc_kernel(const __grid_constant__ CUtensorMap mapL,
                   const __grid_constant__ CUtensorMap mapR, int num_kb, TcEpilogue ep) {
  extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
  // 1024-byte alignment for the 128B-swizzled operand slabs
  unsigned char *smem = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
  constexpr int SLAB = TC_BM * TC_BK * 2;  // 16 KB
  unsigned char *slabA = smem;
  unsigned char *slabB = smem + TC_STAGES * SLAB;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + 2 * TC_STAGES * SLAB);
  uint64_t *empty = full + TC_STAGES;
  uint64_t *done = empty + TC_STAGES;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
  int *abort_flag = reinterpret_cast<int *>(tmem_slot + 1);
  uint32_t *colbits = reinterpret_cast<uint32_t *>(abort_flag + 1);  // [TC_BN][words]
  float2 *colh = reinterpret_cast<float2 *>(
      (reinterpret_cast<uintptr_t>(colbits + TC_BN * 9) + 7) & ~uintptr_t(7));  // [TC_BN]
  float2 *colw = colh + TC_BN;                                                  // [TC_BN]

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // once any CTA has timed out, the remaining ones do no work
  if (tid == 0) *reinterpret_cast<volatile int *>(tmem_slot + 1) =
      (ep.status && (*reinterpret_cast<volatile int32_t *>(ep.status) & VMCK_DEV_TIMEOUT)) ? 1 : 0;
  __syncthreads();
  if (*reinterpret_cast<volatile int *>(tmem_slot + 1)) return;
  __syncthreads();
  int64_t I, J;
  tc_tri_tile(blockIdx.x, I, J);
  const int64_t r0 = I * TC_BM, c0 = J * TC_BN;

  if (warp == 0) {
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
    mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapL)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapR)) : "memory");
  }
  // stage the column-side epilogue inputs while the pipeline runs
  for (int e = tid; e < TC_BN * ep.words; e += TC_THREADS) {
    const int c = e / ep.words, w = e % ep.words;
    colbits[c * 9 + w] = (c0 + c < ep.n) ? ep.bits[(c0 + c) * ep.words + w] : 0u;
  }
  for (int c = tid; c < TC_BN; c += TC_THREADS) {
    colh[c] = (c0 + c < ep.n) ? ep.h[c0 + c] : make_float2(0.0f, 0.0f);
    colw[c] = (c0 + c < ep.n) ? ep.w[c0 + c] : make_float2(0.0f, 0.0f);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  // ---------------- producer + MMA issuer: one thread drives the ring
  if (tid == 0) {
    const uint32_t idesc = umma_idesc_bf16(TC_BM, TC_BN);
    const int pre = num_kb < TC_STAGES ? num_kb : TC_STAGES;
    bool ok = true;
    int issued = 0;
    for (int kb = 0; kb < pre; ++kb) {
      mbar_expect_tx(&full[kb], 2 * SLAB);
      tma_load_2d(slabA + kb * SLAB, &mapL, &full[kb], kb * TC_BK, (int)r0);
      tma_load_2d(slabB + kb * SLAB, &mapR, &full[kb], kb * TC_BK, (int)c0);
      ++issued;
    }
    for (int kb = 0; kb < num_kb && ok; ++kb) {
      const int s = kb % TC_STAGES;
      const uint32_t ph = (kb / TC_STAGES) & 1;
      if (!mbar_wait(&full[s], ph)) {
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t a0 = smem_u32(slabA + s * SLAB), b0 = smem_u32(slabB + s * SLAB);
      // K-blocks rotate over TC_ACC accumulators: the tensor core's FP32
      // accumulation error grows with the number of accumulate steps, so each
      // accumulator takes a quarter of them and the epilogue sums the four.
      const uint32_t dacc = tmem_base + (uint32_t)((kb % TC_ACC) * TC_BN);
#pragma unroll
      for (int k = 0; k < TC_BK / TC_UMMA_K; ++k) {
        const uint32_t off = k * TC_UMMA_K * 2;  // bytes along the swizzled row
        umma_bf16(dacc, umma_desc_sw128(a0 + off), umma_desc_sw128(b0 + off), idesc,
                  (kb >= TC_ACC || k > 0) ? 1u : 0u);
      }
      umma_commit(&empty[s]);
      const int nk = kb + TC_STAGES;
      if (nk < num_kb) {
        // the slab is refilled once the MMAs that read it have completed
        if (!mbar_wait(&empty[s], ph)) {
          ok = false;
          break;
        }
        mbar_expect_tx(&full[s], 2 * SLAB);
        tma_load_2d(slabA + s * SLAB, &mapL, &full[s], nk * TC_BK, (int)r0);
        tma_load_2d(slabB + s * SLAB, &mapR, &full[s], nk * TC_BK, (int)c0);
        ++issued;
      }
    }
    if (ok) {
      umma_commit(done);
    } else {
      // wind down: let every TMA copy this CTA issued land before exiting
      *abort_flag = 1;
      if (ep.status) atomicOr(ep.status, VMCK_DEV_TIMEOUT);
      for (int q = 0; q < issued; ++q) {
        const int s = q % TC_STAGES;
        mbar_wait(&full[s], (q / TC_STAGES) & 1);
      }
      mbar_wait(&empty[(num_kb - 1) % TC_STAGES], ((num_kb - 1) / TC_STAGES) & 1);
    }
  }
  __syncwarp();
  // ---------------- epilogue: all four warps
  bool have = true;
  if (!mbar_wait(done, 0)) have = false;
  __syncthreads();
  if (*abort_flag) have = false;
  if (!have) {
    if (tid == 0 && ep.status) atomicOr(ep.status, VMCK_DEV_TIMEOUT);
  } else {
    tc_fence_after();
    const int r = warp * 32 + lane;  // TMEM lane == tile row
    const int64_t srow = r0 + r;
    uint32_t rb[9];
    float2 hrow = make_float2(0.0f, 0.0f), wrow = hrow;
    if (srow < ep.n) {
      for (int w = 0; w < ep.words; ++w) rb[w] = ep.bits[srow * ep.words + w];
      hrow = ep.h[srow];
      wrow = ep.w[srow];
    }
    const df32 shift = df_from(ep.diag_shift);
    const df32 s0sq = {ep.s0sq->x, ep.s0sq->y};
    const df32 wr_s0 = df_add(df32{wrow.x, wrow.y}, s0sq);
    const uint32_t lane_addr = tmem_base + (static_cast<uint32_t>(warp * 32) << 16);
    const int nacc = num_kb < TC_ACC ? num_kb : TC_ACC;
#pragma unroll 1
    for (int q = 0; q < TC_BN / 32; ++q) {
      df32 acc[32];
      {
        float part[32];
        tmem_ld_32cols(lane_addr + q * 32, part);
#pragma unroll
        for (int j = 0; j < 32; ++j) acc[j] = {part[j], 0.0f};
      }
      for (int r = 1; r < nacc; ++r) {
        float part[32];
        tmem_ld_32cols(lane_addr + r * TC_BN + q * 32, part);
#pragma unroll
        for (int j = 0; j < 32; ++j) acc[j] = df_add(acc[j], part[j]);
      }
      if (srow < ep.n) {
        double *o64 = ep.T64 ? ep.T64 + srow * ep.n : nullptr;
        float *o32 = ep.T32 + srow * ep.n;
#pragma unroll 4
        for (int j = 0; j < 32; ++j) {
          const int c = q * 32 + j;
          const int64_t scol = c0 + c;
          if (scol < ep.n && scol <= srow) {
            int diff = 0;
            for (int w = 0; w < ep.words; ++w) diff += __popc(rb[w] ^ colbits[c * 9 + w]);
            const int B = ep.N - 2 * diff;
            df32 a = df_add(df_add(wr_s0, df32{colw[c].x, colw[c].y}), acc[j]);
            df32 v = df_mul(a, (float)(1 + B));
            v = df_add(v, (float)B);
            v = df_add(v, df32{-hrow.x, -hrow.y});
            v = df_add(v, df32{-colh[c].x, -colh[c].y});
            v = df_mul(v, ep.inv_n);
            if (scol == srow) v = df_add(v, shift);
            if (o64) o64[scol] = df_to_double(v);
            o32[scol] = v.hi + v.lo;
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "r"(TC_TMEM_COLS)
                 : "memory");
  }
}

// ------------------------------------------------------------ host side
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

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

static int64_t tc_kp(int M, bool split) {
  const int64_t k = split ? 4 * (int64_t)M : M;
  return (k + TC_BK - 1) / TC_BK * TC_BK;
}

int64_t gram_tc_workspace_doubles(int M, int64_t n) {
  // two bf16 panels of n x Kp (split layout, the larger one), plus alignment
  return (2 * n * tc_kp(M, true) * 2 + 1024) / 8 + 1;
}

static size_t tc_smem_bytes() {
  return 1024 /*align*/ + 2 * TC_STAGES * TC_BM * TC_BK * 2 + 8 * (2 * TC_STAGES + 1) + 16 +
         TC_BN * 9 * 4 + 8 + 2 * TC_BN * 8 + 256 /*margin*/;
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
  tc_split_kernel<<<ceil_div(n * Kp, 256), 256, 0, st>>>(tanh_theta, n, M, (int)Kp, split, L, R);
  int rc = check_launch("gram_tc split");
  if (rc) return rc;
  CUtensorMap mL, mR;
  if ((rc = make_map(&mL, L, n, Kp))) return rc;
  if ((rc = make_map(&mR, R, n, Kp))) return rc;
  const size_t smem = tc_smem_bytes();
  VMCK_CUDA(cudaFuncSetAttribute(gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
  const int64_t nt = (n + TC_BM - 1) / TC_BM;
  TcEpilogue ep{bits, words, N, n, h, w, s0sq, (float)inv_n, diag_shift, T64, T32, status};
  gram_tc_kernel<<<(unsigned)(nt * (nt + 1) / 2), TC_THREADS, smem, st>>>(mL, mR,
                                                                          (int)(Kp / TC_BK), ep);
  return check_launch("gram_tc");
}

}  // namespace vmck

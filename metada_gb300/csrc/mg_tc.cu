// Tensor-core GEMM for sm_103a: C = A B^T (+ bias, optional SiLU), A (M x K)
// and B (N x K) BF16 K-major in global memory, FP32 accumulation in tensor
// memory, written with inline PTX.  A persistent CTA per SM (warp-specialised):
//   * warp 0 (one lane): TMA (cp.async.bulk.tensor.2d) of 128-row x 64-column
//     k-blocks of A and BN x 64 of B into a 3- or 4-stage ring with the 128-byte
//     swizzle, completion by mbarrier (arrive.expect_tx / complete_tx);
//   * warp 1 (one lane): tcgen05.mma.cta_group::1.kind::f16 (M = 128, N = BN,
//     K = 16 per instruction, four per k-block), shared-memory descriptors in
//     the SM100 format (SWIZZLE_128B K-major, SBO = 1024 B), into one of two
//     TMEM accumulators; tcgen05.commit frees ring stages and hands finished
//     accumulators over;
//   * warps 2-9: the epilogue of the other accumulator (tcgen05.ld.32x32b,
//     bias, SiLU, FP32 and/or BF16 stores; two warps per 32 TMEM lanes, one
//     column half each), overlapping the next tile's MMAs.
// Every mbarrier wait is bounded; a role that gives up records an error flag
// and raises an abort the other roles see at their next wait; copies and
// MMAs in flight are waited for (bounded) and TMEM is freed, so the host sees
// MG_ERR_TIMEOUT instead of a hung GPU.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "mg_internal.h"
#include "mg_tcgen05.cuh"

namespace {

constexpr int kBM = 128;       // rows per tile (MMA M)
constexpr int kBK = 64;        // K per stage (one 128-byte swizzle row of BF16)
constexpr int kEpiWarps = 8;   // epilogue warps: two per 32 TMEM lanes (column halves)
constexpr int kThreads = 64 + 32 * kEpiWarps;  // TMA warp, MMA warp, epilogue warps
// Shared-memory ring of A and B k-blocks (the widest tile keeps three so the
// ring and the epilogue staging fit in 227 KB).
__host__ __device__ constexpr int ring_stages(int bn) { return bn >= 256 ? 3 : 4; }
using namespace mg::t5;

__device__ __forceinline__ float silu_f(float z) { return z / (1.0f + expf(-z)); }
// SiLU for BF16-only outputs (hidden activations): the hardware exp2-based
// exponential and the approximate division, a few ulp, far below BF16's
// 2^-8; for z < -88 the denominator is +inf and the result 0, the limit.
__device__ __forceinline__ float silu_bf16(float z) { return __fdividef(z, 1.0f + __expf(-z)); }

// Persistent, warp-specialised GEMM: one CTA per SM walks the 128-row tiles
// (t = blockIdx.x, + gridDim.x, ...).  Warp 0 (one lane) streams A and B
// k-blocks through a kStages ring (full/empty mbarriers); warp 1 (one lane)
// issues the MMAs into one of two TMEM accumulators (acc_full/acc_empty);
// warps 2-9 drain the other accumulator (bias, SiLU, stores), so the
// epilogue of tile t overlaps the MMAs of tile t + 1 and the loads beyond.
// Every wait is bounded; a role that gives up raises `abort`, the others
// leave at their next wait, copies and MMAs in flight are waited for
// (bounded), and TMEM is freed before the CTA exits.
template <int BN>
__global__ void __launch_bounds__(kThreads, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, int M,
                   int N, int K, const float* __restrict__ bias, int act, float* __restrict__ C32,
                   __nv_bfloat16* __restrict__ C16, int ldc, int* __restrict__ err, int skip_kb) {
  // skip_kb >= 0 (the wait self-test only): the producer never issues that
  // k-block of the CTA's first tile, so the MMA warp's wait for it runs out.
  static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256, "N tile");
  constexpr int kStages = ring_stages(BN);
  constexpr uint32_t kABytes = kBM * kBK * 2, kBBytes = BN * kBK * 2, kStageBytes = kABytes + kBBytes;
  constexpr uint32_t kAccCols = BN < 32 ? 32 : BN;  // one accumulator; allocation unit a power of two >= 32
  constexpr uint32_t kTmemCols = 2 * kAccCols;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte aligned stage buffers (required by the 128-byte swizzle).
  unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* sA = base;                      // kStages x kABytes
  unsigned char* sB = base + kStages * kABytes;  // kStages x kBBytes
  float* stg_all = reinterpret_cast<float*>(base + kStages * kStageBytes);  // kEpiWarps x 32 x 33
  __shared__ uint64_t full_bar[kStages];   // k-block landed
  __shared__ uint64_t empty_bar[kStages];  // MMAs reading the stage have drained
  __shared__ uint64_t accf_bar[2];         // accumulator complete
  __shared__ uint64_t acce_bar[2];         // accumulator read out by the epilogue warps
  __shared__ uint64_t done_bar;            // every MMA of this CTA drained
  __shared__ uint32_t tmem_base_s;
  __shared__ int abort_s;
  __shared__ float sbias[BN];  // bias (0 past N or without one)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = (K + kBK - 1) / kBK;
  const int ntiles = (M + kBM - 1) / kBM;
  volatile int* abort = &abort_s;

  for (int n = threadIdx.x; n < BN; n += kThreads) sbias[n] = (bias && n < N) ? bias[n] : 0.0f;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(&accf_bar[a], 1);
      mbar_init(&acce_bar[a], kEpiWarps);
    }
    mbar_init(&done_bar, 1);
    abort_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {  // TMEM: two accumulators of BN FP32 columns x 128 lanes
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base_s;

  if (warp == 0) {
    if (lane == 0) {  // TMA producer
      uint32_t g = 0;  // k-blocks issued
      uint32_t skipped = 0xffffffffu;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const int m0 = t * kBM;
        for (int kb = 0; kb < nk; ++kb) {
          const int s = (int)(g % kStages);
          const uint32_t ph = (g / kStages) & 1u;
          if (!mbar_wait_ab(&empty_bar[s], ph ^ 1u, abort)) {
            ok = false;
            break;
          }
          if (t == (int)blockIdx.x && kb == skip_kb) {
            skipped = g++;
            continue;
          }
          mbar_expect_tx(&full_bar[s], kStageBytes);
          tma_load_2d(sA + s * kABytes, &mapA, &full_bar[s], kb * kBK, m0);
          tma_load_2d(sB + s * kBBytes, &mapB, &full_bar[s], kb * kBK, 0);
          ++g;
        }
      }
      if (!ok) {
        *abort = 1;
        atomicExch(err, 1);
      }
      // Copies into this CTA's shared memory must land before it exits: wait
      // (bounded) for the last issue of every stage.
      for (uint32_t j = g > (uint32_t)kStages ? g - kStages : 0u; j < g; ++j)
        if (j != skipped) mbar_wait(&full_bar[j % kStages], (j / kStages) & 1u);
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      constexpr uint32_t idesc = idesc_bf16_f32(kBM, BN);
      uint32_t g = 0;
      int lt = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++lt) {
        const int ab = lt & 1;
        if (!mbar_wait_ab(&acce_bar[ab], (((uint32_t)lt >> 1) & 1u) ^ 1u, abort)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t dacc = tmem + (uint32_t)ab * kAccCols;
        for (int kb = 0; kb < nk; ++kb) {
          const int s = (int)(g % kStages);
          const uint32_t ph = (g / kStages) & 1u;
          if (!mbar_wait_ab(&full_bar[s], ph, abort)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t a0 = smem_u32(sA + s * kABytes), b0 = smem_u32(sB + s * kBBytes);
#pragma unroll
          for (int kk = 0; kk < kBK / 16; ++kk)
            mma_bf16(dacc, smem_desc_sw128(a0 + kk * 32), smem_desc_sw128(b0 + kk * 32), idesc,
                     (kb > 0 || kk > 0) ? 1u : 0u);
          mma_commit(&empty_bar[s]);
          ++g;
        }
        if (!ok) break;
        mma_commit(&accf_bar[ab]);
      }
      if (!ok) {
        *abort = 1;
        atomicExch(err, 1);
      }
      // Every MMA issued must drain before TMEM is freed.
      mma_commit(&done_bar);
      mbar_wait(&done_bar, 0);
    }
  } else {  // epilogue warps: TMEM lanes 32 (warp % 4) .. + 31 are rows of the tile
    const int eg = warp & 3;
    float* stg = stg_all + (warp - 2) * (32 * 33);
    // Columns of this warp: one half each for the two warps of a lane group
    // (tiles narrower than 64 columns: the first warp of the group takes all).
    const int half = (warp - 2) / 4;
    const int cb = BN >= 64 ? half * (BN / 2) : 0;
    const int ce = BN >= 64 ? cb + BN / 2 : (half == 0 ? BN : 0);
    const bool pairs16 = C16 && (ldc % 2 == 0) && (((uintptr_t)C16 & 3) == 0);
    // BF16-only output with 16-byte aligned rows: each lane packs its row's
    // 32 columns and stores them directly (no staging).
    const bool direct16 = C16 && !C32 && (ldc % 8 == 0) && (((uintptr_t)C16 & 15) == 0);
    int lt = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++lt) {
      const int ab = lt & 1;
      const bool ready = mbar_wait_ab(&accf_bar[ab], ((uint32_t)lt >> 1) & 1u, abort);
      if (!__all_sync(0xffffffffu, ready)) {  // one decision per warp, so tcgen05.ld stays converged
        if (lane == 0) {
          *abort = 1;
          atomicExch(err, 1);
        }
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int rbase = t * kBM + eg * 32;
      const uint32_t trow = tmem + (uint32_t)ab * kAccCols + ((uint32_t)(eg * 32) << 16);
#pragma unroll 1
      for (int c0 = cb; c0 < ce; c0 += 32) {
        uint32_t v[32];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
              "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
              "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
              "=r"(v[30]), "=r"(v[31])
            : "r"(trow + (uint32_t)c0));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (direct16 && c0 + 32 <= N) {
          uint32_t pk[16];
#pragma unroll
          for (int j = 0; j < 32; j += 2) {
            float x0 = __uint_as_float(v[j]) + sbias[c0 + j];
            float x1 = __uint_as_float(v[j + 1]) + sbias[c0 + j + 1];
            if (act) {
              x0 = silu_bf16(x0);
              x1 = silu_bf16(x1);
            }
            const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
            pk[j / 2] = *reinterpret_cast<const uint32_t*>(&h);
          }
          const int row = rbase + lane;
          if (row < M) {
            uint4* dst = reinterpret_cast<uint4*>(C16 + (int64_t)row * ldc + c0);
#pragma unroll
            for (int q = 0; q < 4; ++q) dst[q] = make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
          }
          continue;
        }
        // Otherwise the warp stages its 32 rows x 32 columns through shared
        // memory, so the global stores are row segments: 128 B (FP32) or two
        // 64 B rows (BF16) per warp instruction.
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          float x = __uint_as_float(v[j]) + sbias[c0 + j];
          if (act) x = C32 ? silu_f(x) : silu_bf16(x);
          stg[lane * 33 + j] = x;
        }
        __syncwarp();
        if (C32) {
          const int n = c0 + lane;
#pragma unroll 4
          for (int r = 0; r < 32; ++r) {
            const int row = rbase + r;
            if (row < M && n < N) C32[(int64_t)row * ldc + n] = stg[r * 33 + lane];
          }
        }
        if (C16) {
          if (pairs16) {
            const int half = lane >> 4, cc = (lane & 15) * 2, n = c0 + cc;
#pragma unroll 4
            for (int r = 0; r < 32; r += 2) {
              const int row = rbase + r + half;
              if (row >= M) continue;
              const float x0 = stg[(r + half) * 33 + cc], x1 = stg[(r + half) * 33 + cc + 1];
              __nv_bfloat16* dst = C16 + (int64_t)row * ldc + n;
              if (n + 1 < N) *reinterpret_cast<__nv_bfloat162*>(dst) = __floats2bfloat162_rn(x0, x1);
              else if (n < N) *dst = __float2bfloat16_rn(x0);
            }
          } else {
            const int n = c0 + lane;
            for (int r = 0; r < 32; ++r) {
              const int row = rbase + r;
              if (row < M && n < N) C16[(int64_t)row * ldc + n] = __float2bfloat16_rn(stg[r * 33 + lane]);
            }
          }
        }
        __syncwarp();
      }
      // This warp's reads of the accumulator are done: hand it back.
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce_bar[ab]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

// ---- host side: tensor maps through the driver entry point ----
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    cudaGetLastError();
  });
  return fn;
}

// rows x cols BF16 row-major (cols contiguous), box box_rows x 64, 128-byte swizzle.
bool make_map(CUtensorMap* map, const void* ptr, int64_t rows, int64_t cols, int box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
int launch(mg_context* ctx, const CUtensorMap& ma, const CUtensorMap& mb, int M, int N, int K, const float* bias,
           int act, float* C32, __nv_bfloat16* C16, int ldc, int* err, int skip_kb) {
  const size_t smem =
      1024 + (size_t)ring_stages(BN) * (kBM * kBK * 2 + BN * kBK * 2) + sizeof(float) * kEpiWarps * 32 * 33;
  MG_TRY_CUDA(cudaFuncSetAttribute(tc_gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int tiles = (M + kBM - 1) / kBM;
  const int grid = std::max(1, std::min(tiles, ctx->num_sms));
  tc_gemm_kernel<BN><<<(unsigned)grid, kThreads, smem, ctx->stream>>>(ma, mb, M, N, K, bias, act, C32, C16, ldc, err,
                                                                      skip_kb);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // namespace

namespace mg {

// Internal entry used by the MLP inference path as well.
int tc_gemm_run(mg_context* ctx, const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K,
                const float* bias, int act, float* C32, __nv_bfloat16* C16, int ldc, int* err, int skip_kb) {
  if (N < 1 || N > 256 || K % 8 != 0 || M <= 0 || K <= 0)
    return fail(ctx, MG_ERR_ARG, "tensor-core GEMM: need 1 <= N <= 256, K > 0, K % 8 == 0");
  if (((uintptr_t)A | (uintptr_t)B) & 15)
    return fail(ctx, MG_ERR_ARG, "tensor-core GEMM: operands must be 16-byte aligned");
  CUtensorMap ma, mb;
  const int bn = N <= 16 ? 16 : N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
  if (!make_map(&ma, A, M, K, kBM) || !make_map(&mb, B, N, K, bn))
    return fail(ctx, MG_ERR_CUDA, "tensor-core GEMM: cuTensorMapEncodeTiled failed");
  switch (bn) {
    case 16: return launch<16>(ctx, ma, mb, M, N, K, bias, act, C32, C16, ldc, err, skip_kb);
    case 32: return launch<32>(ctx, ma, mb, M, N, K, bias, act, C32, C16, ldc, err, skip_kb);
    case 64: return launch<64>(ctx, ma, mb, M, N, K, bias, act, C32, C16, ldc, err, skip_kb);
    case 128: return launch<128>(ctx, ma, mb, M, N, K, bias, act, C32, C16, ldc, err, skip_kb);
    default: return launch<256>(ctx, ma, mb, M, N, K, bias, act, C32, C16, ldc, err, skip_kb);
  }
}

int tc_gemm_bf16(mg_context* ctx, const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K,
                 const float* bias, int act, float* C32, __nv_bfloat16* C16, int ldc, int* err) {
  return tc_gemm_run(ctx, A, B, M, N, K, bias, act, C32, C16, ldc, err, -1);
}

}  // namespace mg

extern "C" int mg_gemm_bf16_tc(mg_context* ctx, const void* A, const void* B, int32_t M, int32_t N, int32_t K,
                               const float* bias, int32_t silu, float* C) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(A && B && C, "mg_gemm_bf16_tc: null operand");
  int* err = static_cast<int*>(mg::workspace(ctx, 256));
  if (!err) return MG_ERR_NOMEM;
  MG_TRY_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  const int rc = mg::tc_gemm_bf16(ctx, static_cast<const __nv_bfloat16*>(A), static_cast<const __nv_bfloat16*>(B), M,
                                  N, K, bias, silu, C, nullptr, N, err);
  if (rc != MG_OK) return rc;
  int h = 0;
  MG_TRY_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MG_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
  if (h) return mg::fail(ctx, MG_ERR_TIMEOUT, "mg_gemm_bf16_tc: a bounded mbarrier wait gave up");
  return MG_OK;
}

// Self-test of the bounded waits: the same GEMM with one k-block of every
// CTA's first tile never loaded, so the MMA warp's wait for it gives up
// after its time limit and the others follow the abort.  *observed is the
// status the launch reports (MG_ERR_TIMEOUT when the waits work); the call
// returns MG_OK when the kernel came back and the context is usable.
extern "C" int mg_gemm_bf16_tc_wait_selftest(mg_context* ctx, const void* A, const void* B, int32_t M, int32_t N,
                                             int32_t K, float* C, int32_t* observed) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(A && B && C && observed, "mg_gemm_bf16_tc_wait_selftest: null argument");
  int* err = static_cast<int*>(mg::workspace(ctx, 256));
  if (!err) return MG_ERR_NOMEM;
  MG_TRY_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  const int rc = mg::tc_gemm_run(ctx, static_cast<const __nv_bfloat16*>(A), static_cast<const __nv_bfloat16*>(B), M,
                                 N, K, nullptr, 0, C, nullptr, N, err, 0);
  if (rc != MG_OK) return rc;
  int h = 0;
  MG_TRY_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MG_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
  *observed = h ? MG_ERR_TIMEOUT : MG_OK;
  return MG_OK;
}

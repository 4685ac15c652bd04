// TF32 tensor-core operands in shared memory and the 3-pass product:
// K-major operands with the 128-byte swizzle (a slab holds 32 TF32 columns
// of all its rows, 128 bytes per row, 8-row groups 1024 bytes apart), each
// value stored as a hi and a lo copy (hi = x rounded to TF32, lo = x - hi),
// and D += A B^T issued as hi*hi + hi*lo + lo*hi per K-step of 8.  Shared by
// the tensor-core local analyses (mg_letkf_tc.cu) and the tensor-core
// ensemble update of the uneven batch (mg_batch.cu).
#pragma once

#include <stdint.h>

#include "mg_tcgen05.cuh"

namespace mg {
namespace t5 {

// ---- operand addressing: K-major, 128-byte swizzle, TF32 in 32-bit words ----
// Byte offset of element (row r, column c) in an operand whose slabs (32
// columns each) hold `rows` rows.
static __device__ __forceinline__ uint32_t sw_off(int r, int c, uint32_t rows) {
  return (uint32_t)(c >> 5) * rows * 128u + (uint32_t)(r >> 3) * 1024u + (uint32_t)(r & 7) * 128u +
         ((uint32_t)(((c & 31) >> 2) ^ (r & 7)) << 4) + (uint32_t)(c & 3) * 4u;
}

static __device__ __forceinline__ void split(float x, float& h, float& l) {
  h = tf32_rna(x);
  l = x - h;
}

// The epilogues work on 8 columns at a time inside loops that are not
// unrolled: fully unrolled 32-column bodies at every call site made the
// kernel's code larger than the instruction caches.
//
// Row r, columns c0 .. c0+7 (c0 a multiple of 8): two 16-byte chunks
// (conflict-free across a warp's 32 consecutive rows).
static __device__ __forceinline__ void put_row8(unsigned char* hi, unsigned char* lo, int r, int c0, uint32_t rows,
                                         const float (&x)[8]) {
  const uint32_t base = (uint32_t)(c0 >> 5) * rows * 128u + (uint32_t)(r >> 3) * 1024u + (uint32_t)(r & 7) * 128u;
  const int j0 = (c0 & 31) >> 2;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float4 vh, vl;
    split(x[4 * h + 0], vh.x, vl.x);
    split(x[4 * h + 1], vh.y, vl.y);
    split(x[4 * h + 2], vh.z, vl.z);
    split(x[4 * h + 3], vh.w, vl.w);
    const uint32_t off = base + ((uint32_t)((j0 + h) ^ (r & 7)) << 4);
    *reinterpret_cast<float4*>(hi + off) = vh;
    *reinterpret_cast<float4*>(lo + off) = vl;
  }
}

// Row r, columns c0 .. c0+7 of an operand as values (hi + lo).
static __device__ __forceinline__ void get_row8(const unsigned char* hi, const unsigned char* lo, int r, int c0,
                                         uint32_t rows, float (&x)[8]) {
  const uint32_t base = (uint32_t)(c0 >> 5) * rows * 128u + (uint32_t)(r >> 3) * 1024u + (uint32_t)(r & 7) * 128u;
  const int j0 = (c0 & 31) >> 2;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const uint32_t off = base + ((uint32_t)((j0 + h) ^ (r & 7)) << 4);
    const float4 vh = *reinterpret_cast<const float4*>(hi + off);
    const float4 vl = *reinterpret_cast<const float4*>(lo + off);
    x[4 * h + 0] = vh.x + vl.x;
    x[4 * h + 1] = vh.y + vl.y;
    x[4 * h + 2] = vh.z + vl.z;
    x[4 * h + 3] = vh.w + vl.w;
  }
}

// Transposed: the thread's row kk of a matrix, columns n0 .. n0+7, goes to
// operand rows n0 .. n0+7 at column kk (4-byte stores, conflict-free across
// a warp's 32 consecutive kk).
static __device__ __forceinline__ void put_col8(unsigned char* hi, unsigned char* lo, int kk, int n0, uint32_t rows,
                                         const float (&x)[8]) {
  const uint32_t cb = (uint32_t)(kk >> 5) * rows * 128u + (uint32_t)(kk & 3) * 4u + (uint32_t)(n0 >> 3) * 1024u;
  const int ch = (kk & 31) >> 2;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const uint32_t off = cb + (uint32_t)j * 128u + ((uint32_t)(ch ^ j) << 4);
    float vh, vl;
    split(x[j], vh, vl);
    *reinterpret_cast<float*>(hi + off) = vh;
    *reinterpret_cast<float*>(lo + off) = vl;
  }
}

// Column c, rows r0 .. r0+7 (r0 a multiple of 8) of an operand as values.
static __device__ __forceinline__ void get_col8(const unsigned char* hi, const unsigned char* lo, int c, int r0,
                                         uint32_t rows, float (&x)[8]) {
  const uint32_t cb = (uint32_t)(c >> 5) * rows * 128u + (uint32_t)(c & 3) * 4u + (uint32_t)(r0 >> 3) * 1024u;
  const int ch = (c & 31) >> 2;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const uint32_t off = cb + (uint32_t)j * 128u + ((uint32_t)(ch ^ j) << 4);
    x[j] = *reinterpret_cast<const float*>(hi + off) + *reinterpret_cast<const float*>(lo + off);
  }
}

// D (TMEM) += A B over nslab slabs of 32 K-columns, 3 passes per K-step of 8.
// A: 128 rows from a_hi/a_lo (slab stride a_slab); B: N rows from b_hi/b_lo.
// Called by all of warp 0 with the same arguments (lane 0 issues); out of
// line: one copy of the issue loop for every product of the kernel.
static __device__ __noinline__ void issue3(uint32_t dtm, uint32_t a_hi, uint32_t a_lo, uint32_t a_slab, uint32_t b_hi,
                                       uint32_t b_lo, uint32_t b_slab, int nslab, uint32_t idesc, bool accumulate) {
  // Descriptors of the first K-step; later steps add (byte offset >> 4) to
  // the 14-bit start-address field (shared addresses stay below 256 KB).
  const uint64_t ah = smem_desc_sw128(a_hi), al = smem_desc_sw128(a_lo);
  const uint64_t bh = smem_desc_sw128(b_hi), bl = smem_desc_sw128(b_lo);
  for (int s = 0; s < nslab; ++s) {
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const uint64_t ao = (uint64_t)((s * a_slab + kk * 32) >> 4), bo = (uint64_t)((s * b_slab + kk * 32) >> 4);
      mma_tf32_elect(dtm, ah + ao, bh + bo, idesc, (accumulate || s > 0 || kk > 0) ? 1u : 0u);
      mma_tf32_elect(dtm, ah + ao, bl + bo, idesc, 1u);
      mma_tf32_elect(dtm, al + ao, bh + bo, idesc, 1u);
    }
  }
}

// Operands written by the generic proxy become visible to the tensor core,
// earlier TMEM reads are ordered before what follows the barrier.
static __device__ __forceinline__ void operands_ready() {
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
}

// Every thread waits (bounded) for the phase; one CTA-wide decision.
static __device__ __forceinline__ bool wait_all(uint64_t* bar, uint32_t parity) {
  const bool ok = mbar_wait(bar, parity);
  const int bad = __syncthreads_or(ok ? 0 : 1);
  tc_fence_after();
  return bad == 0;
}

}  // namespace t5
}  // namespace mg

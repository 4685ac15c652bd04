// The mixed-precision ensemble update Xa = m + X' T, fused with the member
// mean, on FP64 members in place (member-major, leading dimension ld).
//
// For each tile of kUpdS states: load the k members of the tile (all loads
// of a batch issued before any is used; the first batch of the next tile is
// loaded while the current product runs), split each FP64 value into an FP32
// pair (split_double), take the FP32 mean m, form X' = (hi - m) + lo in
// shared memory, compute X'T by a register-tiled FP32 product (thread: R
// consecutive members x 4 states; T staged once per call, zero-padded to
// KMAX columns), and write m + X'T back in place as FP64 through a TwoSum
// pair (pair_to_double).  No FP64 instruction touches an element.
//
// With STATS the routine also returns, per thread, the sums of X'^2 (the
// background spread) and of (Xa_i - mean_i Xa)^2 (the analysis spread), and
// mean_out receives the analysis mean; without it mean_out receives the
// background mean m.
#pragma once

#include <cstdint>

#include "mg_ffloat.cuh"

namespace mg {

constexpr int kUpdThreads = 256;
constexpr int kUpdS = 64;  // states per tile

__host__ __device__ constexpr int upd_kmax(int k) { return k <= 32 ? 32 : (k <= 64 ? 64 : 128); }
__host__ __device__ constexpr size_t upd_ts_floats(int maxk) { return (size_t)maxk * upd_kmax(maxk); }
// Dynamic shared memory of a CTA running cases with k <= maxk.
__host__ __device__ constexpr size_t upd_bytes(int maxk) {
  return sizeof(float) * (upd_ts_floats(maxk) + (size_t)maxk * kUpdS + 5 * kUpdS);
}

template <int R>
__device__ __forceinline__ void upd_load_row(const float* p, float (&v)[R]) {
  if constexpr (R % 4 == 0) {
#pragma unroll
    for (int a = 0; a < R; a += 4) {
      const float4 t = *reinterpret_cast<const float4*>(p + a);
      v[a] = t.x;
      v[a + 1] = t.y;
      v[a + 2] = t.z;
      v[a + 3] = t.w;
    }
  } else {
#pragma unroll
    for (int a = 0; a < R; a += 2) {
      const float2 t = *reinterpret_cast<const float2*>(p + a);
      v[a] = t.x;
      v[a + 1] = t.y;
    }
  }
}

// States [a, b) of members X (k <= KMAX <= 128); T32 is k x k row-major
// (T[j][i]: member j's weight in analysis member i).  smem: upd_bytes(maxk)
// for the largest k of the launch, carved as Ts (upd_ts_floats(maxk)), Xs
// (maxk x kUpdS), then 5 kUpdS floats.  Every thread of the CTA
// (kUpdThreads) calls it.
template <int KMAX, bool STATS>
__device__ __forceinline__ void update_mixed_range(double* X, int64_t ld, int k, int64_t a, int64_t b,
                                                   const float* __restrict__ T32, double* mean_out, float* smem,
                                                   int maxk, float& bg_sq, float& an_sq) {
  constexpr int R = KMAX / 16, JQ = KMAX / 4;
  float* Ts = smem;
  float* Xs = Ts + upd_ts_floats(maxk);
  float* part = Xs + (size_t)maxk * kUpdS;
  float* ms = part + 4 * kUpdS;
  const int tid = threadIdx.x;
  for (int e = tid; e < k * KMAX; e += kUpdThreads) {
    const int j = e / KMAX, i = e % KMAX;
    Ts[e] = i < k ? T32[j * k + i] : 0.0f;
  }
  const float inv_k = 1.0f / (float)k;
  const int s = tid % kUpdS, q = tid / kUpdS;        // mean phase: state, member quarter
  const int ti = tid / 16, ts = tid % 16, i0 = ti * R;  // product: members i0.., states 4 ts..
  constexpr int LB = JQ < 16 ? JQ : 16;
  auto load_batch = [&](double(&dst)[LB], int64_t t0, int u0) {
    const bool in = t0 + s < b;
#pragma unroll
    for (int v = 0; v < LB; ++v) {
      const int j = q + 4 * (u0 + v);
      dst[v] = (j < k && in) ? __ldcs(X + (int64_t)j * ld + t0 + s) : 0.0;
    }
  };
  double pre[LB];
  load_batch(pre, a, 0);
  for (int64_t s0 = a; s0 < b; s0 += kUpdS) {
    const int cnt = (int)(b - s0 < kUpdS ? b - s0 : kUpdS);
    float lo[JQ];
    float sum = 0.0f;
#pragma unroll
    for (int u0 = 0; u0 < JQ; u0 += LB) {
      double raw[LB];
      if (u0 == 0) {
#pragma unroll
        for (int v = 0; v < LB; ++v) raw[v] = pre[v];
      } else {
        load_batch(raw, s0, u0);
      }
#pragma unroll
      for (int v = 0; v < LB; ++v) {
        const int j = q + 4 * (u0 + v);
        float h, l;
        split_double(raw[v], h, l);
        lo[u0 + v] = l;
        if (j < k) Xs[j * kUpdS + s] = h;
        sum += h + l;
      }
    }
    part[q * kUpdS + s] = sum;
    __syncthreads();
    const float mf = (((part[s] + part[kUpdS + s]) + part[2 * kUpdS + s]) + part[3 * kUpdS + s]) * inv_k;
    if (q == 0) ms[s] = mf;
#pragma unroll
    for (int u = 0; u < JQ; ++u) {
      const int j = q + 4 * u;
      if (j < k) {
        const float pv = __fadd_rn(__fsub_rn(Xs[j * kUpdS + s], mf), lo[u]);
        Xs[j * kUpdS + s] = pv;
        if (STATS) bg_sq = fmaf(pv, pv, bg_sq);
      }
    }
    __syncthreads();
    if (s0 + kUpdS < b) load_batch(pre, s0 + kUpdS, 0);
    float acc[R][4];
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r][0] = acc[r][1] = acc[r][2] = acc[r][3] = 0.0f;
    if (i0 < k) {
#pragma unroll 4
      for (int j = 0; j < k; ++j) {
        const float4 xv = *reinterpret_cast<const float4*>(Xs + j * kUpdS + 4 * ts);
        float tv[R];
        upd_load_row<R>(Ts + j * KMAX + i0, tv);
#pragma unroll
        for (int r = 0; r < R; ++r) {
          acc[r][0] = fmaf(tv[r], xv.x, acc[r][0]);
          acc[r][1] = fmaf(tv[r], xv.y, acc[r][1]);
          acc[r][2] = fmaf(tv[r], xv.z, acc[r][2]);
          acc[r][3] = fmaf(tv[r], xv.w, acc[r][3]);
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (i0 + r < k)
        *reinterpret_cast<float4*>(Xs + (i0 + r) * kUpdS + 4 * ts) = make_float4(acc[r][0], acc[r][1], acc[r][2],
                                                                                 acc[r][3]);
    __syncthreads();
    if (STATS) {  // member mean of X'T per state (part is free again)
      if (tid < kUpdS) {
        float am = 0.0f;
        for (int i = 0; i < k; ++i) am += Xs[i * kUpdS + tid];
        part[tid] = am * inv_k;
      }
      __syncthreads();
    }
    for (int e = tid; e < k * kUpdS; e += kUpdThreads) {
      const int i = e / kUpdS, ss = e % kUpdS;
      if (ss < cnt) {
        float y, ye;
        const float v = Xs[e];
        two_sum(ms[ss], v, y, ye);
        X[(int64_t)i * ld + s0 + ss] = pair_to_double(y, ye);
        if (STATS) {
          const float dv = v - part[ss];
          an_sq = fmaf(dv, dv, an_sq);
        }
      }
    }
    if (mean_out && tid < cnt) {
      if (STATS) {
        float y, ye;
        two_sum(ms[tid], part[tid], y, ye);
        mean_out[s0 + tid] = pair_to_double(y, ye);
      } else {
        mean_out[s0 + tid] = pair_to_double(ms[tid], 0.0f);
      }
    }
    __syncthreads();
  }
}

// Dispatch on the member-count class (one branch per CTA).
template <bool STATS>
__device__ __forceinline__ void update_mixed(double* X, int64_t ld, int k, int64_t a, int64_t b, const float* T32,
                                             double* mean_out, float* smem, int maxk, float& bg_sq, float& an_sq) {
  const int km = upd_kmax(k);
  if (km == 32)
    update_mixed_range<32, STATS>(X, ld, k, a, b, T32, mean_out, smem, maxk, bg_sq, an_sq);
  else if (km == 64)
    update_mixed_range<64, STATS>(X, ld, k, a, b, T32, mean_out, smem, maxk, bg_sq, an_sq);
  else
    update_mixed_range<128, STATS>(X, ld, k, a, b, T32, mean_out, smem, maxk, bg_sq, an_sq);
}

}  // namespace mg

// Ensemble diagnostics: Metrics<double>::CalculateAll (Metrics.hpp:74-94).
//
// Per state element: mean (member-order sum, then a division by k, as
// CalculateEnsembleMean :108-121), spread sqrt(sum (x - mean)^2 / (k - 1))
// (:137-150) and the element's CRPS term
//     sum_j |x_j - t| / k - sum_j sum_l |x_j - x_l| / (2 k^2)   (:232-252).
// The mean and spread use explicit round-to-nearest operations (no FMA
// contraction), so they equal the reference's element for element.  The
// state-wide sums (RMSE :265-273, bias :166-173, correlation by the
// single-pass sums formula :189-206, CRPS, average spread :286-293) are
// taken per CTA, then over the CTAs in a fixed order by one CTA:
// deterministic, and equal to the reference's sequential sums to rounding.
//
// A CTA stages a tile of 32 state elements x k members in shared memory,
// with an order-preserving integer key per value; each element has a group
// of 8 threads.  GB300 runs FP64 at about 2 operations per clock per SM, so
// the CRPS pair term is not the k^2 sum of |x_j - x_l| but its sorted form
//     sum_j sum_l |x_j - x_l| = 2 sum_j (2 r_j - k + 1) x_j,
// r_j the rank of x_j (ties broken by member index), with the ranks counted
// by 32-bit integer comparisons of the keys' top halves (exact recount on
// the full keys where two members share them): k FP64 FMAs per element
// instead of 2 k^2 FP64 operations.  Member order of the mean and spread is
// kept; they are computed by one full warp, a lane per element.
#include "mg_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kTile = 32;     // state elements per tile
constexpr int kGroup = kThreads / kTile;  // threads per element
constexpr int kSums = 9;
// sums: m - t, (m - t)^2, m, t, m t, m^2, t^2, crps_i, spread_i
constexpr int kMaxBlocks = 152 * 8;
constexpr int kOwn = 8;  // members ranked at once by one thread

// Signed 64-bit keys that order like the doubles (NaN aside; -0 < +0 only
// separates values whose difference is zero).
__device__ __forceinline__ long long order_key(double x) {
  const long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}

__global__ void __launch_bounds__(kThreads) metrics_elem_kernel(const double* __restrict__ X, int64_t n, int k,
                                                                int64_t ld, const double* __restrict__ truth,
                                                                double* __restrict__ mean_out,
                                                                double* __restrict__ spread_out,
                                                                double* __restrict__ partial) {
  extern __shared__ double xs[];  // k x kTile values, then k x kTile top-32-bit keys
  int* ks = reinterpret_cast<int*>(xs + (size_t)k * kTile);
  __shared__ double coef[256];     // 2 r - k + 1 for rank r
  __shared__ double sd_sh[kTile], st_sh[kTile];
  __shared__ double red[kSums][kThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int e = tid / kGroup, g = tid % kGroup;  // element of the tile, thread within its group
  for (int r = tid; r < k; r += kThreads) coef[r] = (double)(2 * r - k + 1);
  const double inv_k = 1.0 / (double)k, inv_k2 = inv_k * inv_k;
  double acc[kSums];
#pragma unroll
  for (int s = 0; s < kSums; ++s) acc[s] = 0.0;
  for (int64_t t0 = (int64_t)blockIdx.x * kTile; t0 < n; t0 += (int64_t)gridDim.x * kTile) {
    const int cnt = (int)(n - t0 < kTile ? n - t0 : kTile);
    for (int q = tid; q < k * kTile; q += kThreads) {
      const int j = q / kTile, c = q - j * kTile;
      const double v = (c < cnt) ? X[(int64_t)j * ld + t0 + c] : 0.0;
      xs[q] = v;
      ks[q] = (int)(order_key(v) >> 32);
    }
    __syncthreads();
    const bool valid = e < cnt;
    const int64_t i = t0 + e;
    double tr = 0.0, sd = 0.0, st = 0.0;
    if (valid) {
      tr = truth[i];
      // ranks of members j = g + kGroup u, kOwn at a time, counted on the top
      // 32 bits of the keys (ordered like the keys); a member that shares
      // them with another member is recounted on the full keys with ties
      // broken by member index.  Then the sorted-form sum.
      for (int u0 = 0; g + kGroup * u0 < k; u0 += kOwn) {
        int hk[kOwn], lt[kOwn], eq[kOwn];
#pragma unroll
        for (int u = 0; u < kOwn; ++u) {
          const int j = g + kGroup * (u0 + u);
          hk[u] = j < k ? ks[j * kTile + e] : 0x7fffffff;
          lt[u] = 0;
          eq[u] = 0;
        }
        for (int l = 0; l < k; ++l) {
          const int hl = ks[l * kTile + e];
#pragma unroll
          for (int u = 0; u < kOwn; ++u) {
            lt[u] += hl < hk[u] ? 1 : 0;
            eq[u] += hl == hk[u] ? 1 : 0;
          }
        }
#pragma unroll
        for (int u = 0; u < kOwn; ++u) {
          const int j = g + kGroup * (u0 + u);
          if (j < k) {
            const double xj = xs[j * kTile + e];
            int r = lt[u];
            if (eq[u] > 1) {  // another member with the same top 32 bits: exact count
              const long long kj = order_key(xj);
              r = 0;
              for (int l = 0; l < k; ++l) {
                const long long kl = order_key(xs[l * kTile + e]);
                r += (kl < kj || (kl == kj && l < j)) ? 1 : 0;
              }
            }
            sd = fma(coef[r], xj, sd);
            st += fabs(xj - tr);
          }
        }
      }
    }
#pragma unroll
    for (int off = kGroup / 2; off > 0; off >>= 1) {  // every lane, outside any branch
      sd += __shfl_down_sync(0xffffffffu, sd, off, kGroup);
      st += __shfl_down_sync(0xffffffffu, st, off, kGroup);
    }
    if (g == 0) {
      sd_sh[e] = sd;
      st_sh[e] = st;
    }
    __syncthreads();
    // Mean, spread and the sums: one full warp, a lane per element (an FP64
    // instruction costs the FP64 pipe the same with one active lane or 32).
    if (warp == 0 && lane < cnt) {
      const int64_t il = t0 + lane;
      const double trl = truth[il];
      double m = 0.0;
      for (int j = 0; j < k; ++j) m = __dadd_rn(m, xs[j * kTile + lane]);
      m = __ddiv_rn(m, (double)k);
      double sp = 0.0;
      for (int j = 0; j < k; ++j) {
        const double d = __dsub_rn(xs[j * kTile + lane], m);
        sp = __dadd_rn(sp, __dmul_rn(d, d));
      }
      sp = __dsqrt_rn(__ddiv_rn(sp, (double)(k - 1)));
      if (mean_out) mean_out[il] = m;
      if (spread_out) spread_out[il] = sp;
      const double dm = m - trl;
      acc[0] += dm;
      acc[1] += dm * dm;
      acc[2] += m;
      acc[3] += trl;
      acc[4] += m * trl;
      acc[5] += m * m;
      acc[6] += trl * trl;
      acc[7] += st_sh[lane] * inv_k - sd_sh[lane] * inv_k2;  // sum_j sum_l |x_j - x_l| = 2 sd
      acc[8] += sp;
    }
    __syncthreads();
  }
#pragma unroll
  for (int s = 0; s < kSums; ++s) {
    double v = acc[s];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) red[s][warp] = v;
  }
  __syncthreads();
  if (tid < kSums) {
    double v = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) v += red[tid][w];
    partial[(int64_t)blockIdx.x * kSums + tid] = v;
  }
}

// One CTA: the CTA partials in block order, then the five statistics.
__global__ void metrics_final_kernel(const double* __restrict__ partial, int nblocks, int64_t n,
                                     double* __restrict__ out5) {
  if (threadIdx.x != 0) return;
  double S[kSums];
  for (int s = 0; s < kSums; ++s) S[s] = 0.0;
  for (int b = 0; b < nblocks; ++b)
    for (int s = 0; s < kSums; ++s) S[s] += partial[(int64_t)b * kSums + s];
  const double nn = (double)n;
  out5[0] = sqrt(S[1] / nn);                                                            // RMSE
  out5[1] = S[0] / nn;                                                                  // bias
  out5[2] = (nn * S[4] - S[2] * S[3]) / sqrt((nn * S[5] - S[2] * S[2]) * (nn * S[6] - S[3] * S[3]));
  out5[3] = S[7] / nn;                                                                  // CRPS
  out5[4] = S[8] / nn;                                                                  // average spread
}

}  // namespace

extern "C" int mg_ens_metrics(mg_context* ctx, const double* X, int64_t n, int32_t k, int64_t ld,
                              const double* truth, double* mean_out, double* spread_out, mg_ens_metrics_t* out) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(X && truth && out && n > 0 && k >= 2 && k <= 256 && ld >= n, "mg_ens_metrics: bad arguments");
  const int64_t tiles = (n + kTile - 1) / kTile;
  const int nblocks = (int)(tiles < kMaxBlocks ? tiles : kMaxBlocks);
  const size_t smem = (sizeof(double) + sizeof(int)) * (size_t)k * kTile;
  void* ws = mg::workspace(ctx, sizeof(double) * ((size_t)nblocks * kSums + 8));
  if (!ws) return MG_ERR_NOMEM;
  double* partial = static_cast<double*>(ws);
  double* dout = partial + (size_t)nblocks * kSums;
  MG_TRY_CUDA(cudaFuncSetAttribute(metrics_elem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  metrics_elem_kernel<<<nblocks, kThreads, smem, ctx->stream>>>(X, n, k, ld, truth, mean_out, spread_out, partial);
  MG_COUNT_LAUNCH();
  metrics_final_kernel<<<1, 32, 0, ctx->stream>>>(partial, nblocks, n, dout);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  double h[5];
  MG_TRY_CUDA(cudaMemcpyAsync(h, dout, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  MG_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
  out->rmse = h[0];
  out->bias = h[1];
  out->correlation = h[2];
  out->crps = h[3];
  out->avg_spread = h[4];
  return MG_OK;
}

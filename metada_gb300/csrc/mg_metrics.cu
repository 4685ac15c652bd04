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
// A CTA walks tiles of 32 state elements x k members, staged in shared
// memory with an order-preserving integer key per value.  GB300 runs FP64 at
// about 2 operations per clock per SM, so the CRPS pair term is not the k^2
// sum of |x_j - x_l| but its sorted form
//     sum_j sum_l |x_j - x_l| = 2 sum_j (2 r_j - k + 1) x_j,
// r_j the rank of x_j (ties broken by member index), with the ranks counted
// by 32-bit integer comparisons of the keys' top halves (exact recount on
// the full keys where two members share them): k FP64 FMAs per element
// instead of 2 k^2 FP64 operations.  The member-order mean and spread (one
// dependent FP64 chain per element) run on warp 0, a lane per element, for
// tile t - 1 while warps 1-7 (seven threads per element) rank tile t and
// load tile t + 1: tiles are triple-buffered and the rank partials double-
// buffered, so the chain no longer stalls the other warps at a barrier.
#include "mg_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kRankThreads = kThreads - 32;  // warps 1-7
constexpr int kSums = 9;
// sums: m - t, (m - t)^2, m, t, m t, m^2, t^2, crps_i, spread_i
constexpr int kMaxBlocks = 152 * 8;
constexpr int kOwn = 10;  // members ranked at once by one thread

// Signed 64-bit keys that order like the doubles (NaN aside; -0 < +0 only
// separates values whose difference is zero).
__device__ __forceinline__ long long order_key(double x) {
  const long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}

// kTile elements per tile (32: a full warp-0 lane set; 16 for k > 160, where
// three buffers of 32 would not fit in shared memory), kGroup rank threads
// per element (kTile x kGroup = 224).
template <int kTile>
__global__ void __launch_bounds__(kThreads) metrics_elem_kernel(const double* __restrict__ X, int64_t n, int k,
                                                                int64_t ld, const double* __restrict__ truth,
                                                                double* __restrict__ mean_out,
                                                                double* __restrict__ spread_out,
                                                                double* __restrict__ partial) {
  constexpr int kGroup = kRankThreads / kTile;
  static_assert(kTile * kGroup == kRankThreads, "tile x group");
  extern __shared__ double smem_d[];  // 3 x (k x kTile values), then 3 x (k x kTile top-32-bit keys)
  const size_t tile_vals = (size_t)k * kTile;
  double* xs_all = smem_d;
  int* ks_all = reinterpret_cast<int*>(smem_d + 3 * tile_vals);
  __shared__ double coef[256];  // 2 r - k + 1 for rank r
  __shared__ double part_sd[2][kTile * kGroup], part_st[2][kTile * kGroup];
  __shared__ double tr_sh[3][kTile];
  __shared__ double red[kSums][kThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int r = tid; r < k; r += kThreads) coef[r] = (double)(2 * r - k + 1);
  const double inv_k = 1.0 / (double)k, inv_k2 = inv_k * inv_k;
  double acc[kSums];
#pragma unroll
  for (int q = 0; q < kSums; ++q) acc[q] = 0.0;
  // This CTA's tiles: t = 0, 1, ... at elements (blockIdx.x + t gridDim.x) kTile.
  const int64_t stride = (int64_t)gridDim.x * kTile;
  const int64_t first = (int64_t)blockIdx.x * kTile;
  const int ntile = first < n ? (int)((n - first + stride - 1) / stride) : 0;
  auto tile_start = [&](int t) { return first + (int64_t)t * stride; };
  auto tile_cnt = [&](int t) {
    const int64_t t0 = tile_start(t);
    return (int)(n - t0 < kTile ? n - t0 : kTile);
  };
  // Loads tile t into buffer t % 3 (threads [lo, lo + nthr)).
  auto load_tile = [&](int t, int lo, int nthr) {
    const int b = t % 3;
    const int64_t t0 = tile_start(t);
    const int cnt = tile_cnt(t);
    double* xs = xs_all + b * tile_vals;
    int* ks = ks_all + b * tile_vals;
    for (int q = tid - lo; q < k * kTile; q += nthr) {
      const int j = q / kTile, c = q - j * kTile;
      const double v = (c < cnt) ? X[(int64_t)j * ld + t0 + c] : 0.0;
      xs[q] = v;
      ks[q] = (int)(order_key(v) >> 32);
    }
    for (int c = tid - lo; c < kTile; c += nthr) tr_sh[b][c] = c < cnt ? truth[t0 + c] : 0.0;
  };
  if (ntile > 0) load_tile(0, 0, kThreads);
  __syncthreads();
  for (int t = 0; t <= ntile; ++t) {
    if (warp > 0) {
      if (t + 1 < ntile) load_tile(t + 1, 32, kThreads - 32);
      if (t < ntile) {  // ranks and the CRPS partials of tile t
        const int b = t % 3, cnt = tile_cnt(t);
        const double* xs = xs_all + b * tile_vals;
        const int* ks = ks_all + b * tile_vals;
        const int r7 = tid - 32, e = r7 / kGroup, g = r7 - e * kGroup;
        double sd = 0.0, st = 0.0;
        if (e < cnt) {
          const double tr = tr_sh[b][e];
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
        part_sd[t & 1][r7] = sd;
        part_st[t & 1][r7] = st;
      }
    } else if (t >= 1) {
      // Warp 0: mean, spread and the sums of tile t - 1, a lane per element
      // (every FP64 warp instruction carries 32 lanes of work).
      const int tp = t - 1, b = tp % 3, cnt = tile_cnt(tp);
      const double* xs = xs_all + b * tile_vals;
      if (lane < cnt) {
        const int64_t il = tile_start(tp) + lane;
        const double trl = tr_sh[b][lane];
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
        double sd = 0.0, st = 0.0;
        for (int g = 0; g < kGroup; ++g) {
          sd += part_sd[tp & 1][lane * kGroup + g];
          st += part_st[tp & 1][lane * kGroup + g];
        }
        const double dm = m - trl;
        acc[0] += dm;
        acc[1] += dm * dm;
        acc[2] += m;
        acc[3] += trl;
        acc[4] += m * trl;
        acc[5] += m * m;
        acc[6] += trl * trl;
        acc[7] += st * inv_k - sd * inv_k2;  // sum_j sum_l |x_j - x_l| = 2 sd
        acc[8] += sp;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < kSums; ++q) {
    double v = acc[q];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) red[q][warp] = v;
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
  const int tile = k <= 160 ? 32 : 16;
  const int64_t tiles = (n + tile - 1) / tile;
  const int nblocks = (int)(tiles < kMaxBlocks ? tiles : kMaxBlocks);
  const size_t smem = 3 * (sizeof(double) + sizeof(int)) * (size_t)k * tile;
  void* ws = mg::workspace(ctx, sizeof(double) * ((size_t)nblocks * kSums + 8));
  if (!ws) return MG_ERR_NOMEM;
  double* partial = static_cast<double*>(ws);
  double* dout = partial + (size_t)nblocks * kSums;
  if (tile == 32) {
    MG_TRY_CUDA(cudaFuncSetAttribute(metrics_elem_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    metrics_elem_kernel<32><<<nblocks, kThreads, smem, ctx->stream>>>(X, n, k, ld, truth, mean_out, spread_out,
                                                                      partial);
  } else {
    MG_TRY_CUDA(cudaFuncSetAttribute(metrics_elem_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    metrics_elem_kernel<16><<<nblocks, kThreads, smem, ctx->stream>>>(X, n, k, ld, truth, mean_out, spread_out,
                                                                      partial);
  }
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

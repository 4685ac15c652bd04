// Stochastic EnKF with perturbed observations (EnKF.hpp:139-254) in the
// k-dimensional form.
//
// The reference forms the p x p matrix S = Y'Y'^T/(k-1) + R, inverts it and
// builds the n x p gain K = X'Y'^T S^-1/(k-1).  By the push-through identity
// Y'^T (Y'Y'^T + (k-1) R)^-1 = (Y'^T R^-1 Y' + (k-1) I)^-1 Y'^T R^-1, so with
// A = Y'^T R^-1 Y' + (k-1) I (k x k) the update of member i,
//     xa_i = xm + X'_i + K (yo + eps_i - Yb_i),
// becomes Xa = xm 1^T + X' T with T = I + A^-1 Y'^T R^-1 D and
// D = d 1^T + eps - Y' (yo - Yb_i = d - Y'_i).  Y'^T R^-1 D = b 1^T + F - G
// with G = Y'^T R^-1 Y', F = Y'^T R^-1 eps and b = Y'^T R^-1 d: two Gram
// passes over the obs and one k x k Cholesky solve, no p x p matrix.  X' is
// the inflated perturbation sqrt(rho)(x_i - xm) (applyInflation :322-335),
// Y' comes from the raw members (:168-174).  The analysis mean is recomputed
// at the end (:237).  Diagnostics: ||d|| (:184), background and analysis
// spread (:334, :240-253); the gain's max/min and S's condition number need
// the n x p gain or the p x p S and are not formed.
#include <algorithm>
#include <cmath>

#include "mg_dense.cuh"
#include "mg_internal.h"
#include "mg_update.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kRedBlocks = 304;

// C = sum_o rinv_o U[o]^T W[o] over this CTA's obs range (U, W: p x k
// row-major); with bout, also b = sum_o rinv_o d_o U[o].  TE is the
// arithmetic type (FP64, or FP32 on the mixed path).
template <typename TE, int KMAX>
__global__ void __launch_bounds__(kThreads) enkf_cross_kernel(const TE* __restrict__ U, const TE* __restrict__ W,
                                                              const TE* __restrict__ rinv,
                                                              const TE* __restrict__ dinn, int64_t p, int k,
                                                              int64_t per_block, TE* __restrict__ Cpart,
                                                              TE* __restrict__ bpart) {
  constexpr int CH = (KMAX >= 128 && sizeof(TE) == 8) ? 16 : 32, R = KMAX / 16;
  __shared__ TE Us[CH * KMAX], Ws[CH * KMAX];
  __shared__ TE sr[CH], sd[CH];
  const int tid = threadIdx.x, ti = tid / 16, tj = tid % 16;
  const int64_t o0 = (int64_t)blockIdx.x * per_block;
  const int64_t o1 = min(p, o0 + per_block);
  TE acc[R][R];
#pragma unroll
  for (int a = 0; a < R; ++a)
#pragma unroll
    for (int b = 0; b < R; ++b) acc[a][b] = TE(0);
  TE bacc = TE(0);
  for (int64_t c0 = o0; c0 < o1; c0 += CH) {
    const int cnt = (int)(o1 - c0 < (int64_t)CH ? o1 - c0 : (int64_t)CH);
    for (int e = tid; e < cnt * KMAX; e += kThreads) {
      const int r = e / KMAX, j = e - r * KMAX;
      Us[e] = (j < k) ? U[(c0 + r) * k + j] : TE(0);
      Ws[e] = (j < k) ? W[(c0 + r) * k + j] : TE(0);
    }
    if (tid < cnt) {
      sr[tid] = rinv[c0 + tid];
      sd[tid] = dinn[c0 + tid];
    }
    __syncthreads();
    for (int r = 0; r < cnt; ++r) {
      const TE w = sr[r];
      TE av[R], bv[R];
#pragma unroll
      for (int a = 0; a < R; ++a) av[a] = Us[r * KMAX + ti + 16 * a] * w;
#pragma unroll
      for (int b = 0; b < R; ++b) bv[b] = Ws[r * KMAX + tj + 16 * b];
#pragma unroll
      for (int a = 0; a < R; ++a)
#pragma unroll
        for (int b = 0; b < R; ++b) acc[a][b] += av[a] * bv[b];
    }
    if (bpart && tid < k)
      for (int r = 0; r < cnt; ++r) bacc += (Us[r * KMAX + tid] * sr[r]) * sd[r];
    __syncthreads();
  }
  TE* C = Cpart + (size_t)blockIdx.x * k * k;
#pragma unroll
  for (int a = 0; a < R; ++a)
#pragma unroll
    for (int b = 0; b < R; ++b) {
      const int i = ti + 16 * a, j = tj + 16 * b;
      if (i < k && j < k) C[i * k + j] = acc[a][b];
    }
  if (bpart && tid < k) bpart[(size_t)blockIdx.x * k + tid] = bacc;
}

// out[e] = sum over the nblk partials of element e (len elements each), in
// block order: one thread per element, so the sums of the k x k partials
// run on many SMs instead of inside the one-CTA solve.
template <typename TE>
__global__ void __launch_bounds__(kThreads) reduce_partials_kernel(const TE* __restrict__ part, int nblk, int64_t len,
                                                                   double* __restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (e >= len) return;
  double t = 0.0;
  for (int b = 0; b < nblk; ++b) t += (double)part[(size_t)b * len + e];
  out[e] = t;
}

// T = sqrt(rho) (I + A^-1 (b 1^T + F - G)), A = G + (k-1) I, by Cholesky
// A = L L^T and two triangular solves on the k right-hand sides.
__global__ void __launch_bounds__(kThreads) enkf_solve_kernel(const double* __restrict__ Gpart,
                                                              const double* __restrict__ Fpart,
                                                              const double* __restrict__ bpart, int nblk, int k,
                                                              double rho, double* __restrict__ T,
                                                              float* __restrict__ T32, int* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lda = k + 1;
  double* A = reinterpret_cast<double*>(smem_raw);  // k x lda
  double* B = A + (size_t)k * lda;                 // k x lda
  __shared__ int flag;
  const int tid = threadIdx.x;
  for (int e = tid; e < k * k; e += kThreads) {
    const int i = e / k, j = e - i * k;
    double g = 0.0, f = 0.0;
    for (int b = 0; b < nblk; ++b) {
      g += Gpart[(size_t)b * k * k + e];
      f += Fpart[(size_t)b * k * k + e];
    }
    double bi = 0.0;
    for (int b = 0; b < nblk; ++b) bi += bpart[(size_t)b * k + i];
    A[i * lda + j] = g + (i == j ? (double)(k - 1) : 0.0);
    B[i * lda + j] = (bi + f) - g;
  }
  __syncthreads();
  const bool ok = mg::cta_cholesky<double>(A, k, lda, &flag);
  for (int i = 0; i < k; ++i) {  // B <- L^-1 B, all columns at once
    for (int c = tid; c < k; c += kThreads) {
      double s = B[i * lda + c];
      for (int m = 0; m < i; ++m) s -= A[i * lda + m] * B[m * lda + c];
      B[i * lda + c] = s / A[i * lda + i];
    }
    __syncthreads();
  }
  for (int i = k - 1; i >= 0; --i) {  // B <- L^-T B
    for (int c = tid; c < k; c += kThreads) {
      double s = B[i * lda + c];
      for (int m = i + 1; m < k; ++m) s -= A[m * lda + i] * B[m * lda + c];
      B[i * lda + c] = s / A[i * lda + i];
    }
    __syncthreads();
  }
  const double sr = sqrt(rho);
  for (int e = tid; e < k * k; e += kThreads) {
    const int i = e / k, j = e - i * k;
    const double t = sr * ((i == j ? 1.0 : 0.0) + B[i * lda + j]);
    T[i * k + j] = t;
    if (T32) T32[i * k + j] = (float)t;
  }
  if (tid == 0 && !ok) *status = 1;
}

// Xa_i[s] = xm[s] + sum_j X'_j[s] T_ji for a tile of 32 state indices.
template <typename TE>
__global__ void __launch_bounds__(kThreads) enkf_update_kernel(const TE* __restrict__ Xp, int64_t ldp,
                                                               const double* __restrict__ mean,
                                                               const double* __restrict__ T, int64_t n, int k,
                                                               double* __restrict__ X, int64_t ld) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TE* Ts = reinterpret_cast<TE*>(smem_raw);  // k x k
  TE* Xt = Ts + k * k;                       // 32 x (k + 1)
  const int64_t s0 = (int64_t)blockIdx.x * 32;
  for (int e = threadIdx.x; e < k * k; e += kThreads) Ts[e] = (TE)T[e];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j = warp; j < k; j += kThreads / 32) {
    const int64_t s = s0 + lane;
    Xt[lane * (k + 1) + j] = (s < n) ? Xp[(int64_t)j * ldp + s] : TE(0);
  }
  __syncthreads();
  const int64_t s = s0 + lane;
  if (s < n) {
    const double m = mean[s];
    for (int i = warp; i < k; i += kThreads / 32) {
      TE acc = TE(0);
      for (int j = 0; j < k; ++j) acc += Xt[lane * (k + 1) + j] * Ts[j * k + i];
      X[(int64_t)i * ld + s] = m + (double)acc;
    }
  }
}

// Deterministic sum of squares: fixed grid, per-CTA partials, one CTA sums
// them in order into *out.
template <typename TE>
__global__ void __launch_bounds__(kThreads) sumsq_partial_kernel(const TE* __restrict__ v, int64_t n,
                                                                 double* __restrict__ partial) {
  __shared__ double red[kThreads / 32];
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
    const double x = (double)v[i];
    s += x * x;
  }
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) t += red[w];
    partial[blockIdx.x] = t;
  }
}

// *out = sum of nb partials by one CTA: thread t sums t, t + kThreads, ...
// in order, then a fixed-order tree (deterministic).
__global__ void __launch_bounds__(kThreads) sum_partials_kernel(const double* __restrict__ partial, int nb,
                                                                double* __restrict__ out) {
  __shared__ double red[kThreads];
  double t = 0.0;
  for (int b = threadIdx.x; b < nb; b += kThreads) t += partial[b];
  red[threadIdx.x] = t;
  __syncthreads();
  for (int h = kThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

template <typename TE>
int sumsq(mg_context* ctx, const TE* v, int64_t n, double* partial, double* out) {
  sumsq_partial_kernel<TE><<<kRedBlocks, kThreads, 0, ctx->stream>>>(v, n, partial);
  MG_COUNT_LAUNCH();
  sum_partials_kernel<<<1, kThreads, 0, ctx->stream>>>(partial, kRedBlocks, out);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

template <typename TE>
int launch_cross(mg_context* ctx, const TE* U, const TE* W, const TE* rinv, const TE* d, int64_t p, int k, int nblk,
                 int64_t per_block, TE* Cpart, TE* bpart) {
  if (k <= 32)
    enkf_cross_kernel<TE, 32><<<nblk, kThreads, 0, ctx->stream>>>(U, W, rinv, d, p, k, per_block, Cpart, bpart);
  else if (k <= 64)
    enkf_cross_kernel<TE, 64><<<nblk, kThreads, 0, ctx->stream>>>(U, W, rinv, d, p, k, per_block, Cpart, bpart);
  else
    enkf_cross_kernel<TE, 128><<<nblk, kThreads, 0, ctx->stream>>>(U, W, rinv, d, p, k, per_block, Cpart, bpart);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

template <typename TE>
int reduce_partials(mg_context* ctx, const TE* part, int nblk, int64_t len, double* out) {
  reduce_partials_kernel<TE><<<(unsigned)((len + kThreads - 1) / kThreads), kThreads, 0, ctx->stream>>>(part, nblk,
                                                                                                       len, out);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

int launch_solve(mg_context* ctx, const double* G, const double* F, const double* b, int k, double rho, double* T,
                 float* T32, int* status) {
  const size_t smem = sizeof(double) * 2 * (size_t)k * (k + 1);
  MG_TRY_CUDA(cudaFuncSetAttribute(enkf_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  enkf_solve_kernel<<<1, kThreads, smem, ctx->stream>>>(G, F, b, 1, k, rho, T, T32, status);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

int finish(mg_context* ctx, int64_t n, int k, double rho, const double* mean, double* mean_out, const int* status,
           const double* sums, mg_enkf_diag* diag) {
  cudaStream_t s = ctx->stream;
  if (mean_out) MG_TRY_CUDA(cudaMemcpyAsync(mean_out, mean, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  int hs = 0;
  double hsum[3] = {0.0, 0.0, 0.0};
  MG_TRY_CUDA(cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (diag) MG_TRY_CUDA(cudaMemcpyAsync(hsum, sums, sizeof(hsum), cudaMemcpyDeviceToHost, s));
  MG_TRY_CUDA(cudaStreamSynchronize(s));
  if (hs) return mg::fail(ctx, MG_ERR_NUMERIC, "mg_enkf: the k x k system was not positive definite");
  if (diag) {
    const double nk = (double)n * (double)k;
    diag->innovation_norm = std::sqrt(hsum[0]);
    diag->background_spread = std::sqrt(rho * hsum[1] / nk);
    diag->analysis_spread = std::sqrt(hsum[2] / nk);
  }
  return MG_OK;
}

// FP64 path: every stage in FP64, the analysis mean and spread recomputed
// from the analysed members in member order.
int run_enkf_fp64(mg_context* ctx, double* X, int64_t n, int k, int64_t ld, const double* HX, const double* yo,
                  const double* rvar, const double* eps, int64_t p, double rho, double* mean_out,
                  mg_enkf_diag* diag) {
  const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>((p + 255) / 256, 2 * ctx->num_sms));
  const int64_t per_block = (p + nblk - 1) / nblk;
  const int64_t kk = (int64_t)k * k;
  mg::Carver cv;
  cv.reserve<double>(n);
  cv.reserve<double>((size_t)n * k);
  cv.reserve<double>((size_t)(p + 1) * k);
  cv.reserve<double>(p + 1);
  cv.reserve<double>(p + 1);
  cv.reserve<double>((size_t)nblk * kk);
  cv.reserve<double>((size_t)nblk * kk);
  cv.reserve<double>((size_t)nblk * k);
  cv.reserve<double>(2 * kk + k);
  cv.reserve<double>(kk);
  cv.reserve<double>(kRedBlocks);
  cv.reserve<double>(4);
  cv.reserve<int>(4);
  void* ws = mg::workspace(ctx, cv.off);
  if (!ws) return MG_ERR_NOMEM;
  cv = mg::Carver{static_cast<char*>(ws), 0};
  double* mean = cv.take<double>(n);
  double* Xp = cv.take<double>((size_t)n * k);
  double* Y = cv.take<double>((size_t)(p + 1) * k);
  double* dinn = cv.take<double>(p + 1);
  double* rinv = cv.take<double>(p + 1);
  double* Gpart = cv.take<double>((size_t)nblk * kk);
  double* Fpart = cv.take<double>((size_t)nblk * kk);
  double* bpart = cv.take<double>((size_t)nblk * k);
  double* GFb = cv.take<double>(2 * kk + k);
  double* T = cv.take<double>(kk);
  double* red = cv.take<double>(kRedBlocks);
  double* sums = cv.take<double>(4);
  int* status = cv.take<int>(4);
  cudaStream_t s = ctx->stream;
  int rc;
  MG_TRY_CUDA(mg::launch_mean_pert_members(X, n, k, ld, mean, Xp, nullptr, n, s));
  MG_TRY_CUDA(mg::launch_obs_prior(HX, yo, rvar, p, k, Y, nullptr, dinn, rinv, s));
  if (diag) {
    if ((rc = sumsq<double>(ctx, dinn, p, red, sums + 0)) != MG_OK) return rc;
    if ((rc = sumsq<double>(ctx, Xp, (int64_t)n * k, red, sums + 1)) != MG_OK) return rc;
  }
  if ((rc = launch_cross<double>(ctx, Y, Y, rinv, dinn, p, k, nblk, per_block, Gpart, bpart)) != MG_OK ||
      (rc = launch_cross<double>(ctx, Y, eps, rinv, dinn, p, k, nblk, per_block, Fpart, nullptr)) != MG_OK ||
      (rc = reduce_partials<double>(ctx, Gpart, nblk, kk, GFb)) != MG_OK ||
      (rc = reduce_partials<double>(ctx, Fpart, nblk, kk, GFb + kk)) != MG_OK ||
      (rc = reduce_partials<double>(ctx, bpart, nblk, k, GFb + 2 * kk)) != MG_OK)
    return rc;
  MG_TRY_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * 4, s));
  if ((rc = launch_solve(ctx, GFb, GFb + kk, GFb + 2 * kk, k, rho, T, nullptr, status)) != MG_OK) return rc;
  const size_t usmem = sizeof(double) * ((size_t)k * k + 32 * (size_t)(k + 1));
  MG_TRY_CUDA(cudaFuncSetAttribute(enkf_update_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)usmem));
  enkf_update_kernel<double><<<(unsigned)((n + 31) / 32), kThreads, usmem, s>>>(Xp, n, mean, T, n, k, X, ld);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  // Analysis mean and perturbations (Ensemble::RecomputeMean/Perturbations).
  MG_TRY_CUDA(mg::launch_mean_pert_members(X, n, k, ld, mean, diag ? Xp : nullptr, nullptr, n, s));
  if (diag && (rc = sumsq<double>(ctx, Xp, (int64_t)n * k, red, sums + 2)) != MG_OK) return rc;
  return finish(ctx, n, k, rho, mean, mean_out, status, sums, diag);
}

// Mixed path: Y', the perturbations, d and 1/sigma^2 in FP32 from FP32
// pairs of the FP64 inputs (no FP64 instruction per element), FP32 cross
// products, the k x k solve in FP64, and the fused update (mg_update.cuh)
// that also returns the background and analysis spread sums and the
// analysis mean.
constexpr int kObsWarp = 4;
constexpr int kObsBlock = kObsWarp * (kThreads / 32);
constexpr int kUpdItemS = 512;

__global__ void __launch_bounds__(kThreads) enkf_prior_mixed_kernel(const double* __restrict__ HX,
                                                                    const double* __restrict__ yo,
                                                                    const double* __restrict__ rvar,
                                                                    const double* __restrict__ eps, int64_t p, int k,
                                                                    float* __restrict__ Y32, float* __restrict__ E32,
                                                                    float* __restrict__ d32,
                                                                    float* __restrict__ rinv32,
                                                                    double* __restrict__ dsq_part) {
  __shared__ float wsum[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t ob = (int64_t)blockIdx.x * kObsBlock + (int64_t)warp * kObsWarp;
  double hv[kObsWarp][4], ev[kObsWarp][4];
#pragma unroll
  for (int u = 0; u < kObsWarp; ++u)
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int64_t o = ob + u;
      const int i = lane + 32 * t;
      const bool in = o < p && i < k;
      hv[u][t] = in ? HX[o * k + i] : 0.0;
      ev[u][t] = in ? eps[o * k + i] : 0.0;
    }
  const float inv_k = 1.0f / (float)k;
  float dsq = 0.0f;
#pragma unroll
  for (int u = 0; u < kObsWarp; ++u) {
    const int64_t o = ob + u;
    float hh[4], hl[4], s1 = 0.0f;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      mg::split_double(hv[u][t], hh[t], hl[t]);
      s1 += hh[t] + hl[t];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s1 += __shfl_xor_sync(0xffffffffu, s1, off);
    const float m1 = s1 * inv_k;
    float pv[4], s2 = 0.0f;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      pv[t] = (lane + 32 * t < k) ? __fadd_rn(__fsub_rn(hh[t], m1), hl[t]) : 0.0f;
      s2 += pv[t];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, off);
    const float m2 = s2 * inv_k;
    if (o < p) {
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int i = lane + 32 * t;
        if (i < k) {
          float eh, el;
          mg::split_double(ev[u][t], eh, el);
          Y32[o * k + i] = pv[t] - m2;
          E32[o * k + i] = __fadd_rn(eh, el);
        }
      }
      if (lane == 0) {
        float yh, yl, vh, vl;
        mg::split_double(yo[o], yh, yl);
        mg::split_double(rvar[o], vh, vl);
        const float dd = __fsub_rn(__fadd_rn(__fsub_rn(yh, m1), yl), m2);
        d32[o] = dd;
        rinv32[o] = 1.0f / __fadd_rn(vh, vl);
        dsq = fmaf(dd, dd, dsq);
      }
    }
  }
  if (lane == 0) wsum[warp] = dsq;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < kThreads / 32; ++w) t += wsum[w];
    dsq_part[blockIdx.x] = (double)t;
  }
}

__global__ void __launch_bounds__(mg::kUpdThreads, 2) enkf_update_mixed_kernel(double* X, int64_t ld, int64_t n,
                                                                                 int k, const float* __restrict__ T32,
                                                                                 double* mean,
                                                                                 double* __restrict__ bg_part,
                                                                                 double* __restrict__ an_part) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ float red[2][mg::kUpdThreads / 32];
  const int64_t a = (int64_t)blockIdx.x * kUpdItemS;
  const int64_t b = min(n, a + kUpdItemS);
  float bg = 0.0f, an = 0.0f;
  mg::update_mixed<true>(X, ld, k, a, b, T32, mean, reinterpret_cast<float*>(smem_raw), k, bg, an);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    bg += __shfl_xor_sync(0xffffffffu, bg, off);
    an += __shfl_xor_sync(0xffffffffu, an, off);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][warp] = bg;
    red[1][warp] = an;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float tb = 0.0f, ta = 0.0f;
    for (int w = 0; w < mg::kUpdThreads / 32; ++w) {
      tb += red[0][w];
      ta += red[1][w];
    }
    bg_part[blockIdx.x] = (double)tb;
    an_part[blockIdx.x] = (double)ta;
  }
}

int run_enkf_mixed(mg_context* ctx, double* X, int64_t n, int k, int64_t ld, const double* HX, const double* yo,
                   const double* rvar, const double* eps, int64_t p, double rho, double* mean_out,
                   mg_enkf_diag* diag) {
  const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>((p + 255) / 256, 2 * ctx->num_sms));
  const int64_t per_block = (p + nblk - 1) / nblk;
  const int64_t kk = (int64_t)k * k;
  const int nprior = (int)((p + kObsBlock - 1) / kObsBlock);
  const int nupd = (int)((n + kUpdItemS - 1) / kUpdItemS);
  mg::Carver cv;
  cv.reserve<double>(n);
  cv.reserve<float>((size_t)p * k);
  cv.reserve<float>((size_t)p * k);
  cv.reserve<float>(p);
  cv.reserve<float>(p);
  cv.reserve<float>((size_t)nblk * kk);
  cv.reserve<float>((size_t)nblk * kk);
  cv.reserve<float>((size_t)nblk * k);
  cv.reserve<double>(2 * kk + k);
  cv.reserve<double>(kk);
  cv.reserve<float>(kk);
  cv.reserve<double>(nprior);
  cv.reserve<double>(nupd);
  cv.reserve<double>(nupd);
  cv.reserve<double>(4);
  cv.reserve<int>(4);
  void* ws = mg::workspace(ctx, cv.off);
  if (!ws) return MG_ERR_NOMEM;
  cv = mg::Carver{static_cast<char*>(ws), 0};
  double* mean = cv.take<double>(n);
  float* Y32 = cv.take<float>((size_t)p * k);
  float* E32 = cv.take<float>((size_t)p * k);
  float* d32 = cv.take<float>(p);
  float* rinv32 = cv.take<float>(p);
  float* Gpart = cv.take<float>((size_t)nblk * kk);
  float* Fpart = cv.take<float>((size_t)nblk * kk);
  float* bpart = cv.take<float>((size_t)nblk * k);
  double* GFb = cv.take<double>(2 * kk + k);
  double* T = cv.take<double>(kk);
  float* T32 = cv.take<float>(kk);
  double* dsq_part = cv.take<double>(nprior);
  double* bg_part = cv.take<double>(nupd);
  double* an_part = cv.take<double>(nupd);
  double* sums = cv.take<double>(4);
  int* status = cv.take<int>(4);
  cudaStream_t s = ctx->stream;
  int rc;
  enkf_prior_mixed_kernel<<<nprior, kThreads, 0, s>>>(HX, yo, rvar, eps, p, k, Y32, E32, d32, rinv32, dsq_part);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  if ((rc = launch_cross<float>(ctx, Y32, Y32, rinv32, d32, p, k, nblk, per_block, Gpart, bpart)) != MG_OK ||
      (rc = launch_cross<float>(ctx, Y32, E32, rinv32, d32, p, k, nblk, per_block, Fpart, nullptr)) != MG_OK ||
      (rc = reduce_partials<float>(ctx, Gpart, nblk, kk, GFb)) != MG_OK ||
      (rc = reduce_partials<float>(ctx, Fpart, nblk, kk, GFb + kk)) != MG_OK ||
      (rc = reduce_partials<float>(ctx, bpart, nblk, k, GFb + 2 * kk)) != MG_OK)
    return rc;
  MG_TRY_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * 4, s));
  if ((rc = launch_solve(ctx, GFb, GFb + kk, GFb + 2 * kk, k, rho, T, T32, status)) != MG_OK) return rc;
  const size_t usmem = mg::upd_bytes(k);
  MG_TRY_CUDA(cudaFuncSetAttribute(enkf_update_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)usmem));
  enkf_update_mixed_kernel<<<nupd, mg::kUpdThreads, usmem, s>>>(X, ld, n, k, T32, mean, bg_part, an_part);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  if (diag) {
    sum_partials_kernel<<<1, kThreads, 0, s>>>(dsq_part, nprior, sums + 0);
    sum_partials_kernel<<<1, kThreads, 0, s>>>(bg_part, nupd, sums + 1);
    sum_partials_kernel<<<1, kThreads, 0, s>>>(an_part, nupd, sums + 2);
    MG_COUNT_LAUNCH();
    MG_COUNT_LAUNCH();
    MG_COUNT_LAUNCH();
    MG_TRY_CUDA(cudaGetLastError());
  }
  return finish(ctx, n, k, rho, mean, mean_out, status, sums, diag);
}

}  // namespace

extern "C" int mg_enkf(mg_context* ctx, double* X, int64_t n, int32_t k, int64_t ld, const double* HX,
                       const double* yo, const double* rvar, const double* obs_pert, int64_t p, double inflation,
                       int32_t precision, double* mean_out, mg_enkf_diag* diag) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(X && n > 0 && k >= 2 && k <= 112 && ld >= n && p >= 1 && HX && yo && rvar && obs_pert &&
                   inflation > 0.0,
               "mg_enkf: bad arguments (k must be 2..112, p >= 1)");
  MG_CHECK_ARG(precision == MG_PREC_FP64 || precision == MG_PREC_MIXED, "mg_enkf: bad precision");
  if (precision == MG_PREC_FP64)
    return run_enkf_fp64(ctx, X, n, k, ld, HX, yo, rvar, obs_pert, p, inflation, mean_out, diag);
  return run_enkf_mixed(ctx, X, n, k, ld, HX, yo, rvar, obs_pert, p, inflation, mean_out, diag);
}

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

namespace {

constexpr int kThreads = 256;
constexpr int kRedBlocks = 304;

// C = sum_o rinv_o U[o]^T W[o] over this CTA's obs range (U, W: p x k
// row-major); with bout, also b = sum_o rinv_o d_o U[o].
template <int KMAX>
__global__ void __launch_bounds__(kThreads) enkf_cross_kernel(const double* __restrict__ U, const double* __restrict__ W,
                                                              const double* __restrict__ rinv,
                                                              const double* __restrict__ dinn, int64_t p, int k,
                                                              int64_t per_block, double* __restrict__ Cpart,
                                                              double* __restrict__ bpart) {
  constexpr int CH = (KMAX >= 128) ? 16 : 32, R = KMAX / 16;
  __shared__ double Us[CH * KMAX], Ws[CH * KMAX];
  __shared__ double sr[CH], sd[CH];
  const int tid = threadIdx.x, ti = tid / 16, tj = tid % 16;
  const int64_t o0 = (int64_t)blockIdx.x * per_block;
  const int64_t o1 = min(p, o0 + per_block);
  double acc[R][R];
#pragma unroll
  for (int a = 0; a < R; ++a)
#pragma unroll
    for (int b = 0; b < R; ++b) acc[a][b] = 0.0;
  double bacc = 0.0;
  for (int64_t c0 = o0; c0 < o1; c0 += CH) {
    const int cnt = (int)(o1 - c0 < (int64_t)CH ? o1 - c0 : (int64_t)CH);
    for (int e = tid; e < cnt * KMAX; e += kThreads) {
      const int r = e / KMAX, j = e - r * KMAX;
      Us[e] = (j < k) ? U[(c0 + r) * k + j] : 0.0;
      Ws[e] = (j < k) ? W[(c0 + r) * k + j] : 0.0;
    }
    if (tid < cnt) {
      sr[tid] = rinv[c0 + tid];
      sd[tid] = dinn[c0 + tid];
    }
    __syncthreads();
    for (int r = 0; r < cnt; ++r) {
      const double w = sr[r];
      double av[R], bv[R];
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
  double* C = Cpart + (size_t)blockIdx.x * k * k;
#pragma unroll
  for (int a = 0; a < R; ++a)
#pragma unroll
    for (int b = 0; b < R; ++b) {
      const int i = ti + 16 * a, j = tj + 16 * b;
      if (i < k && j < k) C[i * k + j] = acc[a][b];
    }
  if (bpart && tid < k) bpart[(size_t)blockIdx.x * k + tid] = bacc;
}

// T = sqrt(rho) (I + A^-1 (b 1^T + F - G)), A = G + (k-1) I, by Cholesky
// A = L L^T and two triangular solves on the k right-hand sides.
__global__ void __launch_bounds__(kThreads) enkf_solve_kernel(const double* __restrict__ Gpart,
                                                              const double* __restrict__ Fpart,
                                                              const double* __restrict__ bpart, int nblk, int k,
                                                              double rho, double* __restrict__ T, int* status) {
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
    T[i * k + j] = sr * ((i == j ? 1.0 : 0.0) + B[i * lda + j]);
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

__global__ void sum_partials_kernel(const double* __restrict__ partial, int nb, double* __restrict__ out) {
  if (threadIdx.x != 0) return;
  double t = 0.0;
  for (int b = 0; b < nb; ++b) t += partial[b];
  *out = t;
}

template <typename TE>
int sumsq(mg_context* ctx, const TE* v, int64_t n, double* partial, double* out) {
  sumsq_partial_kernel<TE><<<kRedBlocks, kThreads, 0, ctx->stream>>>(v, n, partial);
  MG_COUNT_LAUNCH();
  sum_partials_kernel<<<1, 32, 0, ctx->stream>>>(partial, kRedBlocks, out);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

template <int KMAX>
int launch_cross(mg_context* ctx, const double* U, const double* W, const double* rinv, const double* d, int64_t p,
                 int k, int nblk, int64_t per_block, double* Cpart, double* bpart) {
  enkf_cross_kernel<KMAX><<<nblk, kThreads, 0, ctx->stream>>>(U, W, rinv, d, p, k, per_block, Cpart, bpart);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

template <typename TE>
int run_enkf(mg_context* ctx, double* X, int64_t n, int k, int64_t ld, const double* HX, const double* yo,
             const double* rvar, const double* eps, int64_t p, double rho, double* mean_out, mg_enkf_diag* diag) {
  const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>((p + 255) / 256, 2 * ctx->num_sms));
  const int64_t per_block = (p + nblk - 1) / nblk;
  mg::Carver cv;
  cv.reserve<double>(n);
  cv.reserve<TE>((size_t)n * k);
  cv.reserve<double>((size_t)(p + 1) * k);
  cv.reserve<double>(p + 1);
  cv.reserve<double>(p + 1);
  cv.reserve<double>((size_t)nblk * k * k);
  cv.reserve<double>((size_t)nblk * k * k);
  cv.reserve<double>((size_t)nblk * k);
  cv.reserve<double>((size_t)k * k);
  cv.reserve<double>(kRedBlocks);
  cv.reserve<double>(4);
  cv.reserve<int>(4);
  void* ws = mg::workspace(ctx, cv.off);
  if (!ws) return MG_ERR_NOMEM;
  cv = mg::Carver{static_cast<char*>(ws), 0};
  double* mean = cv.take<double>(n);
  TE* Xp = cv.take<TE>((size_t)n * k);
  double* Y = cv.take<double>((size_t)(p + 1) * k);
  double* dinn = cv.take<double>(p + 1);
  double* rinv = cv.take<double>(p + 1);
  double* Gpart = cv.take<double>((size_t)nblk * k * k);
  double* Fpart = cv.take<double>((size_t)nblk * k * k);
  double* bpart = cv.take<double>((size_t)nblk * k);
  double* T = cv.take<double>((size_t)k * k);
  double* red = cv.take<double>(kRedBlocks);
  double* sums = cv.take<double>(4);
  int* status = cv.take<int>(4);
  cudaStream_t s = ctx->stream;
  const bool f64 = sizeof(TE) == 8;
  int rc;
  MG_TRY_CUDA(mg::launch_mean_pert_members(X, n, k, ld, mean, f64 ? (double*)Xp : nullptr,
                                           f64 ? nullptr : (float*)Xp, n, s));
  MG_TRY_CUDA(mg::launch_obs_prior(HX, yo, rvar, p, k, Y, nullptr, dinn, rinv, s));
  if (diag) {
    if ((rc = sumsq<double>(ctx, dinn, p, red, sums + 0)) != MG_OK) return rc;
    if ((rc = sumsq<TE>(ctx, Xp, (int64_t)n * k, red, sums + 1)) != MG_OK) return rc;
  }
  if (k <= 32) {
    if ((rc = launch_cross<32>(ctx, Y, Y, rinv, dinn, p, k, nblk, per_block, Gpart, bpart)) != MG_OK ||
        (rc = launch_cross<32>(ctx, Y, eps, rinv, dinn, p, k, nblk, per_block, Fpart, nullptr)) != MG_OK)
      return rc;
  } else if (k <= 64) {
    if ((rc = launch_cross<64>(ctx, Y, Y, rinv, dinn, p, k, nblk, per_block, Gpart, bpart)) != MG_OK ||
        (rc = launch_cross<64>(ctx, Y, eps, rinv, dinn, p, k, nblk, per_block, Fpart, nullptr)) != MG_OK)
      return rc;
  } else {
    if ((rc = launch_cross<128>(ctx, Y, Y, rinv, dinn, p, k, nblk, per_block, Gpart, bpart)) != MG_OK ||
        (rc = launch_cross<128>(ctx, Y, eps, rinv, dinn, p, k, nblk, per_block, Fpart, nullptr)) != MG_OK)
      return rc;
  }
  MG_TRY_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * 4, s));
  const size_t smem = sizeof(double) * 2 * (size_t)k * (k + 1);
  MG_TRY_CUDA(cudaFuncSetAttribute(enkf_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  enkf_solve_kernel<<<1, kThreads, smem, s>>>(Gpart, Fpart, bpart, nblk, k, rho, T, status);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  const size_t usmem = sizeof(TE) * ((size_t)k * k + 32 * (size_t)(k + 1));
  MG_TRY_CUDA(cudaFuncSetAttribute(enkf_update_kernel<TE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)usmem));
  enkf_update_kernel<TE><<<(unsigned)((n + 31) / 32), kThreads, usmem, s>>>(Xp, n, mean, T, n, k, X, ld);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  // Analysis mean and perturbations (Ensemble::RecomputeMean/Perturbations).
  MG_TRY_CUDA(mg::launch_mean_pert_members(X, n, k, ld, mean, (diag && f64) ? (double*)Xp : nullptr,
                                           (diag && !f64) ? (float*)Xp : nullptr, n, s));
  if (diag && (rc = sumsq<TE>(ctx, Xp, (int64_t)n * k, red, sums + 2)) != MG_OK) return rc;
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
    return run_enkf<double>(ctx, X, n, k, ld, HX, yo, rvar, obs_pert, p, inflation, mean_out, diag);
  return run_enkf<float>(ctx, X, n, k, ld, HX, yo, rvar, obs_pert, p, inflation, mean_out, diag);
}

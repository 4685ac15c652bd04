// Global ETKF (ETKF.hpp:100-179).
//
//   1. mean + perturbations (Ensemble.hpp:105-151), member-major;
//   2. obs-space prior ym, Y' = HX - ym, d = yo - ym (ETKF.hpp:128-141);
//   3. Gram G = Y'^T R^-1 Y' and b = Y'^T R^-1 d: every CTA reduces a
//      contiguous obs range into register tiles, partials summed in a fixed
//      order (deterministic) in FP64;
//   4. one CTA solves the k x k system (Cholesky path = the reference's
//      inverse + llt; or the Jacobi symmetric square root) into the
//      transform T (T_ji = rho (wa_j + W_ji) for the reference, whose
//      perturbations carry the inflation, ETKF.hpp:125);
//   5. Xa_i = xm + sum_j X'_j T_ji, streamed over state tiles.
// The Gram, its reduction and the k x k solve are FP64 on both paths (one
// system per analysis, negligible cost; the small eigenvalues of
// (k-1)I + Y'^T R^-1 Y' need it); the mixed path stores X' in FP32 and runs
// the O(n k^2) update in FP32.
// The reference never recomputes the ensemble mean after the update
// (ETKF.hpp:190-191); mean_out receives that background mean.
#include <algorithm>
#include <mutex>

#include "mg_dense.cuh"
#include "mg_internal.h"

namespace {

constexpr int kThreads = 256;

template <typename TE, int KMAX>
__global__ void __launch_bounds__(kThreads) gram_partial_kernel(
    const TE* __restrict__ Y, const double* __restrict__ rinv, const double* __restrict__ dinn,
    int64_t p, int k, int64_t per_block, double* __restrict__ Gpart, double* __restrict__ bpart) {
  constexpr int CH = (KMAX * sizeof(TE) > 512) ? 32 : 64, R = KMAX / 16;
  __shared__ TE Ys[CH * KMAX];
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
      Ys[e] = (j < k) ? Y[(c0 + r) * k + j] : TE(0);
    }
    if (tid < cnt) {
      sr[tid] = (TE)rinv[c0 + tid];
      sd[tid] = (TE)dinn[c0 + tid];
    }
    __syncthreads();
    for (int r = 0; r < cnt; ++r) {
      const TE w = sr[r];
      TE av[R], bv[R];
#pragma unroll
      for (int a = 0; a < R; ++a) av[a] = Ys[r * KMAX + ti * R + a] * w;
#pragma unroll
      for (int b = 0; b < R; ++b) bv[b] = Ys[r * KMAX + tj * R + b];
#pragma unroll
      for (int a = 0; a < R; ++a)
#pragma unroll
        for (int b = 0; b < R; ++b) acc[a][b] += av[a] * bv[b];
    }
    if (tid < k)
      for (int r = 0; r < cnt; ++r) bacc += (Ys[r * KMAX + tid] * sr[r]) * sd[r];
    __syncthreads();
  }
  double* G = Gpart + (size_t)blockIdx.x * k * k;
#pragma unroll
  for (int a = 0; a < R; ++a)
#pragma unroll
    for (int b = 0; b < R; ++b) {
      const int i = ti * R + a, j = tj * R + b;
      if (i < k && j < k) G[i * k + j] = (double)acc[a][b];
    }
  if (tid < k) bpart[(size_t)blockIdx.x * k + tid] = (double)bacc;
}

// Sums the partials (fixed order), adds the diagonal, solves, writes T.
template <typename TE>
__global__ void __launch_bounds__(kThreads) etkf_solve_kernel(const double* __restrict__ Gpart,
                                                              const double* __restrict__ bpart,
                                                              int nblk, int k, int flags, double rho,
                                                              double tol, int sweep_cap,
                                                              TE* __restrict__ Tout, int* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int kp = k + (k & 1), lda = kp + 1;
  TE* A = reinterpret_cast<TE*>(smem_raw);
  TE* V = A + kp * lda;
  TE* bvec = V + kp * lda;
  TE* wa = bvec + kp;
  TE* lam = wa + kp;
  TE* uvec = lam + kp;
  TE* rot = uvec + kp;
  int* pairbuf = reinterpret_cast<int*>(rot + 2 * kp);
  int* misc = pairbuf + kp;
  const int tid = threadIdx.x;
  const bool compat_infl = flags & MG_INFL_COMPAT;
  // The reference inflates the perturbations (ETKF.hpp:125), so its A keeps
  // (k-1) I; the Hunt form puts 1/rho on the prior term instead.
  const double diag = compat_infl ? (double)(k - 1) : (double)(k - 1) / rho;
  for (int e = tid; e < kp * kp; e += kThreads) {
    const int i = e / kp, j = e % kp;
    double s = 0.0;
    if (i < k && j < k) {
      for (int b = 0; b < nblk; ++b) s += Gpart[(size_t)b * k * k + i * k + j];
      if (i == j) s += diag;
    } else if (i == j) {
      s = 1.0;
    }
    A[i * lda + j] = (TE)s;
  }
  for (int i = tid; i < k; i += kThreads) {
    double s = 0.0;
    for (int b = 0; b < nblk; ++b) s += bpart[(size_t)b * k + i];
    bvec[i] = (TE)s;
  }
  __syncthreads();
  int sweeps = 0;
  // In the reference form the inflation is applied to X' rather than Pa.
  const bool ok = mg::solve_transform<TE, 128, kThreads>(A, V, bvec, wa, lam, uvec, rot, pairbuf, misc, k, kp, lda,
                                          flags & MG_SQRT_CHOLESKY, false, rho, (TE)tol, sweep_cap,
                                          &sweeps);
  const TE scale = compat_infl ? (TE)rho : TE(1);
  for (int e = tid; e < k * k; e += kThreads) {
    const int j = e / k, i = e - j * k;
    Tout[j * k + i] = scale * (wa[j] + A[j * lda + i]);
  }
  if (tid == 0 && !ok) *status = 1;
}

// Xa_i[s] = xm[s] + sum_j X'_j[s] T_ji for a tile of 32 state indices.
template <typename TE>
__global__ void __launch_bounds__(kThreads) etkf_update_kernel(const TE* __restrict__ Xp, int64_t ldp,
                                                               const double* __restrict__ mean,
                                                               const double* __restrict__ T, int64_t n,
                                                               int k, double* __restrict__ X,
                                                               int64_t ld) {
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

template <typename TE, int KMAX>
cudaError_t launch_gram(const TE* Y, const double* rinv, const double* d, int64_t p, int k,
                        int nblk, int64_t per_block, double* Gpart, double* bpart, cudaStream_t s) {
  gram_partial_kernel<TE, KMAX><<<nblk, kThreads, 0, s>>>(Y, rinv, d, p, k, per_block, Gpart, bpart);
  MG_COUNT_LAUNCH();
  return cudaGetLastError();
}

template <typename TE>
int run_etkf(mg_context* ctx, double* X, int64_t n, int k, int64_t ld, const double* HX,
             const double* yo, const double* rvar, int64_t p, double rho, int flags,
             double* mean_out) {
  const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>((p + 255) / 256, 2 * ctx->num_sms));
  const int64_t per_block = (p + nblk - 1) / nblk;
  mg::Carver cv;
  cv.reserve<double>(n);
  cv.reserve<TE>((size_t)n * k);
  cv.reserve<double>((size_t)(p + 1) * k);
  cv.reserve<double>(p + 1);
  cv.reserve<double>(p + 1);
  cv.reserve<double>((size_t)nblk * k * k);
  cv.reserve<double>((size_t)nblk * k);
  cv.reserve<double>((size_t)k * k);
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
  double* bpart = cv.take<double>((size_t)nblk * k);
  double* T = cv.take<double>((size_t)k * k);
  int* status = cv.take<int>(4);
  cudaStream_t s = ctx->stream;
  const bool f64 = sizeof(TE) == 8;
  MG_TRY_CUDA(mg::launch_mean_pert_members(X, n, k, ld, mean, f64 ? (double*)Xp : nullptr,
                                           f64 ? nullptr : (float*)Xp, n, s));
  MG_TRY_CUDA(mg::launch_obs_prior(HX, yo, rvar, p, k, Y, nullptr, dinn, rinv, s));
  if (k <= 32) MG_TRY_CUDA((launch_gram<double, 32>(Y, rinv, dinn, p, k, nblk, per_block, Gpart, bpart, s)));
  else if (k <= 64) MG_TRY_CUDA((launch_gram<double, 64>(Y, rinv, dinn, p, k, nblk, per_block, Gpart, bpart, s)));
  else MG_TRY_CUDA((launch_gram<double, 128>(Y, rinv, dinn, p, k, nblk, per_block, Gpart, bpart, s)));
  MG_TRY_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * 4, s));
  const int kp = k + (k & 1);
  const size_t smem = sizeof(double) * (2 * (size_t)kp * (kp + 1) + 6 * (size_t)kp) + sizeof(int) * (kp + 8) + 64;
  if (smem > 227 * 1024) return mg::fail(ctx, MG_ERR_ARG, "mg_etkf: k too large");
  MG_TRY_CUDA(cudaFuncSetAttribute(etkf_solve_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
  etkf_solve_kernel<double><<<1, kThreads, smem, s>>>(Gpart, bpart, nblk, k, flags, rho, 1e-14, 30, T, status);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  const size_t usmem = sizeof(TE) * ((size_t)k * k + 32 * (size_t)(k + 1));
  MG_TRY_CUDA(cudaFuncSetAttribute(etkf_update_kernel<TE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)usmem));
  etkf_update_kernel<TE><<<(unsigned)((n + 31) / 32), kThreads, usmem, s>>>(Xp, n, mean, T, n, k, X, ld);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  if (mean_out)
    MG_TRY_CUDA(cudaMemcpyAsync(mean_out, mean, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  int hs = 0;
  MG_TRY_CUDA(cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, s));
  MG_TRY_CUDA(cudaStreamSynchronize(s));
  if (hs) return mg::fail(ctx, MG_ERR_NUMERIC, "mg_etkf: the k x k system was not positive definite");
  return MG_OK;
}

}  // namespace

extern "C" int mg_etkf(mg_context* ctx, double* X, int64_t n, int32_t k, int64_t ld,
                       const double* HX, const double* yo, const double* rvar, int64_t p,
                       double rho, int32_t flags, int32_t precision, double* mean_out) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(X && n > 0 && k >= 2 && ld >= n && p >= 1 && HX && yo && rvar && rho > 0.0,
               "mg_etkf: bad arguments (k must be 2..128, p >= 1)");
  MG_CHECK_ARG(precision == MG_PREC_FP64 || precision == MG_PREC_MIXED, "mg_etkf: bad precision");
  MG_CHECK_ARG(k <= 112, "mg_etkf: k must be <= 112 (FP64 k x k solve in shared memory)");
  if (precision == MG_PREC_FP64) return run_etkf<double>(ctx, X, n, k, ld, HX, yo, rvar, p, rho, flags, mean_out);
  return run_etkf<float>(ctx, X, n, k, ld, HX, yo, rvar, p, rho, flags, mean_out);
}

// ---------------------------------------------------------------------------
// Allocation-free global ETKF.
//
// Some callers cannot allocate device memory at the point where they run the
// analysis: real-time loops whose memory budget is fixed at start-up, and
// host frameworks that own every device allocation through their own pool.
// mg_etkf_noalloc serves them: it runs the same kernels as mg_etkf, but its
// scratch lives in one file-scope device array of fixed size, so the call
// itself performs no cudaMalloc/cudaFree and no allocating library call.  It
// ends by copying the status word to the host and synchronising the stream.
// The array is part of this library's module: every GPU that loads the
// library keeps kStaticScratchBytes reserved until the process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kStaticScratchBytes = size_t(32) << 20;  // 32 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

struct StaticSetup {
  std::mutex mu;
  void* addr[kMaxDevices] = {};
  int sms[kMaxDevices] = {};
};
StaticSetup& static_setup() {
  static StaticSetup s;
  return s;
}

// Device address of g_static_scratch on the current device (and its SM
// count), looked up once per device.  In host code the array's name is only
// a host-side stand-in, never a device address.
cudaError_t static_scratch_for_current_device(void** addr, int* sms) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  StaticSetup& st = static_setup();
  std::lock_guard<std::mutex> lock(st.mu);
  if (!st.addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    int n = 0;
    e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    st.addr[dev] = p;
    st.sms[dev] = n;
  }
  *addr = st.addr[dev];
  *sms = st.sms[dev];
  return cudaSuccess;
}

template <typename TE>
int run_etkf_static(cudaStream_t s, double* X, int64_t n, int k, int64_t ld, const double* HX,
                    const double* yo, const double* rvar, int64_t p, double rho, int flags,
                    double* mean_out) {
  void* base = nullptr;
  int num_sms = 0;
  if (static_scratch_for_current_device(&base, &num_sms) != cudaSuccess) {
    cudaGetLastError();
    return MG_ERR_CUDA;
  }
  const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>((p + 255) / 256, 2 * num_sms));
  const int64_t per_block = (p + nblk - 1) / nblk;
  mg::Carver cv;
  cv.reserve<double>(n);
  cv.reserve<TE>((size_t)n * k);
  cv.reserve<double>((size_t)(p + 1) * k);
  cv.reserve<double>(p + 1);
  cv.reserve<double>(p + 1);
  cv.reserve<double>((size_t)nblk * k * k);
  cv.reserve<double>((size_t)nblk * k);
  cv.reserve<double>((size_t)k * k);
  cv.reserve<int>(4);
  if (cv.off > kStaticScratchBytes) return MG_ERR_CAPACITY;
  cv = mg::Carver{static_cast<char*>(base), 0};
  double* mean = cv.take<double>(n);
  TE* Xp = cv.take<TE>((size_t)n * k);
  double* Y = cv.take<double>((size_t)(p + 1) * k);
  double* dinn = cv.take<double>(p + 1);
  double* rinv = cv.take<double>(p + 1);
  double* Gpart = cv.take<double>((size_t)nblk * k * k);
  double* bpart = cv.take<double>((size_t)nblk * k);
  double* T = cv.take<double>((size_t)k * k);
  int* status = cv.take<int>(4);
  const bool f64 = sizeof(TE) == 8;
  auto cuda = [](cudaError_t e) { return e == cudaSuccess ? MG_OK : (cudaGetLastError(), MG_ERR_CUDA); };
  int rc;
  if ((rc = cuda(mg::launch_mean_pert_members(X, n, k, ld, mean, f64 ? (double*)Xp : nullptr,
                                              f64 ? nullptr : (float*)Xp, n, s))) != MG_OK) return rc;
  if ((rc = cuda(mg::launch_obs_prior(HX, yo, rvar, p, k, Y, nullptr, dinn, rinv, s))) != MG_OK) return rc;
  cudaError_t e;
  if (k <= 32) e = launch_gram<double, 32>(Y, rinv, dinn, p, k, nblk, per_block, Gpart, bpart, s);
  else if (k <= 64) e = launch_gram<double, 64>(Y, rinv, dinn, p, k, nblk, per_block, Gpart, bpart, s);
  else e = launch_gram<double, 128>(Y, rinv, dinn, p, k, nblk, per_block, Gpart, bpart, s);
  if ((rc = cuda(e)) != MG_OK) return rc;
  // The status word carries the previous call's value: clear it.
  if ((rc = cuda(cudaMemsetAsync(status, 0, sizeof(int) * 4, s))) != MG_OK) return rc;
  const int kp = k + (k & 1);
  const size_t smem = sizeof(double) * (2 * (size_t)kp * (kp + 1) + 6 * (size_t)kp) + sizeof(int) * (kp + 8) + 64;
  if (smem > 227 * 1024) return MG_ERR_ARG;
  if ((rc = cuda(cudaFuncSetAttribute(etkf_solve_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem))) != MG_OK) return rc;
  etkf_solve_kernel<double><<<1, kThreads, smem, s>>>(Gpart, bpart, nblk, k, flags, rho, 1e-14, 30, T, status);
  MG_COUNT_LAUNCH();
  if ((rc = cuda(cudaGetLastError())) != MG_OK) return rc;
  const size_t usmem = sizeof(TE) * ((size_t)k * k + 32 * (size_t)(k + 1));
  if ((rc = cuda(cudaFuncSetAttribute(etkf_update_kernel<TE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)usmem))) != MG_OK) return rc;
  etkf_update_kernel<TE><<<(unsigned)((n + 31) / 32), kThreads, usmem, s>>>(Xp, n, mean, T, n, k, X, ld);
  MG_COUNT_LAUNCH();
  if ((rc = cuda(cudaGetLastError())) != MG_OK) return rc;
  if (mean_out &&
      (rc = cuda(cudaMemcpyAsync(mean_out, mean, sizeof(double) * n, cudaMemcpyDeviceToDevice, s))) != MG_OK)
    return rc;
  int hs = 0;
  if ((rc = cuda(cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, s))) != MG_OK) return rc;
  if ((rc = cuda(cudaStreamSynchronize(s))) != MG_OK) return rc;
  return hs ? MG_ERR_NUMERIC : MG_OK;
}

}  // namespace

extern "C" int mg_etkf_noalloc(void* stream, double* X, int64_t n, int32_t k, int64_t ld, const double* HX,
                               const double* yo, const double* rvar, int64_t p, double rho, int32_t flags,
                               int32_t precision, double* mean_out) {
  if (!(X && n > 0 && k >= 2 && k <= 112 && ld >= n && p >= 1 && HX && yo && rvar && rho > 0.0))
    return MG_ERR_ARG;
  if (precision != MG_PREC_FP64 && precision != MG_PREC_MIXED) return MG_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (precision == MG_PREC_FP64)
    return run_etkf_static<double>(s, X, n, k, ld, HX, yo, rvar, p, rho, flags, mean_out);
  return run_etkf_static<float>(s, X, n, k, ld, HX, yo, rvar, p, rho, flags, mean_out);
}

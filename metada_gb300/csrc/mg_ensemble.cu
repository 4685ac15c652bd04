// Ensemble mean / perturbation formation (Ensemble.hpp:105-151) and the
// member-major <-> point-major transposes used by the analyses.
//
// HBM streaming kernels: every byte of the ensemble is read once and every
// output written once; the member loop runs in member order with separately
// rounded adds so that the mean is bit-identical to the reference's
// `mean += m_i` sequence followed by `mean *= 1.0/k`.
#include "mg_internal.h"

namespace {

constexpr int kTile = 32;  // state indices per transpose tile

template <typename TX>
__global__ void __launch_bounds__(256) mean_pert_members_kernel(
    const TX* __restrict__ X, int64_t n, int k, int64_t ld, double inv_k,
    double* __restrict__ mean, double* __restrict__ Xp64, float* __restrict__ Xp32, int64_t ldp) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += stride) {
    double m = 0.0;
    for (int i = 0; i < k; ++i) m = __dadd_rn(m, (double)__ldg(X + (int64_t)i * ld + s));
    m = __dmul_rn(m, inv_k);
    if (mean) mean[s] = m;
    if (Xp64 || Xp32) {
      for (int i = 0; i < k; ++i) {
        const double v = __dsub_rn((double)__ldg(X + (int64_t)i * ld + s), m);
        if (Xp64) Xp64[(int64_t)i * ldp + s] = v;
        if (Xp32) Xp32[(int64_t)i * ldp + s] = (float)v;
      }
    }
  }
}

// Member-major X -> point-major perturbations P[s*k + i] = X_i[s] - mean[s].
// One block per 32 consecutive state indices; tile staged in shared memory so
// both the member rows (input) and the point rows (output) are coalesced.
template <typename TX, typename TP>
__global__ void __launch_bounds__(256) to_point_major_kernel(const TX* __restrict__ X, int64_t n,
                                                             int k, int64_t ld, double inv_k,
                                                             double* __restrict__ mean,
                                                             TP* __restrict__ P) {
  extern __shared__ double tile[];  // [k][kTile + 1]
  __shared__ double smean[kTile];
  const int64_t s0 = (int64_t)blockIdx.x * kTile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = warp; i < k; i += nw) {
    const int64_t s = s0 + lane;
    tile[i * (kTile + 1) + lane] = (s < n) ? (double)__ldg(X + (int64_t)i * ld + s) : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < kTile) {
    double m = 0.0;
    for (int i = 0; i < k; ++i) m = __dadd_rn(m, tile[i * (kTile + 1) + threadIdx.x]);
    m = __dmul_rn(m, inv_k);
    smean[threadIdx.x] = m;
    const int64_t s = s0 + threadIdx.x;
    if (mean && s < n) mean[s] = m;
  }
  __syncthreads();
  const int total = kTile * k;
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int j = e / k, i = e - j * k;
    const int64_t s = s0 + j;
    if (s < n) P[s * k + i] = (TP)__dsub_rn(tile[i * (kTile + 1) + j], smean[j]);
  }
}

// Point-major P[s*k + i] -> member-major X_i[s] (TX: the members' storage type).
template <typename TP, typename TX>
__global__ void __launch_bounds__(256) point_major_to_members_kernel(const TP* __restrict__ P,
                                                                     int64_t n, int k,
                                                                     TX* __restrict__ X,
                                                                     int64_t ld) {
  extern __shared__ double tile[];  // [kTile][k + 1]
  const int64_t s0 = (int64_t)blockIdx.x * kTile;
  const int total = kTile * k;
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int j = e / k, i = e - j * k;
    const int64_t s = s0 + j;
    tile[j * (k + 1) + i] = (s < n) ? (double)__ldg(P + s * k + i) : 0.0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = warp; i < k; i += nw) {
    const int64_t s = s0 + lane;
    if (s < n) X[(int64_t)i * ld + s] = (TX)tile[lane * (k + 1) + i];
  }
}

inline int grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return (int)b;
}

}  // namespace

namespace mg {

cudaError_t launch_mean_pert_members(const double* X, int64_t n, int k, int64_t ld, double* mean,
                                     double* Xp64, float* Xp32, int64_t ldp, cudaStream_t s) {
  mean_pert_members_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(X, n, k, ld, 1.0 / (double)k, mean,
                                                                   Xp64, Xp32, ldp);
  MG_COUNT_LAUNCH();
  return cudaGetLastError();
}

cudaError_t launch_to_point_major(const double* X, int64_t n, int k, int64_t ld, double* mean,
                                  double* P64, float* P32, cudaStream_t s) {
  const int64_t blocks = (n + kTile - 1) / kTile;
  const size_t smem = (size_t)k * (kTile + 1) * sizeof(double);
  if (P64)
    to_point_major_kernel<double, double><<<(unsigned)blocks, 256, smem, s>>>(X, n, k, ld, 1.0 / (double)k,
                                                                              mean, P64);
  else
    to_point_major_kernel<double, float><<<(unsigned)blocks, 256, smem, s>>>(X, n, k, ld, 1.0 / (double)k,
                                                                             mean, P32);
  MG_COUNT_LAUNCH();
  return cudaGetLastError();
}

cudaError_t launch_point_major_to_members(const double* P, int64_t n, int k, double* X, int64_t ld,
                                          cudaStream_t s) {
  const int64_t blocks = (n + kTile - 1) / kTile;
  const size_t smem = (size_t)kTile * (k + 1) * sizeof(double);
  point_major_to_members_kernel<double, double><<<(unsigned)blocks, 256, smem, s>>>(P, n, k, X, ld);
  MG_COUNT_LAUNCH();
  return cudaGetLastError();
}

// Members stored as FP32: the mean in FP64 of the widened values (member
// order), FP32 perturbations point-major, and the FP32 write-back.
cudaError_t launch_mean_members_f32(const float* X, int64_t n, int k, int64_t ld, double* mean, cudaStream_t s) {
  mean_pert_members_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(X, n, k, ld, 1.0 / (double)k, mean, nullptr,
                                                                  nullptr, 0);
  MG_COUNT_LAUNCH();
  return cudaGetLastError();
}

cudaError_t launch_to_point_major_f32(const float* X, int64_t n, int k, int64_t ld, double* mean, float* P32,
                                      cudaStream_t s) {
  const int64_t blocks = (n + kTile - 1) / kTile;
  const size_t smem = (size_t)k * (kTile + 1) * sizeof(double);
  to_point_major_kernel<float, float><<<(unsigned)blocks, 256, smem, s>>>(X, n, k, ld, 1.0 / (double)k, mean, P32);
  MG_COUNT_LAUNCH();
  return cudaGetLastError();
}

cudaError_t launch_point_major_to_members_f32(const float* P, int64_t n, int k, float* X, int64_t ld,
                                              cudaStream_t s) {
  const int64_t blocks = (n + kTile - 1) / kTile;
  const size_t smem = (size_t)kTile * (k + 1) * sizeof(double);
  point_major_to_members_kernel<float, float><<<(unsigned)blocks, 256, smem, s>>>(P, n, k, X, ld);
  MG_COUNT_LAUNCH();
  return cudaGetLastError();
}

}  // namespace mg

extern "C" {

int mg_ens_mean(mg_context* ctx, const double* X, int64_t n, int32_t k, int64_t ld,
                double* mean) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(X && mean && n > 0 && k > 0 && ld >= n, "mg_ens_mean: bad arguments");
  MG_TRY_CUDA(mg::launch_mean_pert_members(X, n, k, ld, mean, nullptr, nullptr, 0, ctx->stream));
  return MG_OK;
}

int mg_ens_mean_pert(mg_context* ctx, const double* X, int64_t n, int32_t k, int64_t ld,
                     double* mean, double* Xp, int64_t ldp) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(X && mean && Xp && n > 0 && k > 0 && ld >= n && ldp >= n,
               "mg_ens_mean_pert: bad arguments");
  MG_TRY_CUDA(mg::launch_mean_pert_members(X, n, k, ld, mean, Xp, nullptr, ldp, ctx->stream));
  return MG_OK;
}

}  // extern "C"

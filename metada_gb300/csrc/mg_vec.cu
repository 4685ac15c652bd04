// Element-wise state arithmetic on the device for the device-resident state
// backend (the vector operations of SimpleState, SimpleState.hpp:96-140):
// y += x, y -= x, y *= a with one IEEE operation per element (the same
// results as the reference's host loops), and a dot product.
#include "mg_internal.h"

namespace {

__global__ void vec_update_kernel(double* __restrict__ y, const double* __restrict__ x, int64_t n, int sub) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] = sub ? __dsub_rn(y[i], x[i]) : __dadd_rn(y[i], x[i]);
}

__global__ void vec_scale_kernel(double* __restrict__ y, int64_t n, double a) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) y[i] = __dmul_rn(y[i], a);
}

// Per-block partial dot products (fixed grid and order: deterministic).
__global__ void vec_dot_kernel(const double* __restrict__ x, const double* __restrict__ y, int64_t n,
                               double* __restrict__ part) {
  __shared__ double red[32];
  double s = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) s = fma(x[i], y[i], s);
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
  }
}

__global__ void vec_sum_kernel(const double* __restrict__ part, int m, double* __restrict__ out) {
  double s = 0.0;
  for (int i = threadIdx.x; i < m; i += 32) s += part[i];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (threadIdx.x == 0) *out = s;
}

inline unsigned vec_grid(const mg_context* ctx, int64_t n) {
  int64_t b = (n + 255) / 256;
  const int64_t cap = (int64_t)(ctx->num_sms > 0 ? ctx->num_sms : 152) * 8;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace

extern "C" {

int mg_vec_update(mg_context* ctx, double* y, const double* x, int64_t n, int32_t subtract) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(y && x && n >= 0, "mg_vec_update: bad arguments");
  if (n == 0) return MG_OK;
  vec_update_kernel<<<vec_grid(ctx, n), 256, 0, ctx->stream>>>(y, x, n, subtract ? 1 : 0);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

int mg_vec_scale(mg_context* ctx, double* y, int64_t n, double a) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(y && n >= 0, "mg_vec_scale: bad arguments");
  if (n == 0) return MG_OK;
  vec_scale_kernel<<<vec_grid(ctx, n), 256, 0, ctx->stream>>>(y, n, a);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

int mg_vec_dot(mg_context* ctx, const double* x, const double* y, int64_t n, double* result) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(x && y && n >= 0 && result, "mg_vec_dot: bad arguments");
  const unsigned g = vec_grid(ctx, n);
  double* part = static_cast<double*>(mg::workspace(ctx, sizeof(double) * (g + 1)));
  if (!part) return MG_ERR_NOMEM;
  if (n == 0) {
    *result = 0.0;
    return MG_OK;
  }
  vec_dot_kernel<<<g, 256, 0, ctx->stream>>>(x, y, n, part);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  vec_sum_kernel<<<1, 32, 0, ctx->stream>>>(part, (int)g, part + g);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  MG_TRY_CUDA(cudaMemcpyAsync(result, part + g, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  MG_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
  return MG_OK;
}

}  // extern "C"

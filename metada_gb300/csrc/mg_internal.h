// Internal declarations shared by the CUDA translation units of
// libmetada_gb300.so.  Not part of the C-ABI.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "metada_gb300.h"

struct mg_context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  void* ws = nullptr;  // device workspace, grown on demand
  size_t ws_bytes = 0;
  void* host_stage = nullptr;  // pinned host staging for small read-backs
  size_t host_stage_bytes = 0;
  std::string last_error;
  mg_letkf_stats stats{};
  int64_t io_host_items = 0;  // lines or values the last text I/O call converted on the host
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};  // stage timing
};

namespace mg {

// Hand-written kernel launches on this host thread (CUB scan/sort kernels and
// memsets are not counted).  Contexts are single-threaded, so the count of a
// thread is the count of the contexts it drives.
extern thread_local int64_t g_launches;

int fail(mg_context* ctx, int code, const std::string& msg);
// Device workspace of at least `bytes`; nullptr (with last_error set) on failure.
void* workspace(mg_context* ctx, size_t bytes);
// Pinned host staging of at least `bytes`.
void* host_stage(mg_context* ctx, size_t bytes);

// Carves 256-byte aligned sub-buffers out of one workspace block.
struct Carver {
  char* base = nullptr;
  size_t off = 0;
  template <typename T>
  T* take(size_t count) {
    off = (off + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base + off);
    off += count * sizeof(T);
    return p;
  }
  template <typename T>
  void reserve(size_t count) {
    off = (off + 255) & ~size_t(255);
    off += count * sizeof(T);
  }
};

// Exclusive prefix sum of n int64 counts into offsets[0..n] (offsets[n] =
// total), using `tmp` (scan_temp_bytes(n) bytes of workspace).
size_t scan_temp_bytes(int64_t n);
cudaError_t exclusive_scan(const int64_t* counts, int64_t* offsets, int64_t n, void* tmp,
                           size_t tmp_bytes, cudaStream_t s);

// Internal stages shared between entry points (device pointers).
cudaError_t launch_mean_pert_members(const double* X, int64_t n, int k, int64_t ld, double* mean,
                                     double* Xp64, float* Xp32, int64_t ldp, cudaStream_t s);
cudaError_t launch_to_point_major(const double* X, int64_t n, int k, int64_t ld, double* mean,
                                  double* P64, float* P32, cudaStream_t s);
cudaError_t launch_point_major_to_members(const double* P, int64_t n, int k, double* X,
                                          int64_t ld, cudaStream_t s);
// The same stages for members stored as FP32 (FP64 mean of the widened values).
cudaError_t launch_mean_members_f32(const float* X, int64_t n, int k, int64_t ld, double* mean, cudaStream_t s);
cudaError_t launch_to_point_major_f32(const float* X, int64_t n, int k, int64_t ld, double* mean, float* P32,
                                      cudaStream_t s);
cudaError_t launch_point_major_to_members_f32(const float* P, int64_t n, int k, float* X, int64_t ld,
                                              cudaStream_t s);
// Obs-space prior: ym = rowmean(HX), Y' = HX - ym (FP64 and/or FP32 copies),
// d = yo - ym, rinv = 1/rvar.
cudaError_t launch_obs_prior(const double* HX, const double* yo, const double* rvar, int64_t p,
                             int k, double* Y64, float* Y32, double* d, double* rinv,
                             cudaStream_t s);

// Tensor-core GEMM (tcgen05): C = A B^T + bias, SiLU if act != 0; A (M x K)
// and B (N x K) BF16 row-major, 16-byte aligned, 1 <= N <= 256, K % 8 == 0.
// Writes C32 (FP32) and/or C16 (BF16) with leading dimension ldc; *err is
// set to 1 (not cleared) if a bounded wait gave up.
int tc_gemm_bf16(mg_context* ctx, const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K,
                 const float* bias, int act, float* C32, __nv_bfloat16* C16, int ldc, int* err);

}  // namespace mg

#define MG_TRY_CUDA(call)                                                                  \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return mg::fail(ctx, MG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define MG_COUNT_LAUNCH() (++mg::g_launches)

#define MG_CHECK_ARG(cond, msg)                              \
  do {                                                       \
    if (!(cond)) return mg::fail(ctx, MG_ERR_ARG, (msg));    \
  } while (0)

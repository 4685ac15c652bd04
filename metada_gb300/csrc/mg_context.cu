// Context, workspace, error reporting and the prefix-sum utility.
#include <cub/device/device_scan.cuh>

#include <new>

#include "mg_internal.h"

namespace mg {

thread_local int64_t g_launches = 0;

int fail(mg_context* ctx, int code, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return code;
}

void* workspace(mg_context* ctx, size_t bytes) {
  if (bytes <= ctx->ws_bytes) return ctx->ws;
  // Grow: the old block may still be read by queued work, so drain first.
  if (ctx->ws) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->ws);
    ctx->ws = nullptr;
    ctx->ws_bytes = 0;
  }
  const size_t want = bytes + bytes / 8 + (1u << 20);
  if (cudaMalloc(&ctx->ws, want) != cudaSuccess) {
    cudaGetLastError();
    ctx->last_error = "device workspace allocation of " + std::to_string(want) + " bytes failed";
    return nullptr;
  }
  ctx->ws_bytes = want;
  return ctx->ws;
}

void* host_stage(mg_context* ctx, size_t bytes) {
  if (bytes <= ctx->host_stage_bytes) return ctx->host_stage;
  if (ctx->host_stage) cudaFreeHost(ctx->host_stage);
  ctx->host_stage = nullptr;
  ctx->host_stage_bytes = 0;
  if (cudaMallocHost(&ctx->host_stage, bytes) != cudaSuccess) {
    cudaGetLastError();
    ctx->last_error = "pinned host staging allocation failed";
    return nullptr;
  }
  ctx->host_stage_bytes = bytes;
  return ctx->host_stage;
}

size_t scan_temp_bytes(int64_t n) {
  size_t bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, bytes, (const int64_t*)nullptr, (int64_t*)nullptr,
                                (int64_t)(n + 1));
  return bytes + 256;
}

// Scans n+1 values; the caller sets counts[n] = 0 so that offsets[n] holds
// the total.
cudaError_t exclusive_scan(const int64_t* counts, int64_t* offsets, int64_t n, void* tmp,
                           size_t tmp_bytes, cudaStream_t s) {
  return cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, counts, offsets, (int64_t)(n + 1), s);
}

}  // namespace mg

extern "C" {

const char* mg_version(void) { return "metada_gb300 0.1 (sm_103a)"; }

int mg_create(mg_context** out, int device) {
  if (!out) return MG_ERR_ARG;
  *out = nullptr;
  mg_context* ctx = new (std::nothrow) mg_context();
  if (!ctx) return MG_ERR_NOMEM;
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    delete ctx;
    cudaGetLastError();
    return MG_ERR_CUDA;
  }
  for (auto& ev : ctx->ev) {
    if (cudaEventCreate(&ev) != cudaSuccess) {
      cudaGetLastError();
      mg_destroy(ctx);
      return MG_ERR_CUDA;
    }
  }
  *out = ctx;
  return MG_OK;
}

void mg_destroy(mg_context* ctx) {
  if (!ctx) return;
  if (ctx->ws) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->ws);
  }
  if (ctx->host_stage) cudaFreeHost(ctx->host_stage);
  for (auto& e : ctx->ev)
    if (e) cudaEventDestroy(e);
  delete ctx;
}

int mg_set_stream(mg_context* ctx, void* stream) {
  if (!ctx) return MG_ERR_ARG;
  ctx->stream = static_cast<cudaStream_t>(stream);
  return MG_OK;
}

int mg_synchronize(mg_context* ctx) {
  if (!ctx) return MG_ERR_ARG;
  MG_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
  return MG_OK;
}

const char* mg_last_error(const mg_context* ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

int64_t mg_kernel_launches(const mg_context* ctx) { return ctx ? mg::g_launches : 0; }

int mg_letkf_last_stats(const mg_context* ctx, mg_letkf_stats* stats) {
  if (!ctx || !stats) return MG_ERR_ARG;
  *stats = ctx->stats;
  return MG_OK;
}

}  // extern "C"

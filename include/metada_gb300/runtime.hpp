// C++ RAII layer over the metada_gb300 C-ABI: status codes become
// exceptions (the reference's error convention, e.g. letkf.cpp:69-72 catches
// std::exception), device memory is owned by DeviceBuffer.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../metada_gb300.h"

namespace metada_gb300 {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Error(MG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// One library context (device, stream, workspace).  Not copyable.
class Context {
 public:
  explicit Context(int device = 0, cudaStream_t stream = nullptr) {
    const int rc = mg_create(&ctx_, device);
    if (rc != MG_OK) throw Error(rc, "mg_create failed (is a CUDA device present?)");
    if (stream) check(mg_set_stream(ctx_, stream), "mg_set_stream");
    stream_ = stream;
  }
  ~Context() { mg_destroy(ctx_); }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;

  mg_context* get() const { return ctx_; }
  cudaStream_t stream() const { return stream_; }
  void check(int rc, const char* what) const {
    if (rc != MG_OK) throw Error(rc, std::string(what) + ": " + mg_last_error(ctx_));
  }
  void synchronize() const { check(mg_synchronize(ctx_), "mg_synchronize"); }

 private:
  mg_context* ctx_ = nullptr;
  cudaStream_t stream_ = nullptr;
};

// Device array of T (cudaMalloc'd), with host upload/download helpers.
template <typename T>
class DeviceBuffer {
 public:
  DeviceBuffer() = default;
  explicit DeviceBuffer(size_t n) { resize(n); }
  ~DeviceBuffer() { release(); }
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  DeviceBuffer(DeviceBuffer&& o) noexcept : p_(std::exchange(o.p_, nullptr)), n_(std::exchange(o.n_, 0)) {}
  DeviceBuffer& operator=(DeviceBuffer&& o) noexcept {
    if (this != &o) {
      release();
      p_ = std::exchange(o.p_, nullptr);
      n_ = std::exchange(o.n_, 0);
    }
    return *this;
  }

  void resize(size_t n) {
    if (n == n_) return;
    release();
    if (n) cuda_check(cudaMalloc(&p_, n * sizeof(T)), "cudaMalloc");
    n_ = n;
  }
  void upload(const T* host, size_t n, cudaStream_t s = nullptr) {
    resize(n);
    if (n) cuda_check(cudaMemcpyAsync(p_, host, n * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
  }
  void upload(const std::vector<T>& v, cudaStream_t s = nullptr) { upload(v.data(), v.size(), s); }
  void download(T* host, size_t n, cudaStream_t s = nullptr) const {
    if (n > n_) throw Error(MG_ERR_ARG, "DeviceBuffer::download: too many elements");
    if (n) cuda_check(cudaMemcpyAsync(host, p_, n * sizeof(T), cudaMemcpyDeviceToHost, s), "download");
    cuda_check(cudaStreamSynchronize(s), "download sync");
  }
  std::vector<T> to_vector(cudaStream_t s = nullptr) const {
    std::vector<T> v(n_);
    download(v.data(), n_, s);
    return v;
  }
  T* data() const { return p_; }
  size_t size() const { return n_; }

 private:
  void release() {
    if (p_) cudaFree(p_);
    p_ = nullptr;
    n_ = 0;
  }
  T* p_ = nullptr;
  size_t n_ = 0;
};

}  // namespace metada_gb300

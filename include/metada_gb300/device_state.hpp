// Device-resident state backend for METADA's State adapter.
//
// DeviceState<Geometry> satisfies the reference's StateBackendImpl concept
// (src/framework/adapters/StateConcepts.hpp:47-84) with the interface of
// SimpleState (src/backends/simple/SimpleState.hpp:20-270): construction
// from (config, geometry) reading the "file" (and "variables") keys,
// getData(), at(), size(), clone(), zero/add/subtract/multiply/dot/norm/
// equals, saveToFile().  The device copy is authoritative:
//  - the state file is parsed on the device (mg_parse_values) and the
//    analysis policies of analysis.hpp read and write the members in device
//    memory (device_data()), device to device;
//  - add, subtract, multiply (so Ensemble::RecomputeMean,
//    Ensemble.hpp:105-114) and dot run on the device (mg_vec_*), with the
//    same IEEE results as SimpleState's loops for add/subtract/multiply;
//  - saveToFile() formats the text on the device (mg_format_state);
//  - a host copy is materialised only when a caller asks for host access
//    (getData(), at(), operator[]); non-const host access marks the device
//    copy stale, and the next device use uploads the host copy.
// host_transfers() counts the uploads and downloads of state data, so a
// caller can check that analysis cycles keep the ensemble on the device.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <iterator>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "runtime.hpp"

namespace metada_gb300 {

// One library context per process for the state backends (device 0 unless
// METADA_GB300_DEVICE names another), created on first use.
inline Context& state_context() {
  static Context ctx([] {
    const char* e = std::getenv("METADA_GB300_DEVICE");
    return e ? std::atoi(e) : 0;
  }());
  return ctx;
}

inline long long& state_transfer_counter() {
  static long long n = 0;
  return n;
}

template <typename Geometry>
class DeviceState {
 public:
  DeviceState() = delete;
  DeviceState(const DeviceState&) = delete;
  DeviceState& operator=(const DeviceState&) = delete;
  DeviceState(DeviceState&& o) noexcept
      : dev_(std::move(o.dev_)),
        host_(std::move(o.host_)),
        names_(std::move(o.names_)),
        geometry_(o.geometry_),
        n_(o.n_),
        host_valid_(o.host_valid_),
        device_valid_(o.device_valid_) {}
  DeviceState& operator=(DeviceState&& o) noexcept {
    if (this != &o) {
      dev_ = std::move(o.dev_);
      host_ = std::move(o.host_);
      names_ = std::move(o.names_);
      n_ = o.n_;
      host_valid_ = o.host_valid_;
      device_valid_ = o.device_valid_;
    }
    return *this;
  }
  ~DeviceState() = default;

  // SimpleState's configuration keys (SimpleState.hpp:45-64): "variables"
  // (string or list, default {"state"}) and "file", read with the same
  // getline + istringstream rules, here on the device.
  template <typename ConfigBackend>
  DeviceState(const ConfigBackend& config, const Geometry& geometry) : geometry_(&geometry) {
    try {
      auto v = config.Get("variables");
      if (v.isString()) names_ = {v.asString()};
      else names_ = v.asVectorString();
    } catch (...) {
      names_ = {"state"};
    }
    const std::string filename = config.Get("file").asString();
    std::ifstream f(filename, std::ios::binary);
    if (!f) throw std::runtime_error("Cannot open state file: " + filename);
    const std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    Context& ctx = state_context();
    const int64_t bound = ((int64_t)text.size() + 1) / 2 + 1;  // two values need a separator
    DeviceBuffer<double> tmp(bound);
    int64_t count = 0;
    ctx.check(mg_parse_values(ctx.get(), text.data(), (int64_t)text.size(), tmp.data(), bound, &count),
              "mg_parse_values");
    n_ = (size_t)count;
    dev_.resize(n_);
    if (n_)
      cuda_check(cudaMemcpyAsync(dev_.data(), tmp.data(), n_ * sizeof(double), cudaMemcpyDeviceToDevice,
                                 ctx.stream()),
                 "state copy");
    ctx.synchronize();
    device_valid_ = true;
    host_valid_ = false;
  }

  // ---- device access (the analysis policies) ----
  double* device_data() {
    sync_device();
    host_valid_ = false;  // the caller may write
    return dev_.data();
  }
  const double* device_data() const {
    sync_device();
    return dev_.data();
  }

  // ---- StateBackendImpl ----
  void* getData() {
    sync_host();
    device_valid_ = false;  // the caller may write through the pointer
    return host_.data();
  }
  const void* getData() const {
    sync_host();
    return host_.data();
  }
  const std::vector<std::string>& getVariableNames() const { return names_; }
  size_t size() const { return n_; }
  const Geometry& geometry() const { return *geometry_; }

  std::unique_ptr<DeviceState> clone() const {
    std::unique_ptr<DeviceState> c(new DeviceState(*geometry_, names_, n_));
    if (device_valid_ || !host_valid_) {
      Context& ctx = state_context();
      if (n_)
        cuda_check(cudaMemcpyAsync(c->dev_.data(), dev_.data(), n_ * sizeof(double), cudaMemcpyDeviceToDevice,
                                   ctx.stream()),
                   "clone");
      c->device_valid_ = true;
      c->host_valid_ = false;
    } else {
      c->host_ = host_;
      c->host_valid_ = true;
      c->device_valid_ = false;
    }
    return c;
  }

  void zero() {
    Context& ctx = state_context();
    dev_.resize(n_);
    if (n_) cuda_check(cudaMemsetAsync(dev_.data(), 0, n_ * sizeof(double), ctx.stream()), "zero");
    device_valid_ = true;
    host_valid_ = false;
  }
  void add(const DeviceState& o) { update(o, 0); }
  // SimpleState::addIncrement (SimpleState.hpp:120-128): the increment (a
  // host backend) is extracted, uploaded and added on the device.
  template <typename IncrementBackend>
  void addIncrement(const IncrementBackend& increment) {
    std::vector<double> tmp(n_);
    increment.extract(tmp.data(), nullptr, nullptr, nullptr, nullptr);
    Context& ctx = state_context();
    DeviceBuffer<double> d;
    d.upload(tmp, ctx.stream());
    ctx.check(mg_vec_update(ctx.get(), device_data(), d.data(), (int64_t)n_, 0), "mg_vec_update");
    ctx.synchronize();
  }
  void subtract(const DeviceState& o) { update(o, 1); }
  void multiply(double a) {
    Context& ctx = state_context();
    ctx.check(mg_vec_scale(ctx.get(), device_data(), (int64_t)n_, a), "mg_vec_scale");
  }
  double dot(const DeviceState& o) const {
    if (o.n_ != n_) throw std::runtime_error("Cannot compute dot product of states of different sizes");
    Context& ctx = state_context();
    double r = 0.0;
    ctx.check(mg_vec_dot(ctx.get(), device_data(), o.device_data(), (int64_t)n_, &r), "mg_vec_dot");
    return r;
  }
  double norm() const { return std::sqrt(dot(*this)); }
  bool equals(const DeviceState& o) const {
    if (o.n_ != n_) return false;
    sync_host();
    o.sync_host();
    for (size_t i = 0; i < n_; ++i)
      if (host_[i] != o.host_[i]) return false;
    return true;
  }

  // SimpleState::saveToFile (SimpleState.hpp:160-188): ny rows of nx
  // "%12.6f" values joined by one space, formatted on the device.
  void saveToFile(const std::string& filename) const {
    std::filesystem::path path(filename);
    if (!path.parent_path().empty() && !std::filesystem::exists(path.parent_path()))
      std::filesystem::create_directories(path.parent_path());
    const int nx = (int)geometry_->x_dim(), ny = (int)geometry_->y_dim();
    if ((size_t)nx * (size_t)ny != n_) throw std::runtime_error("saveToFile: state size differs from the grid");
    Context& ctx = state_context();
    int64_t nbytes = 0;
    std::vector<char> text(25 * n_ + 1);
    ctx.check(mg_format_state(ctx.get(), device_data(), nx, ny, text.data(), (int64_t)text.size(), &nbytes),
              "mg_format_state");
    std::ofstream f(filename, std::ios::binary);
    if (!f.is_open()) throw std::runtime_error("Could not open file for writing: " + filename);
    f.write(text.data(), nbytes);
  }

  // Coordinate and location access (SimpleState.hpp:73-80, 190-199): host copy.
  double& at(const std::pair<int, int>& c) {
    sync_host();
    device_valid_ = false;
    return host_[(size_t)c.second * geometry_->x_dim() + c.first];
  }
  const double& at(const std::pair<int, int>& c) const {
    sync_host();
    return host_[(size_t)c.second * geometry_->x_dim() + c.first];
  }
  template <typename Loc>
  double& at(const Loc& loc) {
    return at(std::pair<int, int>(loc.getGridCoords2D()));
  }
  template <typename Loc>
  const double& at(const Loc& loc) const {
    return at(std::pair<int, int>(loc.getGridCoords2D()));
  }
  double& operator[](size_t i) {
    if (i >= n_) throw std::out_of_range("Index out of range");
    sync_host();
    device_valid_ = false;
    return host_[i];
  }
  const double& operator[](size_t i) const {
    if (i >= n_) throw std::out_of_range("Index out of range");
    sync_host();
    return host_[i];
  }

  // Uploads plus downloads of state data by every DeviceState of the process.
  static long long host_transfers() { return state_transfer_counter(); }

 private:
  DeviceState(const Geometry& g, std::vector<std::string> names, size_t n)
      : names_(std::move(names)), geometry_(&g), n_(n) {
    dev_.resize(n_);
  }

  void update(const DeviceState& o, int sub) {
    if (o.n_ != n_) throw std::runtime_error(sub ? "Cannot subtract states of different sizes"
                                                 : "Cannot add states of different sizes");
    Context& ctx = state_context();
    const double* x = o.device_data();
    ctx.check(mg_vec_update(ctx.get(), device_data(), x, (int64_t)n_, sub), "mg_vec_update");
  }

  void sync_host() const {
    if (host_valid_) return;
    host_.resize(n_);
    if (n_) dev_.download(host_.data(), n_, state_context().stream());
    ++state_transfer_counter();
    host_valid_ = true;
  }
  void sync_device() const {
    if (device_valid_) return;
    Context& ctx = state_context();
    dev_.resize(n_);
    if (n_)
      cuda_check(cudaMemcpyAsync(dev_.data(), host_.data(), n_ * sizeof(double), cudaMemcpyHostToDevice,
                                 ctx.stream()),
                 "state upload");
    cuda_check(cudaStreamSynchronize(ctx.stream()), "state upload sync");
    ++state_transfer_counter();
    device_valid_ = true;
  }

  mutable DeviceBuffer<double> dev_;
  mutable std::vector<double> host_;
  std::vector<std::string> names_;
  const Geometry* geometry_ = nullptr;
  size_t n_ = 0;
  mutable bool host_valid_ = false;
  mutable bool device_valid_ = false;
};

}  // namespace metada_gb300

// Map-backed configuration backend and a backend tag binding the reference's
// Simple backend, GridObservation and IdentityObsOperator, for programs
// that compile the reference's own headers on the host (test
// infrastructure: the reference harness and the drop-in compile check).
// The reference's YAML backend needs yaml-cpp, which is not installed.
#pragma once
#include <sstream>
#include <stdexcept>
#include <string>

#include "ConfigValue.hpp"

namespace harness {

namespace fw = metada::framework;

// Configuration backend over an in-memory ConfigMap (dotted keys allowed).
class MapConfig {
 public:
  MapConfig() = delete;
  MapConfig(const MapConfig&) = delete;
  MapConfig& operator=(const MapConfig&) = delete;
  MapConfig(MapConfig&&) noexcept = default;
  MapConfig& operator=(MapConfig&&) noexcept = default;
  ~MapConfig() = default;

  explicit MapConfig(const std::string& filename) {
    throw std::runtime_error("MapConfig cannot load files: " + filename);
  }
  explicit MapConfig(const fw::ConfigMap& map) : root_(map) {}

  bool LoadFromFile(const std::string&) { return false; }
  bool LoadFromString(const std::string&) { return false; }

  fw::ConfigValue Get(const std::string& key) const {
    fw::ConfigValue cur(root_);
    std::stringstream ss(key);
    std::string part;
    while (std::getline(ss, part, '.')) {
      if (!cur.hasKey(part)) throw std::runtime_error("missing config key: " + key);
      cur = cur.get(part);
    }
    return cur;
  }
  void Set(const std::string& key, const fw::ConfigValue& value) { root_[key] = value; }
  bool HasKey(const std::string& key) const {
    try {
      Get(key);
      return true;
    } catch (...) {
      return false;
    }
  }
  bool SaveToFile(const std::string&) const { return false; }
  std::string ToString() const { return "MapConfig"; }
  void Clear() { root_.clear(); }
  MapConfig CreateSubsection(const std::string& key) const { return MapConfig(Get(key).asMap()); }

 private:
  fw::ConfigMap root_;
};

}  // namespace harness

#include "BackendTraits.hpp"
#include "ConsoleLogger.hpp"
#include "GridObservation.hpp"
#include "IdentityObsOperator.hpp"
#include "SimpleBackgroundErrorCovariance.hpp"
#include "SimpleGeometry.hpp"
#include "SimpleGeometryIterator.hpp"
#include "SimpleIncrement.hpp"
#include "SimpleModel.hpp"
#include "SimpleState.hpp"

namespace harness {
struct HarnessBackendTag {};
}  // namespace harness

namespace metada::traits {
template <>
struct BackendTraits<harness::HarnessBackendTag> {
  using ConfigBackend = harness::MapConfig;
  using LoggerBackend = backends::logger::ConsoleLogger<ConfigBackend>;
  using GeometryBackend = backends::simple::SimpleGeometry;
  using GeometryIteratorBackend =
      backends::simple::SimpleGeometryIterator<typename GeometryBackend::const_iterator>;
  using StateBackend = backends::simple::SimpleState;
  using IncrementBackend = backends::simple::SimpleIncrement;
  using ControlVariableBackend = backends::simple::SimpleIncrement;
  using ObservationBackend = backends::common::observation::GridObservation;
  using ObservationIteratorBackend = backends::common::observation::GridObservationIterator;
  using ObsOperatorBackend =
      backends::common::obsoperator::IdentityObsOperator<StateBackend, ObservationBackend,
                                                         ControlVariableBackend>;
  using ModelBackend = backends::simple::SimpleModel;
  using BackgroundErrorCovarianceBackend = backends::simple::SimpleBackgroundErrorCovariance;
};
}  // namespace metada::traits


// GPU run of the drop-in policies with the device-resident state backend
// (metada_gb300::DeviceState, the Gb300BackendTag state): ensemble members
// are read from SimpleState text files on the device, two LETKF cycles run
// with the members in device memory, Ensemble::RecomputeMean runs on the
// device through the state's add/multiply, and the state writer formats on
// the device.  The adapters below stand in for METADA's State<Tag> and
// Ensemble<Tag> with the same member functions and semantics
// (src/framework/adapters/State.hpp:100-386, Ensemble.hpp:51-160), since the
// reference tree is not available where this runs.
//
// usage: dropin_device CASE_DIR OUT_DIR
//   CASE_DIR/meta.txt: "nx ny k p sigma rho radius"; CASE_DIR/ens_<i>.txt
//   (SimpleState text, i = 1..k); obs_xy.bin (p x 2 int32), yo.bin (p f64).
//   Writes OUT_DIR/cycle1.bin, cycle2.bin (k x n f64), mean.txt (the
//   device-formatted analysis mean), transfers.txt ("before after1 after2":
//   state uploads + downloads counted at those points).
#include <cmath>
#include <cstdint>
#include <fstream>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "metada_gb300/analysis.hpp"
#include "metada_gb300/device_state.hpp"

namespace mock {

struct Location {
  int x, y;
  std::pair<int, int> getGridCoords2D() const { return {x, y}; }
  std::tuple<double, double, double> getGeographicCoords() const {
    throw std::runtime_error("Location is not in geographic coordinate system");
  }
};

struct Geometry {  // SimpleGeometry: x_dim/y_dim, iteration y outer, x inner
  int nx, ny;
  std::vector<Location> pts;
  Geometry(int nx_, int ny_) : nx(nx_), ny(ny_) {
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) pts.push_back({x, y});
  }
  size_t x_dim() const { return (size_t)nx; }
  size_t y_dim() const { return (size_t)ny; }
  auto begin() const { return pts.begin(); }
  auto end() const { return pts.end(); }
};

struct Value {
  std::string s;
  bool isString() const { return true; }
  std::string asString() const { return s; }
  std::vector<std::string> asVectorString() const { return {s}; }
  float asFloat() const { return std::stof(s); }
  int asInt() const { return std::stoi(s); }
};

struct Config {
  std::map<std::string, std::string> kv;
  Value Get(const std::string& k) const {
    auto it = kv.find(k);
    if (it == kv.end()) throw std::runtime_error("missing key " + k);
    return {it->second};
  }
  bool HasKey(const std::string& k) const { return kv.count(k) > 0; }
  const Config& GetSubsection(const std::string&) const { return *this; }
};

using Backend = metada_gb300::DeviceState<Geometry>;

// framework::State<Tag> over the backend (State.hpp:100-386).
class State {
 public:
  State(const Config& c, const Geometry& g) : backend_(c, g), geometry_(&g) {}
  explicit State(Backend&& b, const Geometry* g) : backend_(std::move(b)), geometry_(g) {}
  State(State&&) noexcept = default;
  State& operator=(State&&) noexcept = default;
  State clone() const { return State(std::move(*backend_.clone()), geometry_); }
  State& zero() {
    backend_.zero();
    return *this;
  }
  State& operator+=(const State& o) {
    backend_.add(o.backend_);
    return *this;
  }
  State& operator-=(const State& o) {
    backend_.subtract(o.backend_);
    return *this;
  }
  State& operator*=(double a) {
    backend_.multiply(a);
    return *this;
  }
  template <typename T>
  T* getDataPtr() {
    return static_cast<T*>(backend_.getData());
  }
  template <typename T>
  const T* getDataPtr() const {
    return static_cast<const T*>(backend_.getData());
  }
  size_t size() const { return backend_.size(); }
  const Geometry* geometry() const { return geometry_; }
  void saveToFile(const std::string& f) const { backend_.saveToFile(f); }
  Backend& backend() { return backend_; }
  const Backend& backend() const { return backend_; }

 private:
  Backend backend_;
  const Geometry* geometry_;
};

// framework::Ensemble<Tag> (Ensemble.hpp:51-160).
class Ensemble {
 public:
  std::vector<State> members;
  size_t Size() const { return members.size(); }
  State& GetMember(size_t i) { return members.at(i); }
  const State& GetMember(size_t i) const { return members.at(i); }
  void RecomputeMean() {  // Ensemble.hpp:105-114
    if (!mean_) mean_ = std::make_unique<State>(members[0].clone());
    mean_->zero();
    for (auto& m : members) *mean_ += m;
    *mean_ *= (1.0 / static_cast<double>(members.size()));
  }
  State& Mean() {
    if (!mean_) RecomputeMean();
    return *mean_;
  }
  void RecomputePerturbations() {}

 private:
  std::unique_ptr<State> mean_;
};

struct ObsPoint {
  Location location;
  double value, error;
  bool is_valid;
};

struct Observation {
  std::vector<ObsPoint> pts;
  auto begin() const { return pts.begin(); }
  auto end() const { return pts.end(); }
  std::vector<double> getObservationValues() const {
    std::vector<double> v;
    for (auto& p : pts) v.push_back(p.value);
    return v;
  }
  std::vector<double> getCovariance() const {
    std::vector<double> v;
    for (auto& p : pts) v.push_back(p.is_valid ? p.error * p.error : std::numeric_limits<double>::infinity());
    return v;
  }
};

struct ObsOperator {  // unused: grid observations take the device IDW4 operator
  std::vector<double> apply(const State&, const Observation&) const {
    throw std::runtime_error("host operator not expected");
  }
};

}  // namespace mock

struct DeviceTag {};

template <typename T>
std::vector<T> read_bin(const std::string& path, size_t n) {
  std::vector<T> v(n);
  std::ifstream f(path, std::ios::binary);
  if (!f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(T))))
    throw std::runtime_error("cannot read " + path);
  return v;
}

void write_members(const mock::Ensemble& ens, const std::string& path) {
  std::ofstream f(path, std::ios::binary);
  for (const auto& m : ens.members) {
    const double* d = m.getDataPtr<double>();  // const access: a download, the device copy stays current
    f.write(reinterpret_cast<const char*>(d), (std::streamsize)(m.size() * sizeof(double)));
  }
}

int main(int argc, char** argv) {
  try {
    if (argc != 3) {
      std::cerr << "usage: dropin_device CASE_DIR OUT_DIR\n";
      return 2;
    }
    const std::string dir = argv[1], out = argv[2];
    std::ifstream meta(dir + "/meta.txt");
    int nx, ny, k, p;
    std::string sigma, rho, radius;
    meta >> nx >> ny >> k >> p >> sigma >> rho >> radius;
    mock::Geometry geom(nx, ny);
    mock::Ensemble ens;
    for (int i = 1; i <= k; ++i) {
      mock::Config sc;
      sc.kv = {{"file", dir + "/ens_" + std::to_string(i) + ".txt"}, {"variables", "state"}};
      ens.members.emplace_back(sc, geom);
    }
    const auto xy = read_bin<int32_t>(dir + "/obs_xy.bin", (size_t)p * 2);
    const auto yo = read_bin<double>(dir + "/yo.bin", (size_t)p);
    mock::Observation obs;
    for (int o = 0; o < p; ++o) obs.pts.push_back({{xy[2 * o], xy[2 * o + 1]}, yo[o], std::stod(sigma), true});
    mock::ObsOperator H;
    mock::Config cfg;
    cfg.kv = {{"inflation", rho}, {"localization_radius", radius}, {"output_base_file", out + "/analysis"},
              {"format", "txt"}};
    const long long t0 = mock::Backend::host_transfers();
    metada_gb300::LETKF<DeviceTag> cycle1(ens, obs, H, cfg);
    cycle1.Analyse();
    const long long t1 = mock::Backend::host_transfers();
    write_members(ens, out + "/cycle1.bin");
    const long long t1b = mock::Backend::host_transfers();
    metada_gb300::LETKF<DeviceTag> cycle2(ens, obs, H, cfg);
    cycle2.Analyse();
    const long long t2 = mock::Backend::host_transfers();
    ens.Mean().saveToFile(out + "/mean.txt");
    write_members(ens, out + "/cycle2.bin");
    std::ofstream(out + "/transfers.txt") << t0 << " " << t1 << " " << t1b << " " << t2 << "\n";
    return 0;
  } catch (const std::exception& e) {
    std::cerr << "dropin_device failed: " << e.what() << std::endl;
    return 1;
  }
}

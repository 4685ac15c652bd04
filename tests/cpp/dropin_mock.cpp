// GPU run of the C++ drop-in policies (include/metada_gb300/analysis.hpp)
// through minimal stand-ins for METADA's adapters: the same member functions
// the policies call on framework::Ensemble / State / Geometry / Observation /
// ObsOperator / Config, nothing else.  Built and run by
// tests/test_gpu_cpp.py, which compares the analysis with the golden vectors.
//
// usage: dropin_mock CASE_DIR MODE OUT_DIR
//   CASE_DIR/meta.txt: "nx ny k p sigma rho radius"; X.bin (k x nx*ny f64),
//   obs_xy.bin (p x 2 int32), yo.bin (p f64).
//   MODE: letkf_sequential | letkf_batched_reference | letkf_batched_hunt_mixed |
//         etkf_reference | etkf_reference_host_h | enkf_seed1234
//   writes OUT_DIR/members.bin (k x n f64) and OUT_DIR/mean.bin.
#include <cmath>
#include <cstdint>
#include <fstream>
#include <iostream>
#include <limits>
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "metada_gb300/analysis.hpp"

namespace mock {

struct Location {  // framework::Location, grid coordinates only
  int x, y;
  std::pair<int, int> getGridCoords2D() const { return {x, y}; }
  std::tuple<double, double, double> getGeographicCoords() const {
    throw std::runtime_error("Location is not in geographic coordinate system");
  }
};

struct Geometry {  // SimpleGeometry iteration: y outer, x inner
  int nx, ny;
  std::vector<Location> pts;
  Geometry(int nx_, int ny_) : nx(nx_), ny(ny_) {
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) pts.push_back({x, y});
  }
  auto begin() const { return pts.begin(); }
  auto end() const { return pts.end(); }
};

struct State {
  std::vector<double> data;
  const Geometry* geom;
  size_t size() const { return data.size(); }
  template <typename T>
  T* getDataPtr() { return reinterpret_cast<T*>(data.data()); }
  template <typename T>
  const T* getDataPtr() const { return reinterpret_cast<const T*>(data.data()); }
  const Geometry* geometry() const { return geom; }
  void saveToFile(const std::string&) const {}
};

struct Ensemble {
  std::vector<State> members;
  State mean;
  size_t Size() const { return members.size(); }
  State& GetMember(size_t i) { return members.at(i); }
  const State& GetMember(size_t i) const { return members.at(i); }
  void RecomputeMean() {  // Ensemble.hpp:105-114
    mean.data.assign(members[0].data.size(), 0.0);
    for (auto& m : members)
      for (size_t s = 0; s < m.data.size(); ++s) mean.data[s] += m.data[s];
    for (auto& v : mean.data) v *= 1.0 / static_cast<double>(members.size());
  }
  State& Mean() { return mean; }
  void RecomputePerturbations() {}  // the policies do not read them back
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
  size_t size() const { return pts.size(); }
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

struct ObsOperator {  // IdentityObsOperator::apply for grid obs on SimpleState
  std::vector<double> apply(const State& st, const Observation& obs) const {
    const int nx = st.geom->nx, ny = st.geom->ny;
    std::vector<double> out;
    for (const auto& o : obs.pts) {
      if (!o.is_valid) {
        out.push_back(0.0);
        continue;
      }
      const double x = std::max(0.0, std::min((double)(nx - 1), (double)o.location.x));
      const double y = std::max(0.0, std::min((double)(ny - 1), (double)o.location.y));
      const long i0 = (long)std::floor(x), j0 = (long)std::floor(y);
      const long i1 = std::min(i0 + 1, (long)nx - 1), j1 = std::min(j0 + 1, (long)ny - 1);
      const long ii[4] = {i0, i1, i0, i1}, jj[4] = {j0, j0, j1, j1};
      double ws = 0.0, wsum = 0.0;
      for (int t = 0; t < 4; ++t) {
        const double dx = x - ii[t], dy = y - jj[t];
        const double d = std::sqrt(dx * dx + dy * dy);
        const double w = d == 0.0 ? 1e12 : 1.0 / d;
        ws += w * st.data[jj[t] * nx + ii[t]];
        wsum += w;
      }
      out.push_back(ws / wsum);
    }
    return out;
  }
};

struct Value {
  std::string s;
  float asFloat() const { return std::stof(s); }
  int asInt() const { return std::stoi(s); }
  std::string asString() const { return s; }
};

struct Config {  // one flat map; GetSubsection("analysis") is the map itself
  std::map<std::string, std::string> kv;
  Value Get(const std::string& k) const {
    auto it = kv.find(k);
    if (it == kv.end()) throw std::runtime_error("missing key " + k);
    return {it->second};
  }
  bool HasKey(const std::string& k) const { return kv.count(k) > 0; }
  const Config& GetSubsection(const std::string&) const { return *this; }
};

}  // namespace mock

struct MockTag {};

template <typename T>
std::vector<T> read_bin(const std::string& path, size_t n) {
  std::vector<T> v(n);
  std::ifstream f(path, std::ios::binary);
  if (!f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(T))))
    throw std::runtime_error("cannot read " + path);
  return v;
}

int main(int argc, char** argv) {
  try {
    if (argc != 4) {
      std::cerr << "usage: dropin_mock CASE_DIR MODE OUT_DIR\n";
      return 2;
    }
    const std::string dir = argv[1], mode = argv[2], out = argv[3];
    std::ifstream meta(dir + "/meta.txt");
    int nx, ny, k, p;
    std::string sigma, rho, radius;
    meta >> nx >> ny >> k >> p >> sigma >> rho >> radius;
    const size_t n = (size_t)nx * ny;
    mock::Geometry geom(nx, ny);
    mock::Ensemble ens;
    const auto X = read_bin<double>(dir + "/X.bin", (size_t)k * n);
    for (int i = 0; i < k; ++i)
      ens.members.push_back({std::vector<double>(X.begin() + (size_t)i * n, X.begin() + (size_t)(i + 1) * n), &geom});
    ens.mean = {std::vector<double>(n, 0.0), &geom};
    const auto xy = read_bin<int32_t>(dir + "/obs_xy.bin", (size_t)p * 2);
    const auto yo = read_bin<double>(dir + "/yo.bin", (size_t)p);
    mock::Observation obs;
    for (int o = 0; o < p; ++o) obs.pts.push_back({{xy[2 * o], xy[2 * o + 1]}, yo[o], std::stod(sigma), true});
    mock::ObsOperator H;
    mock::Config cfg;
    cfg.kv = {{"inflation", rho}, {"localization_radius", radius}, {"output_base_file", out + "/analysis"},
              {"format", "txt"}};
    if (mode == "letkf_sequential") {
      metada_gb300::LETKF<MockTag> a(ens, obs, H, cfg);
      a.Analyse();
    } else if (mode == "letkf_batched_reference") {
      cfg.kv["order"] = "batched";
      metada_gb300::LETKF<MockTag> a(ens, obs, H, cfg);
      a.Analyse();
    } else if (mode == "letkf_batched_hunt_mixed") {
      cfg.kv["order"] = "batched";
      cfg.kv["semantics"] = "hunt";
      cfg.kv["precision"] = "mixed";
      metada_gb300::LETKF<MockTag> a(ens, obs, H, cfg);
      a.Analyse();
    } else if (mode == "etkf_reference") {
      metada_gb300::ETKF<MockTag> a(ens, obs, H, cfg);
      a.Analyse();
    } else if (mode == "etkf_reference_host_h") {
      cfg.kv["obs_operator_on_device"] = "host";
      metada_gb300::ETKF<MockTag> a(ens, obs, H, cfg);
      a.Analyse();
    } else if (mode == "enkf_seed1234") {
      cfg.kv["inflation_method"] = "multiplicative";
      cfg.kv["seed"] = "1234";
      metada_gb300::EnKF<MockTag> a(ens, obs, H, cfg);
      a.Analyse();
      const auto r = a.getAnalysisResults();
      std::ofstream fd(out + "/diag.bin", std::ios::binary);
      const double d[3] = {r.innovation_norm, r.background_spread, r.analysis_spread};
      fd.write(reinterpret_cast<const char*>(d), sizeof(d));
    } else {
      throw std::runtime_error("unknown mode " + mode);
    }
    std::ofstream fm(out + "/members.bin", std::ios::binary);
    for (int i = 0; i < k; ++i)
      fm.write(reinterpret_cast<const char*>(ens.members[i].data.data()), (std::streamsize)(n * sizeof(double)));
    std::ofstream fmean(out + "/mean.bin", std::ios::binary);
    fmean.write(reinterpret_cast<const char*>(ens.mean.data.data()), (std::streamsize)(n * sizeof(double)));
    return 0;
  } catch (const std::exception& e) {
    std::cerr << "dropin_mock failed: " << e.what() << std::endl;
    return 1;
  }
}

// Reference harness: runs the reference's OWN analysis headers
// (src/framework/algorithms/ETKF.hpp, LETKF.hpp over the Simple backend,
// GridObservation and IdentityObsOperator) unmodified, to pin the oracle.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build_ref.sh from the reference
// tree in place (nothing of it is copied here), against the Eigen subset in
// oracle/eigen_subset and a map-backed configuration backend written here
// (the reference's YAML backend needs yaml-cpp, which is not installed).
// Output goes to oracle/_ref/ and is never shipped.
//
// usage: ref_harness etkf|letkf|enkf NX NY K ENS_PREFIX OBS_FILE ERROR
//                    INFLATION RADIUS OUT_DIR [SEED]
//        ref_harness nearest IN_FILE OUT_FILE   (see nearest::run)
//   reads ENS_PREFIX<i>.txt (i = 1..K, SimpleState text) and OBS_FILE
//   (GridObservation text format, grid coordinates); writes the analysed
//   members as raw little-endian doubles to OUT_DIR/member_<i>.bin
//   (i = 0..K-1) and Ensemble::Mean() to OUT_DIR/mean.bin.  For enkf, the
//   reference's std::random_device is replaced at compile time by a device
//   that returns SEED, so its std::mt19937 / std::normal_distribution draw a
//   reproducible sequence; the harness draws the same sequence again and
//   writes the perturbations it produced (obs-major, p x k) to
//   OUT_DIR/obs_pert.bin, and {||d||, background spread, analysis spread,
//   max gain, min gain} from getAnalysisResults() to OUT_DIR/enkf_diag.bin.
#include <random>

namespace harness {
inline unsigned int g_seed = 0;
}
namespace std {
// Stands in for std::random_device inside EnKF.hpp (see the macro below).
struct harness_seeded_device {
  using result_type = unsigned int;
  result_type operator()() { return harness::g_seed; }
};
}  // namespace std

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "harness_traits.hpp"

#include "Config.hpp"
#include "ETKF.hpp"
#include "Ensemble.hpp"
#include "Geometry.hpp"
#include "IdentityControlVariableBackend.hpp"
#include "LETKF.hpp"
#define random_device harness_seeded_device
#include "EnKF.hpp"
#undef random_device
#include "Logger.hpp"
#include "ObsOperator.hpp"
#include "Observation.hpp"
#include "IdentityObsOperator.hpp"
#include "PointObservation.hpp"

namespace fw = metada::framework;
using Tag = harness::HarnessBackendTag;

// ---- nearest-node mode: the reference's IdentityObsOperator::apply on a
// WRF-style geometry, reaching its geographic branch
// (convertGeographicToGrid, IdentityObsOperator.hpp:484-505 and the vertical
// search below it).  The state holds the node's linear index
// i + nx (j + ny k); at an exact node the 1e12 weight makes apply() return
// that index (the other neighbours add less than 1e-6), so the rounded
// result names the node the reference chose.
namespace nearest {

struct GridInfo {  // the members convertGeographicToGrid reads
  size_t nx = 0, ny = 0;
  std::vector<double> latitude_2d, longitude_2d, vertical_coords;
  bool has_2d_coords() const { return !latitude_2d.empty(); }
  bool has_vertical_coords() const { return !vertical_coords.empty(); }
};

struct Geometry {
  GridInfo info;
  const GridInfo& unstaggered_info() const { return info; }
  size_t x_dim() const { return info.nx; }
  size_t y_dim() const { return info.ny; }
  size_t z_dim() const { return info.vertical_coords.empty() ? 1 : info.vertical_coords.size(); }
  // The operator's generic fallback (not reached: the grid has 2-D coordinates).
  fw::Location getLocation(int i, int j, int) const {
    const size_t t = (size_t)j * info.nx + (size_t)i;
    return fw::Location(info.latitude_2d[t], info.longitude_2d[t], 0.0, fw::CoordinateSystem::GEOGRAPHIC);
  }
};

struct State {
  const Geometry* g;
  std::vector<double> data;
  const Geometry& geometry() const { return *g; }
  std::vector<double> getVariable(const std::string&) const { return data; }
};

using Obs = std::vector<fw::ObservationPoint>;
using Op = metada::backends::common::obsoperator::IdentityObsOperator<State, Obs, int>;

// IN: int64 nx, ny, nz, p; doubles lat2d[nx*ny], lon2d[nx*ny], vcoord[nz],
// obs_lat[p], obs_lon[p], obs_level[p].  OUT: int64 (i, j, k) per obs.
int run(const std::string& in, const std::string& out) {
  std::ifstream f(in, std::ios::binary);
  if (!f) throw std::runtime_error("cannot read " + in);
  int64_t hdr[4];
  f.read(reinterpret_cast<char*>(hdr), sizeof(hdr));
  const size_t nx = (size_t)hdr[0], ny = (size_t)hdr[1], nz = (size_t)hdr[2], p = (size_t)hdr[3];
  auto rd = [&](size_t n) {
    std::vector<double> v(n);
    f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(double)));
    return v;
  };
  Geometry geo;
  geo.info.nx = nx;
  geo.info.ny = ny;
  geo.info.latitude_2d = rd(nx * ny);
  geo.info.longitude_2d = rd(nx * ny);
  geo.info.vertical_coords = rd(nz);
  const auto olat = rd(p), olon = rd(p), olev = rd(p);
  if (!f) throw std::runtime_error("short input " + in);
  const size_t nzz = geo.z_dim();
  State st{&geo, std::vector<double>(nx * ny * nzz)};
  for (size_t t = 0; t < st.data.size(); ++t) st.data[t] = (double)t;
  Obs obs;
  for (size_t o = 0; o < p; ++o)
    obs.emplace_back(fw::Location(olat[o], olon[o], olev[o], fw::CoordinateSystem::GEOGRAPHIC), 0.0, 1.0);
  harness::MapConfig cfg(fw::ConfigMap{});
  Op op(cfg);
  const std::vector<double> h = op.apply(st, obs);
  std::vector<int64_t> ijk(3 * p);
  for (size_t o = 0; o < p; ++o) {
    const int64_t id = (int64_t)std::llround(h[o]);
    ijk[3 * o] = id % (int64_t)nx;
    ijk[3 * o + 1] = (id / (int64_t)nx) % (int64_t)ny;
    ijk[3 * o + 2] = id / (int64_t)(nx * ny);
  }
  std::ofstream fo(out, std::ios::binary);
  fo.write(reinterpret_cast<const char*>(ijk.data()), (std::streamsize)(ijk.size() * sizeof(int64_t)));
  return fo ? 0 : 1;
}

}  // namespace nearest

static void dump(const std::string& path, const double* p, size_t n) {
  std::ofstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot write " + path);
  f.write(reinterpret_cast<const char*>(p), (std::streamsize)(n * sizeof(double)));
}

int main(int argc, char** argv) {
  try {
    if (argc == 4 && std::string(argv[1]) == "nearest") return nearest::run(argv[2], argv[3]);
    if (argc != 11 && argc != 12) {
      std::cerr << "usage: ref_harness etkf|letkf|enkf NX NY K ENS_PREFIX OBS_FILE ERROR INFLATION "
                   "RADIUS OUT_DIR [SEED]\n";
      return 2;
    }
    if (argc == 12) harness::g_seed = (unsigned int)std::strtoul(argv[11], nullptr, 10);
    const std::string algo = argv[1];
    const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), k = std::atoi(argv[4]);
    const std::string ens_prefix = argv[5], obs_file = argv[6];
    const float error = std::strtof(argv[7], nullptr);
    const float inflation = std::strtof(argv[8], nullptr);
    const float radius = std::strtof(argv[9], nullptr);
    const std::string out = argv[10];

    fw::ConfigMap logger_cfg{{"app_name", fw::ConfigValue("ref_harness")},
                             {"level", fw::ConfigValue("error")},
                             {"color", fw::ConfigValue(false)},
                             {"show_timestamp", fw::ConfigValue(false)},
                             {"console", fw::ConfigValue(true)}};
    std::vector<fw::ConfigValue> members;
    for (int i = 1; i <= k; ++i) {
      fw::ConfigMap st{{"variables", fw::ConfigValue("simple")},
                       {"file", fw::ConfigValue(ens_prefix + std::to_string(i) + ".txt")}};
      members.emplace_back(fw::ConfigMap{{"state", fw::ConfigValue(st)}});
    }
    fw::ConfigMap var_cfg{{"if_use", fw::ConfigValue(true)},
                          {"error", fw::ConfigValue(error)},
                          {"missing_value", fw::ConfigValue(-999.0f)}};
    std::vector<fw::ConfigValue> vars{fw::ConfigValue(fw::ConfigMap{{"simple", var_cfg}})};
    fw::ConfigMap type_cfg{{"if_use", fw::ConfigValue(true)},
                           {"file", fw::ConfigValue(obs_file)},
                           {"coordinate", fw::ConfigValue("grid")},
                           {"variables", fw::ConfigValue(vars)}};
    std::vector<fw::ConfigValue> types{fw::ConfigValue(fw::ConfigMap{{"obs_A", type_cfg}})};
    fw::ConfigMap analysis{{"algorithm", fw::ConfigValue(algo)},
                           {"inflation", fw::ConfigValue(inflation)},
                           {"inflation_method", fw::ConfigValue("multiplicative")},
                           {"localization_radius", fw::ConfigValue(radius)},
                           {"format", fw::ConfigValue("txt")},
                           {"output_base_file", fw::ConfigValue(out + "/analysis")}};
    fw::ConfigMap root{
        {"logger", fw::ConfigValue(logger_cfg)},
        {"geometry",
         fw::ConfigValue(fw::ConfigMap{{"x_dim", fw::ConfigValue(nx)}, {"y_dim", fw::ConfigValue(ny)}})},
        {"ensemble", fw::ConfigValue(fw::ConfigMap{{"members", fw::ConfigValue(members)}})},
        {"observations", fw::ConfigValue(fw::ConfigMap{{"types", fw::ConfigValue(types)}})},
        {"obs_operator", fw::ConfigValue(fw::ConfigMap{})},
        {"analysis", fw::ConfigValue(analysis)}};

    fw::Config<Tag> config(root);
    fw::Config<Tag> log_config(logger_cfg);
    fw::Logger<Tag>::Init(log_config);

    fw::Geometry<Tag> geometry(config.GetSubsection("geometry"));
    fw::Config<Tag> ens_cfg = config.GetSubsection("ensemble");
    fw::Ensemble<Tag> ensemble(ens_cfg, geometry);
    fw::Observation<Tag> observations(config.GetSubsection("observations"));
    auto control = std::make_shared<fw::IdentityControlVariableBackend<Tag>>();
    fw::ObsOperator<Tag> obs_operator(config.GetSubsection("obs_operator"), *control);

    // Wall time of the policy's construction and Analyse() (inputs already
    // read), written to OUT_DIR/analyse_seconds.txt.
    const auto t0 = std::chrono::steady_clock::now();
    auto elapsed = [&]() { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); };
    double seconds = 0.0;
    if (algo == "etkf") {
      fw::ETKF<Tag> etkf(ensemble, observations, obs_operator, config.GetSubsection("analysis"));
      etkf.Analyse();
      seconds = elapsed();
    } else if (algo == "letkf") {
      fw::LETKF<Tag> letkf(ensemble, observations, obs_operator, config.GetSubsection("analysis"));
      letkf.Analyse();
      seconds = elapsed();
    } else if (algo == "enkf") {
      // EnKF reads the "analysis" subsection itself (EnKF.hpp:109).
      fw::EnKF<Tag> enkf(ensemble, observations, obs_operator, config);
      enkf.Analyse();
      seconds = elapsed();
      const auto r = enkf.getAnalysisResults();
      const double dg[5] = {r.innovation_norm, r.background_spread, r.analysis_spread, r.max_kalman_gain,
                            r.min_kalman_gain};
      dump(out + "/enkf_diag.bin", dg, 5);
      // The same draws as generateObservationPerturbations (EnKF.hpp:340-360)
      // with R = sigma^2 I (chol_L(R) = sigma I).
      const int p = (int)observations.size();
      std::mt19937 gen(harness::g_seed);
      std::normal_distribution<double> dist(0.0, 1.0);
      const auto cov = observations.getCovariance();
      std::vector<double> eps((size_t)p * k);
      for (int i = 0; i < p; ++i)
        for (int j = 0; j < k; ++j) eps[(size_t)i * k + j] = std::sqrt(cov[(size_t)i]) * dist(gen);
      dump(out + "/obs_pert.bin", eps.data(), eps.size());
    } else {
      throw std::runtime_error("unknown algorithm " + algo);
    }
    std::ofstream(out + "/analyse_seconds.txt") << std::setprecision(9) << seconds << "\n";
    const size_t n = ensemble.GetMember(0).size();
    for (int i = 0; i < k; ++i)
      dump(out + "/member_" + std::to_string(i) + ".bin",
           ensemble.GetMember(i).template getDataPtr<double>(), n);
    dump(out + "/mean.bin", ensemble.Mean().template getDataPtr<double>(), n);
    return 0;
  } catch (const std::exception& e) {
    std::cerr << "ref_harness failed: " << e.what() << std::endl;
    return 1;
  }
}

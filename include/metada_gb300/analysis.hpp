// Drop-in GPU analysis policies for METADA.
//
// metada_gb300::ETKF<Tag>, LETKF<Tag> and EnKF<Tag> (with Metrics<T>) keep the
// signature and
// behaviour of the reference policies (src/framework/algorithms/ETKF.hpp:76-210,
// LETKF.hpp:37-253): construct from (Ensemble&, Observation&, const
// ObsOperator&, const Config&), call Analyse(), then saveEnsemble().  A METADA
// application switches by changing one line, e.g. in
// applications/data_assimilation/ensemble/letkf.cpp:
//     metada_gb300::LETKF<BackendTag> letkf(ensemble, observations,
//                                           obs_operator, config.GetSubsection("analysis"));
// The adapters are used through the calls the reference policies make
// (Ensemble::Size/GetMember/RecomputeMean/Mean, State::getDataPtr<double>/
// size/geometry/saveToFile, Observation iteration + getObservationValues/
// getCovariance, ObsOperator::apply, Config::Get/HasKey), so any backend tag
// the reference accepts for these policies is accepted here.
//
// Config keys: the reference's (inflation, localization_radius,
// output_base_file, format; numbers read with asFloat() as the reference
// does) plus
//   precision: "fp64" (default) | "mixed"
//   semantics: "reference" (default) | "hunt"  (Gaspari-Cohn R-localisation,
//              symmetric square root)
//   order:     LETKF only, "sequential" (default: the reference's in-place
//              grid-point order) | "batched" (all analyses at once, background
//              obs-space prior)
//   obs_operator_on_device: "auto" (default: IDW4 on the GPU for grid
//              observations, the reference's IdentityObsOperator on
//              SimpleState) | "host" (the bound ObsOperator::apply on the
//              host, k calls; any operator)
//   vertical_radius: LETKF, levels (geographic observations with a level)
#pragma once

#include <cmath>
#include <cstdint>
#include <functional>
#include <iomanip>
#include <limits>
#include <memory>
#include <ostream>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "runtime.hpp"

namespace metada_gb300 {

namespace detail {

struct Settings {
  double inflation = 1.0;
  double radius = 0.0;
  double vertical_radius = 0.0;
  int precision = MG_PREC_FP64;
  int flags = MG_COMPAT;
  bool sequential = true;
  bool host_h = false;
  std::string output_base_file = "analysis";
  std::string format = "txt";
};

template <typename Cfg>
std::string cfg_string(const Cfg& c, const char* key, const std::string& def) {
  return c.HasKey(key) ? c.Get(key).asString() : def;
}

template <typename Cfg>
Settings read_settings(const Cfg& c, bool letkf) {
  Settings s;
  s.inflation = static_cast<double>(c.Get("inflation").asFloat());  // ETKF.hpp:91, LETKF.hpp:52
  if (letkf) s.radius = static_cast<double>(c.Get("localization_radius").asFloat());  // LETKF.hpp:53
  if (letkf && c.HasKey("vertical_radius")) s.vertical_radius = static_cast<double>(c.Get("vertical_radius").asFloat());
  s.output_base_file = cfg_string(c, "output_base_file", s.output_base_file);
  s.format = cfg_string(c, "format", letkf ? "nc" : "txt");
  const std::string prec = cfg_string(c, "precision", "fp64");
  if (prec != "fp64" && prec != "mixed") throw std::invalid_argument("precision must be fp64 or mixed");
  s.precision = prec == "fp64" ? MG_PREC_FP64 : MG_PREC_MIXED;
  const std::string sem = cfg_string(c, "semantics", "reference");
  if (sem != "reference" && sem != "hunt") throw std::invalid_argument("semantics must be reference or hunt");
  s.flags = sem == "reference" ? MG_COMPAT : 0;
  const std::string order = cfg_string(c, "order", "sequential");
  if (order != "sequential" && order != "batched") throw std::invalid_argument("order must be sequential or batched");
  s.sequential = letkf && order == "sequential";
  s.host_h = cfg_string(c, "obs_operator_on_device", "auto") == "host";
  return s;
}

// Observation values, variances and locations (LETKF.hpp:71-77, ETKF.hpp:139-147).
struct HostObs {
  bool grid = true;
  std::vector<int32_t> xy;
  std::vector<double> lat, lon, lev;
  std::vector<uint8_t> valid;
  std::vector<double> yo, rvar;
  size_t size() const { return yo.size(); }
};

template <typename Obs>
HostObs collect_obs(const Obs& obs) {
  HostObs h;
  h.yo = obs.getObservationValues();
  h.rvar = obs.getCovariance();
  bool any_grid = false, any_geo = false;
  for (const auto& pt : obs) {
    try {
      const auto xy = pt.location.getGridCoords2D();
      h.xy.push_back(static_cast<int32_t>(xy.first));
      h.xy.push_back(static_cast<int32_t>(xy.second));
      any_grid = true;
    } catch (const std::runtime_error&) {
      const auto geo = pt.location.getGeographicCoords();
      h.lat.push_back(std::get<0>(geo));
      h.lon.push_back(std::get<1>(geo));
      h.lev.push_back(std::get<2>(geo));
      any_geo = true;
    }
    h.valid.push_back(pt.is_valid ? 1 : 0);
  }
  if (any_grid && any_geo) throw std::runtime_error("observations mix grid and geographic locations");
  h.grid = !any_geo;
  if (h.valid.size() != h.yo.size()) throw std::runtime_error("observation count mismatch");
  return h;
}

// Grid or geographic coordinates of the analysis points, in state order
// (SimpleGeometry iterates y outer, x inner: the state index, SimpleGeometry.hpp:49-54).
struct HostGrid {
  bool grid = true;
  int nx = 0, ny = 0;
  std::vector<double> lat, lon;
};

template <typename Geom>
HostGrid collect_grid(const Geom& g) {
  HostGrid h;
  int64_t t = 0, maxx = -1, maxy = -1;
  std::vector<std::pair<int, int>> xy;
  for (const auto& loc : g) {
    try {
      const auto c = loc.getGridCoords2D();
      xy.push_back(c);
      if (c.first > maxx) maxx = c.first;
      if (c.second > maxy) maxy = c.second;
    } catch (const std::runtime_error&) {
      const auto geo = loc.getGeographicCoords();
      h.grid = false;
      h.lat.push_back(std::get<0>(geo));
      h.lon.push_back(std::get<1>(geo));
    }
    ++t;
  }
  if (h.grid) {
    h.nx = static_cast<int>(maxx + 1);
    h.ny = static_cast<int>(maxy + 1);
    if ((int64_t)h.nx * h.ny != t) throw std::runtime_error("grid geometry is not a full nx x ny grid");
    for (int64_t i = 0; i < t; ++i)
      if (xy[i].first != i % h.nx || xy[i].second != i / h.nx)
        throw std::runtime_error("grid geometry is not in row-major (y outer, x inner) order");
  }
  return h;
}

template <typename Ens>
void gather_members(Ens& ens, std::vector<double>& host, int k, size_t n) {
  host.resize((size_t)k * n);
  for (int i = 0; i < k; ++i) {
    const auto& m = ens.GetMember(i);
    if (m.size() != n) throw std::runtime_error("ensemble members differ in size");
    const double* d = m.template getDataPtr<double>();
    std::copy(d, d + n, host.begin() + (size_t)i * n);
  }
}

template <typename Ens>
void scatter_members(Ens& ens, const std::vector<double>& host, int k, size_t n) {
  for (int i = 0; i < k; ++i) {
    double* d = ens.GetMember(i).template getDataPtr<double>();
    std::copy(host.begin() + (size_t)i * n, host.begin() + (size_t)(i + 1) * n, d);
  }
}

// Members whose backend keeps its data on the device (DeviceState, the
// Gb300BackendTag state): the analysis reads and writes them device to device.
template <typename M>
concept DeviceMember = requires(M& m) {
  { m.backend().device_data() } -> std::convertible_to<double*>;
};

template <typename Ens>
constexpr bool device_members() {
  return DeviceMember<std::remove_reference_t<decltype(std::declval<Ens&>().GetMember(0))>>;
}

// Members into (from) the k x n member-major device matrix X: device copies
// when the members live on the device, else a host gather and one upload.
template <typename Ens>
void load_members(Ens& ens, DeviceBuffer<double>& X, std::vector<double>& host, int k, size_t n, cudaStream_t s) {
  if constexpr (device_members<Ens>()) {
    X.resize((size_t)k * n);
    for (int i = 0; i < k; ++i) {
      auto& m = ens.GetMember(i);
      if (m.size() != n) throw std::runtime_error("ensemble members differ in size");
      cuda_check(cudaMemcpyAsync(X.data() + (size_t)i * n, m.backend().device_data(), n * sizeof(double),
                                 cudaMemcpyDeviceToDevice, s),
                 "member gather");
    }
  } else {
    gather_members(ens, host, k, n);
    X.upload(host, s);
  }
}

template <typename Ens>
void store_members(Ens& ens, const DeviceBuffer<double>& X, std::vector<double>& host, int k, size_t n,
                   cudaStream_t s) {
  if constexpr (device_members<Ens>()) {
    for (int i = 0; i < k; ++i)
      cuda_check(cudaMemcpyAsync(ens.GetMember(i).backend().device_data(), X.data() + (size_t)i * n,
                                 n * sizeof(double), cudaMemcpyDeviceToDevice, s),
                 "member scatter");
    cuda_check(cudaStreamSynchronize(s), "member scatter sync");
  } else {
    host.resize((size_t)k * n);
    X.download(host.data(), host.size(), s);
    scatter_members(ens, host, k, n);
  }
}

// HX (p x k) for the raw members: on the device (IDW4 for grid obs) or via
// the bound operator on the host (ETKF.hpp:128-132).
template <typename Ens, typename Obs, typename H>
void obs_space(Context& ctx, Ens& ens, const Obs& obs, const H& op, const HostObs& ho, const HostGrid* grid,
               const DeviceBuffer<double>& X, int k, size_t n, bool host_h, DeviceBuffer<double>& HX) {
  const size_t p = ho.size();
  if (!host_h && ho.grid && grid && grid->grid) {
    DeviceBuffer<int32_t> xy;
    DeviceBuffer<uint8_t> valid;
    xy.upload(ho.xy, ctx.stream());
    valid.upload(ho.valid, ctx.stream());
    HX.resize(p * k);
    ctx.check(mg_hx_idw4(ctx.get(), X.data(), k, (int64_t)n, grid->nx, grid->ny, xy.data(), valid.data(),
                         (int64_t)p, HX.data()),
              "mg_hx_idw4");
    ctx.synchronize();
    return;
  }
  std::vector<double> hx(p * k);
  for (int i = 0; i < k; ++i) {
    const std::vector<double> y = op.apply(ens.GetMember(i), obs);
    if (y.size() != p) throw std::runtime_error("ObsOperator::apply returned the wrong size");
    for (size_t o = 0; o < p; ++o) hx[o * k + i] = y[o];
  }
  HX.upload(hx, ctx.stream());
}

}  // namespace detail

// Global ETKF on the GPU (ETKF.hpp:76-210).
template <typename BackendTag>
class ETKF {
 public:
  template <typename Ens, typename Obs, typename H, typename Cfg>
  ETKF(Ens& ensemble, Obs& obs, const H& obs_op, const Cfg& config, int device = 0)
      : settings_(detail::read_settings(config, false)), ctx_(std::make_shared<Context>(device)) {
    analyse_ = [this, &ensemble, &obs, &obs_op]() { run(ensemble, obs, obs_op); };
    save_ = [this, &ensemble]() { save(ensemble); };
  }

  void Analyse() { analyse_(); }
  void saveEnsemble() const { save_(); }

 private:
  template <typename Ens, typename Obs, typename H>
  void run(Ens& ens, Obs& obs, const H& op) {
    const int k = static_cast<int>(ens.Size());
    const size_t n = ens.GetMember(0).size();
    // Ensemble::Mean() keeps the background mean, as the reference leaves it
    // (ETKF.hpp:111-112, 190-191).
    ens.RecomputeMean();
    std::vector<double> host;
    DeviceBuffer<double> X, HX, yo, rvar;
    detail::load_members(ens, X, host, k, n, ctx_->stream());
    const detail::HostObs ho = detail::collect_obs(obs);
    detail::HostGrid grid;
    const bool have_grid = ho.grid && ens.GetMember(0).geometry() != nullptr;
    if (have_grid) grid = detail::collect_grid(*ens.GetMember(0).geometry());
    detail::obs_space(*ctx_, ens, obs, op, ho, have_grid ? &grid : nullptr, X, k, n, settings_.host_h, HX);
    yo.upload(ho.yo, ctx_->stream());
    rvar.upload(ho.rvar, ctx_->stream());
    ctx_->check(mg_etkf(ctx_->get(), X.data(), (int64_t)n, k, (int64_t)n, HX.data(), yo.data(), rvar.data(),
                        (int64_t)ho.size(), settings_.inflation, settings_.flags, settings_.precision, nullptr),
                "mg_etkf");
    detail::store_members(ens, X, host, k, n, ctx_->stream());
  }

  template <typename Ens>
  void save(Ens& ens) const {  // ETKF.hpp:185-200
    ens.Mean().saveToFile(settings_.output_base_file + "_mean." + settings_.format);
    for (size_t i = 0; i < ens.Size(); ++i)
      ens.GetMember(i).saveToFile(settings_.output_base_file + "_member_" + std::to_string(i) + "." +
                                  settings_.format);
  }

  detail::Settings settings_;
  std::shared_ptr<Context> ctx_;
  std::function<void()> analyse_;
  std::function<void()> save_;
};

// Local ETKF on the GPU (LETKF.hpp:37-253).
template <typename BackendTag>
class LETKF {
 public:
  template <typename Ens, typename Obs, typename H, typename Cfg>
  LETKF(Ens& ensemble, Obs& obs, const H& obs_op, const Cfg& config, int device = 0)
      : settings_(detail::read_settings(config, true)), ctx_(std::make_shared<Context>(device)) {
    analyse_ = [this, &ensemble, &obs, &obs_op]() { run(ensemble, obs, obs_op); };
    save_ = [this, &ensemble]() { save(ensemble); };
  }

  void Analyse() { analyse_(); }
  void saveEnsemble() const { save_(); }
  const mg_letkf_stats& stats() const { return stats_; }

 private:
  template <typename Ens, typename Obs, typename H>
  void run(Ens& ens, Obs& obs, const H& op) {
    const int k = static_cast<int>(ens.Size());
    const size_t n = ens.GetMember(0).size();
    const auto* geometry = ens.GetMember(0).geometry();
    if (!geometry) throw std::runtime_error("Geometry pointer is null in LETKF");  // LETKF.hpp:81-83
    const detail::HostGrid grid = detail::collect_grid(*geometry);
    const detail::HostObs ho = detail::collect_obs(obs);
    const size_t npt = grid.grid ? (size_t)grid.nx * grid.ny : grid.lat.size();
    if (npt != n) throw std::runtime_error("LETKF: one state value per geometry point is required");
    std::vector<double> host;
    DeviceBuffer<double> X, yo, rvar;
    detail::load_members(ens, X, host, k, n, ctx_->stream());
    yo.upload(ho.yo, ctx_->stream());
    rvar.upload(ho.rvar, ctx_->stream());
    const int64_t p = (int64_t)ho.size();
    if (settings_.sequential) {
      if (!grid.grid || !ho.grid || settings_.flags != MG_COMPAT || settings_.precision != MG_PREC_FP64)
        throw std::invalid_argument("order=sequential is the reference LETKF: grid geometry and obs, "
                                    "reference semantics, fp64");
      DeviceBuffer<int32_t> xy;
      DeviceBuffer<uint8_t> valid;
      xy.upload(ho.xy, ctx_->stream());
      valid.upload(ho.valid, ctx_->stream());
      ctx_->check(mg_letkf_compat_grid(ctx_->get(), X.data(), k, (int64_t)n, grid.nx, grid.ny, xy.data(),
                                       valid.data(), yo.data(), p, settings_.radius, settings_.inflation, nullptr),
                  "mg_letkf_compat_grid");
    } else {
      DeviceBuffer<double> HX;
      detail::obs_space(*ctx_, ens, obs, op, ho, &grid, X, k, n, settings_.host_h, HX);
      DeviceBuffer<int64_t> off;
      DeviceBuffer<int32_t> idx;
      DeviceBuffer<double> dist, olev;
      int64_t total = 0;
      off.resize(npt + 1);
      if (grid.grid && ho.grid) {
        DeviceBuffer<int32_t> xy;
        xy.upload(ho.xy, ctx_->stream());
        const int rc = mg_select_grid(ctx_->get(), grid.nx, grid.ny, xy.data(), p, settings_.radius, off.data(),
                                      nullptr, 0, &total);
        if (rc != MG_OK && rc != MG_ERR_CAPACITY) ctx_->check(rc, "mg_select_grid");
        idx.resize(total + 1);
        ctx_->check(mg_select_grid(ctx_->get(), grid.nx, grid.ny, xy.data(), p, settings_.radius, off.data(),
                                   idx.data(), total + 1, &total),
                    "mg_select_grid");
      } else if (!grid.grid && !ho.grid) {
        DeviceBuffer<double> clat, clon, olat, olon;
        clat.upload(grid.lat, ctx_->stream());
        clon.upload(grid.lon, ctx_->stream());
        olat.upload(ho.lat, ctx_->stream());
        olon.upload(ho.lon, ctx_->stream());
        const int rc = mg_select_geo(ctx_->get(), clat.data(), clon.data(), (int64_t)npt, olat.data(),
                                     olon.data(), p, settings_.radius, off.data(), nullptr, nullptr, 0, &total);
        if (rc != MG_OK && rc != MG_ERR_CAPACITY) ctx_->check(rc, "mg_select_geo");
        idx.resize(total + 1);
        dist.resize(total + 1);
        ctx_->check(mg_select_geo(ctx_->get(), clat.data(), clon.data(), (int64_t)npt, olat.data(), olon.data(),
                                  p, settings_.radius, off.data(), idx.data(), dist.data(), total + 1, &total),
                    "mg_select_geo");
      } else {
        throw std::runtime_error("Cannot compute distance between incompatible Location coordinate systems");
      }
      DeviceBuffer<int64_t> col_base;
      std::vector<int64_t> cb(npt);
      for (size_t i = 0; i < npt; ++i) cb[i] = (int64_t)i;
      col_base.upload(cb, ctx_->stream());
      mg_letkf_desc d{};
      d.X = X.data();
      d.n = (int64_t)n;
      d.ld = (int64_t)n;
      d.k = k;
      d.n_var = 1;
      d.nlev = 1;
      d.precision = settings_.precision;
      d.ncol = (int64_t)npt;
      d.col_base = col_base.data();
      d.p = p;
      d.HX = HX.data();
      d.yo = yo.data();
      d.rvar = rvar.data();
      d.loc_off = off.data();
      d.loc_idx = idx.data();
      d.loc_dist = dist.size() ? dist.data() : nullptr;
      d.hsupport = settings_.radius;
      d.vsupport = settings_.vertical_radius;
      d.rho = settings_.inflation;
      d.flags = settings_.flags;
      ctx_->check(mg_letkf_batched(ctx_->get(), &d), "mg_letkf_batched");
      ctx_->check(mg_letkf_last_stats(ctx_->get(), &stats_), "mg_letkf_last_stats");
    }
    detail::store_members(ens, X, host, k, n, ctx_->stream());
    ens.RecomputeMean();  // LETKF.hpp:116
  }

  template <typename Ens>
  void save(Ens& ens) const {  // LETKF.hpp:125-142
    ens.Mean().saveToFile(settings_.output_base_file + "_mean." + settings_.format);
    for (size_t i = 0; i < ens.Size(); ++i)
      ens.GetMember(i).saveToFile(settings_.output_base_file + "_member_" + std::to_string(i) + "." +
                                  settings_.format);
  }

  detail::Settings settings_;
  std::shared_ptr<Context> ctx_;
  mg_letkf_stats stats_{};
  std::function<void()> analyse_;
  std::function<void()> save_;
};

// Stochastic EnKF with perturbed observations on the GPU (EnKF.hpp:66-254).
// Constructed like the reference from the root configuration (it reads the
// "analysis" subsection itself, EnKF.hpp:109): inflation, inflation_method,
// output_base_file, format, plus precision and seed.  The perturbations are
// chol_L(R) z with z drawn obs-major from std::mt19937 and
// std::normal_distribution<double> as generateObservationPerturbations
// draws them (:340-360); the generator is seeded with "seed" when given
// (the reference seeds it from std::random_device, which is what happens
// here without the key), so a run with seed s reproduces the reference run
// whose random_device returned s.  The update runs in the k-dimensional
// form (mg_enkf): the gain's max/min and the condition number of S, which
// need the n x p gain or the p x p S, are reported as NaN.
template <typename BackendTag>
class EnKF {
 public:
  struct AnalysisResults {  // EnKF.hpp:84-96
    double innovation_norm;
    double analysis_increment_norm;
    double background_spread;
    double analysis_spread;
    double max_kalman_gain;
    double min_kalman_gain;
    double condition_number;
    int ensemble_size;
    int observation_count;
    std::string inflation_method;
    double inflation_factor;
  };

  template <typename Ens, typename Obs, typename H, typename Cfg>
  EnKF(Ens& ensemble, Obs& obs, const H& obs_op, const Cfg& config, int device = 0)
      : ctx_(std::make_shared<Context>(device)) {
    const auto a = config.GetSubsection("analysis");
    settings_.inflation = static_cast<double>(a.Get("inflation").asFloat());
    settings_.output_base_file = a.Get("output_base_file").asString();
    settings_.format = a.Get("format").asString();
    method_ = a.Get("inflation_method").asString();
    if (method_ != "multiplicative" && method_ != "additive" && method_ != "relaxation") method_ = "multiplicative";
    const std::string prec = detail::cfg_string(a, "precision", "fp64");
    if (prec != "fp64" && prec != "mixed") throw std::invalid_argument("precision must be fp64 or mixed");
    settings_.precision = prec == "fp64" ? MG_PREC_FP64 : MG_PREC_MIXED;
    settings_.host_h = detail::cfg_string(a, "obs_operator_on_device", "auto") == "host";
    has_seed_ = a.HasKey("seed");
    if (has_seed_) seed_ = static_cast<unsigned int>(a.Get("seed").asInt());
    analyse_ = [this, &ensemble, &obs, &obs_op]() { run(ensemble, obs, obs_op); };
    save_ = [this, &ensemble]() { save(ensemble); };
  }

  void Analyse() { analyse_(); }
  void saveEnsemble() const { save_(); }
  AnalysisResults getAnalysisResults() const { return results_; }

 private:
  template <typename Ens, typename Obs, typename H>
  void run(Ens& ens, Obs& obs, const H& op) {
    const int k = static_cast<int>(ens.Size());
    const size_t n = ens.GetMember(0).size();
    std::vector<double> host;
    DeviceBuffer<double> X, HX, yo, rvar, E, Xb;
    detail::load_members(ens, X, host, k, n, ctx_->stream());
    Xb.resize(X.size());
    cuda_check(cudaMemcpyAsync(Xb.data(), X.data(), X.size() * sizeof(double), cudaMemcpyDeviceToDevice,
                               ctx_->stream()),
               "background copy");
    const detail::HostObs ho = detail::collect_obs(obs);
    detail::HostGrid grid;
    const bool have_grid = ho.grid && ens.GetMember(0).geometry() != nullptr;
    if (have_grid) grid = detail::collect_grid(*ens.GetMember(0).geometry());
    const size_t p = ho.size();
    std::vector<double> eps(p * (size_t)k);
    {
      unsigned int s = seed_;
      if (!has_seed_) {
        std::random_device rd;
        s = rd();
      }
      std::mt19937 gen(s);
      std::normal_distribution<double> dist(0.0, 1.0);
      for (size_t o = 0; o < p; ++o) {
        const double sd = std::isfinite(ho.rvar[o]) ? std::sqrt(ho.rvar[o]) : 0.0;
        for (int j = 0; j < k; ++j) eps[o * k + j] = sd * dist(gen);
      }
    }
    detail::obs_space(*ctx_, ens, obs, op, ho, have_grid ? &grid : nullptr, X, k, n, settings_.host_h, HX);
    yo.upload(ho.yo, ctx_->stream());
    rvar.upload(ho.rvar, ctx_->stream());
    E.upload(eps, ctx_->stream());
    mg_enkf_diag d{};
    ctx_->check(mg_enkf(ctx_->get(), X.data(), (int64_t)n, k, (int64_t)n, HX.data(), yo.data(), rvar.data(),
                        E.data(), (int64_t)p, settings_.inflation, settings_.precision, nullptr, &d),
                "mg_enkf");
    // analysis increment norm on the device: || X_a - X_b ||
    ctx_->check(mg_vec_update(ctx_->get(), Xb.data(), X.data(), (int64_t)X.size(), 1), "mg_vec_update");
    double inc = 0.0;
    ctx_->check(mg_vec_dot(ctx_->get(), Xb.data(), Xb.data(), (int64_t)Xb.size(), &inc), "mg_vec_dot");
    detail::store_members(ens, X, host, k, n, ctx_->stream());
    ens.RecomputeMean();  // EnKF.hpp:237-238
    ens.RecomputePerturbations();
    const double nan = std::numeric_limits<double>::quiet_NaN();
    results_ = AnalysisResults{d.innovation_norm, std::sqrt(inc), d.background_spread, d.analysis_spread, nan, nan,
                               nan, k, (int)p, method_, settings_.inflation};
  }

  template <typename Ens>
  void save(Ens& ens) const {  // EnKF.hpp:260-278
    ens.Mean().saveToFile(settings_.output_base_file + "_mean." + settings_.format);
    for (size_t i = 0; i < ens.Size(); ++i)
      ens.GetMember(i).saveToFile(settings_.output_base_file + "_member_" + std::to_string(i) + "." +
                                  settings_.format);
  }

  detail::Settings settings_;
  std::string method_;
  bool has_seed_ = false;
  unsigned int seed_ = 0;
  std::shared_ptr<Context> ctx_;
  AnalysisResults results_{};
  std::function<void()> analyse_;
  std::function<void()> save_;
};

// Ensemble diagnostics on the GPU with the reference's interface
// (Metrics.hpp:22-295): MetricValues and Metrics<T>::CalculateAll over
// member vectors.
template <typename T = double>
struct MetricValues {
  std::vector<T> mean;
  std::vector<T> spread;
  T rmse;
  T bias;
  T correlation;
  T crps;
  T avg_spread;

  std::string ToString(int precision = 6) const {  // Metrics.hpp:35-45
    std::stringstream ss;
    ss << std::fixed << std::setprecision(precision);
    ss << "Metrics:\n";
    ss << "  RMSE: " << rmse << "\n";
    ss << "  Bias: " << bias << "\n";
    ss << "  Correlation: " << correlation << "\n";
    ss << "  CRPS: " << crps << "\n";
    ss << "  Average Spread: " << avg_spread << "\n";
    return ss.str();
  }
  friend std::ostream& operator<<(std::ostream& os, const MetricValues<T>& m) { return os << m.ToString(); }
};

template <typename T = double>
class Metrics {
 public:
  static MetricValues<T> CalculateAll(const std::vector<std::vector<T>>& ensemble_data, const std::vector<T>& truth,
                                      size_t state_dim, size_t ens_size, int device = 0) {
    static_assert(sizeof(T) == sizeof(double), "the GPU diagnostics run in double precision");
    Context ctx(device);
    std::vector<double> host(ens_size * state_dim);
    for (size_t j = 0; j < ens_size; ++j)
      for (size_t i = 0; i < state_dim; ++i) host[j * state_dim + i] = static_cast<double>(ensemble_data[j][i]);
    std::vector<double> tr(truth.begin(), truth.begin() + state_dim);
    DeviceBuffer<double> X, t, mean, spread;
    X.upload(host, ctx.stream());
    t.upload(tr, ctx.stream());
    mean.resize(state_dim);
    spread.resize(state_dim);
    mg_ens_metrics_t out{};
    ctx.check(mg_ens_metrics(ctx.get(), X.data(), (int64_t)state_dim, (int32_t)ens_size, (int64_t)state_dim,
                             t.data(), mean.data(), spread.data(), &out),
              "mg_ens_metrics");
    MetricValues<T> v;
    v.mean.resize(state_dim);
    v.spread.resize(state_dim);
    std::vector<double> hm(state_dim), hs(state_dim);
    mean.download(hm.data(), state_dim, ctx.stream());
    spread.download(hs.data(), state_dim, ctx.stream());
    for (size_t i = 0; i < state_dim; ++i) {
      v.mean[i] = static_cast<T>(hm[i]);
      v.spread[i] = static_cast<T>(hs[i]);
    }
    v.rmse = out.rmse;
    v.bias = out.bias;
    v.correlation = out.correlation;
    v.crps = out.crps;
    v.avg_spread = out.avg_spread;
    return v;
  }
};

}  // namespace metada_gb300

// Compile check: metada_gb300::LETKF / ETKF / EnKF / Metrics instantiated with the REFERENCE's
// own adapter types (framework::Ensemble/Observation/ObsOperator/Config over
// the Simple backend, GridObservation and IdentityObsOperator), exactly as
// applications/data_assimilation/ensemble/letkf.cpp:46-65 builds them.  Built
// on the host by tests/test_cpp_dropin.py when the reference tree is
// present; it proves the policies are a type-correct drop-in.  Running it
// needs a GPU and the reference data files.
#include "harness_traits.hpp"

#include "Config.hpp"
#include "Ensemble.hpp"
#include "Geometry.hpp"
#include "IdentityControlVariableBackend.hpp"
#include "Logger.hpp"
#include "ObsOperator.hpp"
#include "Observation.hpp"
#include "metada_gb300/analysis.hpp"

namespace fw = metada::framework;
using Tag = harness::HarnessBackendTag;

int run(const fw::ConfigMap& root, const fw::ConfigMap& logger_cfg) {
  fw::Config<Tag> config(root);
  fw::Config<Tag> log_config(logger_cfg);
  fw::Logger<Tag>::Init(log_config);
  fw::Geometry<Tag> geometry(config.GetSubsection("geometry"));
  fw::Config<Tag> ens_cfg = config.GetSubsection("ensemble");
  fw::Ensemble<Tag> ensemble(ens_cfg, geometry);
  fw::Observation<Tag> observations(config.GetSubsection("observations"));
  auto control = std::make_shared<fw::IdentityControlVariableBackend<Tag>>();
  fw::ObsOperator<Tag> obs_operator(config.GetSubsection("obs_operator"), *control);
  // The one-line switch from fw::LETKF<Tag> / fw::ETKF<Tag>:
  metada_gb300::LETKF<Tag> letkf(ensemble, observations, obs_operator, config.GetSubsection("analysis"));
  letkf.Analyse();
  letkf.saveEnsemble();
  metada_gb300::ETKF<Tag> etkf(ensemble, observations, obs_operator, config.GetSubsection("analysis"));
  etkf.Analyse();
  etkf.saveEnsemble();
  // fw::EnKF<Tag> takes the root configuration (EnKF.hpp:100-109).
  metada_gb300::EnKF<Tag> enkf(ensemble, observations, obs_operator, config);
  enkf.Analyse();
  enkf.saveEnsemble();
  const auto results = enkf.getAnalysisResults();
  // Metrics<double>::CalculateAll over member vectors (Metrics.hpp:74-94).
  std::vector<std::vector<double>> data;
  for (size_t i = 0; i < ensemble.Size(); ++i) {
    const auto& m = ensemble.GetMember(i);
    const double* d = m.template getDataPtr<double>();
    data.emplace_back(d, d + m.size());
  }
  const auto mv = metada_gb300::Metrics<>::CalculateAll(data, data[0], data[0].size(), data.size());
  return (results.ensemble_size > 0 && mv.rmse >= 0.0) ? 0 : 1;
}

int main(int argc, char**) { return argc > 100 ? run({}, {}) : 0; }

// Compile check: metada_gb300::LETKF / ETKF instantiated with the REFERENCE's
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
  return 0;
}

int main(int argc, char**) { return argc > 100 ? run({}, {}) : 0; }

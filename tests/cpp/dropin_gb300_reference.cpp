// Compile check of the Gb300BackendTag backend set with the REFERENCE's own
// adapter types: framework::Ensemble / State / Geometry / Observation /
// ObsOperator / Config over metada_gb300::DeviceState (the device-resident
// state), the Simple geometry, GridObservation and IdentityObsOperator, and
// the GPU policies instantiated for that tag, as
// applications/data_assimilation/ensemble/letkf.cpp:46-65 builds them.  Built
// on the host by tests/test_cpp_dropin.py when the reference tree is
// present.  The reference tree does not exist where the GPU runs, so the
// executed GPU run of this backend is tests/cpp/dropin_device.cpp.
#include "harness_traits.hpp"
#define METADA_GB300_CONFIG_BACKEND harness::MapConfig
#include "metada_gb300/gb300_backend_traits.hpp"

#include "Config.hpp"
#include "Ensemble.hpp"
#include "Geometry.hpp"
#include "IdentityControlVariableBackend.hpp"
#include "Logger.hpp"
#include "ObsOperator.hpp"
#include "Observation.hpp"
#include "StateConcepts.hpp"
#include "metada_gb300/analysis.hpp"

namespace fw = metada::framework;
using Tag = metada_gb300::Gb300BackendTag;
using Geom = metada::backends::simple::SimpleGeometry;

// The reference's state concept (StateConcepts.hpp:47-84) holds for the device state.
static_assert(fw::StateBackendImpl<metada_gb300::DeviceState<Geom>, harness::MapConfig, Geom>);
static_assert(metada_gb300::detail::DeviceMember<fw::State<Tag>>);

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
  metada_gb300::LETKF<Tag> letkf(ensemble, observations, obs_operator, config.GetSubsection("analysis"));
  letkf.Analyse();
  letkf.saveEnsemble();
  metada_gb300::ETKF<Tag> etkf(ensemble, observations, obs_operator, config.GetSubsection("analysis"));
  etkf.Analyse();
  metada_gb300::EnKF<Tag> enkf(ensemble, observations, obs_operator, config);
  enkf.Analyse();
  return ensemble.Mean().size() > 0 ? 0 : 1;
}

int main(int argc, char**) { return argc > 100 ? run({}, {}) : 0; }

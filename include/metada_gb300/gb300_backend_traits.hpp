// Backend tag for METADA with the state kept on the GB300.
//
// Gb300BackendTag binds the backend set of SimpleBackendTag
// (src/traits/SimpleBackendTraits.hpp:52-99) with one change: the state
// backend is metada_gb300::DeviceState<SimpleGeometry>, whose data live in
// device memory (the analysis policies of analysis.hpp read and write the
// members there, Ensemble::RecomputeMean runs on the device, saveToFile
// formats on the device).  Geometry, observations and the observation
// operator are the reference's own.  An application selects it with
//     using BackendTag = metada_gb300::Gb300BackendTag;
// (applications/data_assimilation/ensemble/letkf.cpp:28) and the policies
// metada_gb300::LETKF<BackendTag> etc.
//
// This header includes the reference's backend headers, so the reference's
// src/ directories must be on the include path (as for SimpleBackendTraits).
#pragma once

#include "BackendTraits.hpp"
#include "ConsoleLogger.hpp"
#include "GridObservation.hpp"
#include "IdentityObsOperator.hpp"
#include "SimpleBackgroundErrorCovariance.hpp"
#include "SimpleGeometry.hpp"
#include "SimpleGeometryIterator.hpp"
#include "SimpleIncrement.hpp"
#include "SimpleModel.hpp"
#include "device_state.hpp"

namespace metada_gb300 {

struct Gb300BackendTag {};

}  // namespace metada_gb300

namespace metada::traits {

template <typename ConfigBackendT>
struct Gb300BackendTraitsFor {
  using ConfigBackend = ConfigBackendT;
  using LoggerBackend = backends::logger::ConsoleLogger<ConfigBackend>;
  using GeometryBackend = backends::simple::SimpleGeometry;
  using GeometryIteratorBackend =
      backends::simple::SimpleGeometryIterator<typename GeometryBackend::const_iterator>;
  using StateBackend = metada_gb300::DeviceState<GeometryBackend>;
  using IncrementBackend = backends::simple::SimpleIncrement;
  using ControlVariableBackend = backends::simple::SimpleIncrement;
  using ObservationBackend = backends::common::observation::GridObservation;
  using ObservationIteratorBackend = backends::common::observation::GridObservationIterator;
  using ObsOperatorBackend =
      backends::common::obsoperator::IdentityObsOperator<StateBackend, ObservationBackend, ControlVariableBackend>;
  using ModelBackend = backends::simple::SimpleModel;
  using BackgroundErrorCovarianceBackend = backends::simple::SimpleBackgroundErrorCovariance;
};

#ifdef METADA_GB300_CONFIG_BACKEND
// The application names its configuration backend (the reference's default
// is YamlConfig, SimpleBackendTraits.hpp:54-61).
template <>
struct BackendTraits<metada_gb300::Gb300BackendTag> : Gb300BackendTraitsFor<METADA_GB300_CONFIG_BACKEND> {};
#endif

}  // namespace metada::traits

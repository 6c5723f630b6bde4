// Stub of kalypsso-core's viscosity parameters for the functor bridge ([viscosity] enabled, mu,
// hancock_predictor_enabled).
#pragma once
#include <kalypsso/core/real_type.h>
#include <kalypsso/utils/config/ConfigMap.h>

namespace kalypsso
{
struct ViscosityParams
{
  bool   enabled = false;
  real_t mu = 0;
  bool   hancock_predictor_enabled = false;
  ViscosityParams() = default;
  explicit ViscosityParams(ConfigMap const & cm)
    : enabled(cm.getBool("viscosity", "enabled", false))
    , mu(cm.getReal("viscosity", "mu", 0.0))
    , hancock_predictor_enabled(cm.getBool("viscosity", "hancock_predictor_enabled", false))
  {}
};
} // namespace kalypsso

// Stub of kalypsso-core's time-integrator selection for the functor bridge ([amr] time_integrator).
#pragma once
#include <enum.h>
#include <kalypsso/utils/config/ConfigMap.h>

namespace kalypsso
{
BETTER_ENUM(TimeIntegrator, int, HANCOCK, RK2_SSP, RK3_SSP)
struct TimeIntegratorConfig
{
  static TimeIntegrator
  get_time_integrator(ConfigMap const & cm)
  {
    return cm.getString("amr", "time_integrator", "HANCOCK") == "RK2_SSP" ? +TimeIntegrator::RK2_SSP
                                                                           : +TimeIntegrator::HANCOCK;
  }
};
} // namespace kalypsso

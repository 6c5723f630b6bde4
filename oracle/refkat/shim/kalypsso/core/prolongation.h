// Stub of kalypsso-core's prolongation settings for the functor bridge: [amr]
// cell_centered_prolongation_type, SIMPLE_COPY (default) or EXTRAPOLATE_LINEAR_MINMOD.
#pragma once
#include <string>

#include <enum.h>
#include <kalypsso/utils/config/ConfigMap.h>

namespace kalypsso
{
BETTER_ENUM(CellCenteredProlongationType, int, SIMPLE_COPY, EXTRAPOLATE_LINEAR_MINMOD)

struct ProlongationParam
{
  CellCenteredProlongationType m_cell = CellCenteredProlongationType::SIMPLE_COPY;
  ProlongationParam() = default;
  explicit ProlongationParam(ConfigMap const & cm)
  {
    const std::string v = cm.getString("amr", "cell_centered_prolongation_type", "SIMPLE_COPY");
    if (v == "EXTRAPOLATE_LINEAR_MINMOD")
      m_cell = CellCenteredProlongationType::EXTRAPOLATE_LINEAR_MINMOD;
  }
};
} // namespace kalypsso

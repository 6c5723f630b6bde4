// Stub of kalypsso-core's uniform gravity field for the functor bridge ([gravity] uniform_g*).
#pragma once
#include <kalypsso/core/kokkos_shared.h>
#include <kalypsso/utils/config/ConfigMap.h>

namespace kalypsso
{
template <std::size_t dim>
using UniformGravityField = Kokkos::Array<real_t, dim>;
template <std::size_t dim>
UniformGravityField<dim>
get_uniform_gravity_vector(ConfigMap const & cm)
{
  UniformGravityField<dim> g;
  const char * key[3] = {"uniform_gx", "uniform_gy", "uniform_gz"};
  for (std::size_t d = 0; d < dim; ++d)
    g[d] = cm.getReal("gravity", key[d], 0.0);
  return g;
}
} // namespace kalypsso

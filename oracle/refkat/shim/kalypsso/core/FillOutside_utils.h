// Stub of kalypsso-core's border-condition configuration for FillOutsideCellFunctor: brick sizes and
// periodicity ([p4est_connectivity] nbrick_x/y/z, periodic_x/y/z) and one border condition per domain
// face ([border_conditions] xmin, xmax, ymin, ymax, zmin, zmax: NONE, PERIODIC, ZERO_GRADIENT, WALL,
// CUSTOM), read from the config map.
#pragma once
#include <string>

#include <kalypsso/core/kokkos_shared.h>
#include <kalypsso/core/kalypsso_data_container.h>
#include <kalypsso/utils/config/ConfigMap.h>

namespace kalypsso
{
struct ParallelEnv;

template <std::size_t dim>
brick_size_t<dim>
get_brick_sizes(ConfigMap const & cm)
{
  brick_size_t<dim> b;
  const char *      k[3] = {"nbrick_x", "nbrick_y", "nbrick_z"};
  for (std::size_t a = 0; a < dim; ++a)
    b[a] = cm.getInteger("p4est_connectivity", k[a], 1);
  return b;
}
template <std::size_t dim>
Kokkos::Array<bool, dim>
get_brick_periodicity(ConfigMap const & cm)
{
  Kokkos::Array<bool, dim> p;
  const char *             k[3] = {"periodic_x", "periodic_y", "periodic_z"};
  for (std::size_t a = 0; a < dim; ++a)
    p[a] = cm.getInteger("p4est_connectivity", k[a], 1) != 0;
  return p;
}
template <std::size_t dim>
constexpr Kokkos::Array<bool, dim>
get_bool_array(bool v)
{
  Kokkos::Array<bool, dim> a{};
  for (std::size_t i = 0; i < dim; ++i)
    a.m_data[i] = v;
  return a;
}

template <class BC>
struct BorderConditionsConfig
{
  template <std::size_t dim>
  using bc_array_t = Kokkos::Array<BC, 2 * dim>;

  template <std::size_t dim>
  static bc_array_t<dim>
  read_border_condition(ConfigMap const & cm, ParallelEnv const &)
  {
    const char * k[6] = {"xmin", "xmax", "ymin", "ymax", "zmin", "zmax"};
    bc_array_t<dim> out{BC::NONE, BC::NONE, BC::NONE, BC::NONE};
    for (std::size_t f = 0; f < 2 * dim; ++f)
    {
      const std::string v = cm.getString("border_conditions", k[f], "PERIODIC");
      const auto        e = BC::_from_string_nothrow(v.c_str());
      out[f] = e ? *e : BC(BC::NONE);
    }
    return out;
  }
};
} // namespace kalypsso

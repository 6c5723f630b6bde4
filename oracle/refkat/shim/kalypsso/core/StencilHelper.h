// Stub of kalypsso-core's stencil helper for the functor bridge: the face-side tag, the cell
// location record and the helper's interface. The bridge runs conforming blocks only, where the
// fine-neighbour lookups are never reached; they abort if called.
#pragma once
#include <cstdint>

#include <kalypsso/core/kokkos_shared.h>
#include <kalypsso/core/kalypsso_data_container.h>
#include <kalypsso/core/amr_hashmap.h>
#include <kalypsso/core/orchard_key_base.h>

namespace kalypsso
{
enum class face_type_t : int
{
  LEFT = 0,
  RIGHT = 1
};
template <std::size_t dim>
using shift_t = Kokkos::Array<int, dim>;
template <std::size_t dim>
struct CellLocation
{
  coord_t<dim> coords;
  uint64_t     key;
  int32_t      iOct;
  bool         is_ghost;
};
template <std::size_t dim, typename device_t>
struct StencilHelper
{
  StencilHelper() = default;
  template <class H, class K, class B, class P>
  StencilHelper(H const &, K const &, block_size_t<dim>, B const &, P const &)
  {}
  CellLocation<dim>
  getNeighLocFinerNearer(CellLocation<dim> const &, shift_t<dim> const &) const
  {
    Kokkos::abort("StencilHelper stub: fine-neighbour lookup on a conforming block");
  }
  template <class A>
  real_t
  compute_face_siblings_sum(CellLocation<dim> const &, int, A const &, bool) const
  {
    Kokkos::abort("StencilHelper stub: fine-neighbour flux sum on a conforming block");
  }
};
} // namespace kalypsso

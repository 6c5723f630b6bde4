// Stub of kalypsso-core's ghost-filling helpers used by ConvertToPrimitivesVariablesFunctor: a ghosted
// cell coordinate (-2 .. b+1 per axis) wrapped into the block (coord_in) and the direction of the
// neighbour region holding it (-1, 0, +1 per axis).
#pragma once
#include <kalypsso/core/kokkos_shared.h>
#include <kalypsso/core/kalypsso_data_container.h>

namespace kalypsso
{
template <std::size_t dim>
KOKKOS_INLINE_FUNCTION Kokkos::Array<int32_t, dim>
ghosted_coords_to_inner_coords(coord_t<dim> & coord_in, coord_t<dim> const & coord_out, block_size_t<dim> const & b)
{
  Kokkos::Array<int32_t, dim> dir;
  for (std::size_t a = 0; a < dim; ++a)
  {
    dir[a] = coord_out[a] < 0 ? -1 : (coord_out[a] >= b[a] ? 1 : 0);
    coord_in[a] = coord_out[a] - dir[a] * b[a];
  }
  return dir;
}
} // namespace kalypsso

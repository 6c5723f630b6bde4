// Stub of kalypsso-core's block index helpers for the functor bridge (test infrastructure).
#pragma once
#include <kalypsso/core/kalypsso_data_container.h>
#include <kalypsso/utils/config/ConfigMap.h>

namespace kalypsso
{
// (i, j[, k]) of cell `cell_index` of a ghosted block (x fastest), counted from the first interior cell
template <std::size_t dim>
KOKKOS_INLINE_FUNCTION Kokkos::Array<int32_t, dim>
cellindex_to_coord(int32_t cell_index, block_size_t<dim> ghosted, int32_t shift)
{
  Kokkos::Array<int32_t, dim> c;
  c[0] = cell_index % ghosted[0] - shift;
  c[1] = (cell_index / ghosted[0]) % ghosted[1] - shift;
  if constexpr (dim == 3)
    c[2] = cell_index / (ghosted[0] * ghosted[1]) - shift;
  return c;
}
// cell length of a leaf at `level` with `bx` cells along x over a unit brick (before the scaling factor)
template <std::size_t dim>
KOKKOS_INLINE_FUNCTION real_t
compute_cell_length(int level, int bx)
{
  return 1.0 / (double)((int64_t)bx << level);
}
inline real_t
get_scaling_factor(ConfigMap const & cm)
{
  return cm.getReal("mesh", "scaling_factor", 1.0);
}
} // namespace kalypsso

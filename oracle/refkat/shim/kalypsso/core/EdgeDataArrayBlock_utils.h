// Stub of kalypsso-core's edge-array helpers used by CorrectEmfAtBlockBorderFunctor (the functor's
// call sites fix their meaning): the flat numbering of a block's edges by direction (edges along d
// number b[d] along d and b + 1 across), its inverse, the edge location record, the unit vector of
// an edge direction and the outward vector of a border edge.
#pragma once
#include <cstdint>

#include <kalypsso/core/kokkos_shared.h>
#include <kalypsso/core/kalypsso_data_container.h>

namespace kalypsso
{
// offsets of the x, y and z edges in the flat numbering ([3]: total); 2D: z edges only
using edge_flat_index_offset_t = Kokkos::Array<int32_t, 4>;

template <std::size_t dim>
KOKKOS_INLINE_FUNCTION edge_flat_index_offset_t
compute_edge_flat_index_offsets_emf(block_size_t<dim> const & b)
{
  edge_flat_index_offset_t o;
  if constexpr (dim == 2)
  {
    o[0] = o[1] = o[2] = 0;
    o[3] = (b[0] + 1) * (b[1] + 1);
  }
  else
  {
    o[0] = 0;
    o[1] = b[0] * (b[1] + 1) * (b[2] + 1);
    o[2] = o[1] + (b[0] + 1) * b[1] * (b[2] + 1);
    o[3] = o[2] + (b[0] + 1) * (b[1] + 1) * b[2];
  }
  return o;
}

// (i, j[, k], direction) of edge `flat` (x fastest within a direction)
template <std::size_t dim>
KOKKOS_INLINE_FUNCTION Kokkos::Array<int32_t, dim + 1>
edge_flat_index_unravel_emf(int32_t flat, block_size_t<dim> const & b, edge_flat_index_offset_t const & o)
{
  Kokkos::Array<int32_t, dim + 1> r;
  if constexpr (dim == 2)
  {
    r[0] = flat % (b[0] + 1);
    r[1] = flat / (b[0] + 1);
    r[2] = 2;
  }
  else
  {
    int d = 2;
    while (d > 0 && flat < o[d])
      --d;
    int32_t rem = flat - o[d];
    for (int a = 0; a < 3; ++a)
    {
      const int32_t n = b[a] + (a == d ? 0 : 1);
      r[a] = rem % n;
      rem /= n;
    }
    r[3] = d;
  }
  return r;
}

// DIAGONAL: both transverse axes; DIR1 / DIR2: the first / second transverse axis only (used by the
// reference's unused correct_emf_3d)
enum class EdgeNormalType : int
{
  DIAGONAL = 0,
  DIR1 = 1,
  DIR2 = 2
};

// per transverse axis: -1 on the low border, +1 on the high border, 0 inside; 0 along the edge
template <std::size_t dim>
KOKKOS_INLINE_FUNCTION Kokkos::Array<int32_t, dim>
get_edge_outside_unit_vector(Kokkos::Array<int32_t, dim + 1> const & e, block_size_t<dim> const & b, EdgeNormalType t)
{
  Kokkos::Array<int32_t, dim> v;
  const int dir = dim == 2 ? 2 : e[dim];
  const int t0 = dir == 0 ? 1 : 0, t1 = dir == 2 ? 1 : 2;
  for (std::size_t a = 0; a < dim; ++a)
  {
    const bool keep = t == EdgeNormalType::DIAGONAL || (t == EdgeNormalType::DIR1 && (int)a == t0) ||
                      (t == EdgeNormalType::DIR2 && (int)a == t1);
    v[a] = ((int)a == dir || !keep) ? 0 : (e[a] == 0 ? -1 : (e[a] == b[a] ? 1 : 0));
  }
  return v;
}

template <std::size_t dim>
KOKKOS_INLINE_FUNCTION Kokkos::Array<int32_t, dim>
get_unit_vector(int d)
{
  Kokkos::Array<int32_t, dim> v;
  for (std::size_t a = 0; a < dim; ++a)
    v[a] = (int)a == d ? 1 : 0;
  return v;
}

// an edge seen from one block: its (i, j[, k], direction) there, the block's key (its level here),
// the block, whether it is an MPI ghost; is_valid: the edge exists on that side
template <std::size_t dim>
struct EdgeLocation
{
  Kokkos::Array<int32_t, dim + 1> ijk;
  uint64_t                        key;
  int32_t                         iOct;
  bool                            is_ghost;
  bool                            is_valid = true;
  KOKKOS_INLINE_FUNCTION int      level() const { return (int)(key & 63); }
};
} // namespace kalypsso

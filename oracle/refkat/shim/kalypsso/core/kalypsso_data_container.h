// Stub of kalypsso-core's block data containers for the functor bridge (test infrastructure):
// host arrays of n octants x nvar variables x (b + 2 g)^d cells, variable-major per octant, x fastest
// (the octant-contiguous SoA the reference slices, scheme/GodunovImplemV0.cpp:304-319). Element
// (i, j[, k], var, oct) counts i, j, k from the first interior cell, -g .. b + g - 1. Copies share
// storage, as Kokkos views do.
#pragma once
#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>

#include <kalypsso/core/kokkos_shared.h>
#include <kalypsso/utils/config/ConfigMap.h>

namespace kalypsso
{
template <std::size_t dim>
using block_size_t = Kokkos::Array<int32_t, dim>;
template <std::size_t dim, typename T = int32_t>
using coord_t = Kokkos::Array<T, dim>;
template <std::size_t dim>
using brick_size_t = Kokkos::Array<int32_t, dim>;
// an array with every element v
template <typename T, std::size_t N>
KOKKOS_INLINE_FUNCTION Kokkos::Array<T, N>
init_kokkos_array(T v)
{
  Kokkos::Array<T, N> a;
  for (std::size_t i = 0; i < N; ++i)
    a[i] = v;
  return a;
}
// the four edges of a cell seen by the 2D magnetic Riemann problem
enum class MHDEdgeLocation : int
{
  LB = 0,
  RT = 1,
  RB = 2,
  LT = 3
};

template <std::size_t dim, typename T, typename device_t>
class DataArrayGhostedBlock
{
public:
  DataArrayGhostedBlock() = default;
  DataArrayGhostedBlock(block_size_t<dim> bs, int ghost, int nvar, int noct)
    : m_bs(bs), m_g(ghost), m_nvar(nvar), m_noct(noct)
  {
    m_ncell = 1;
    for (std::size_t d = 0; d < dim; ++d)
      m_ncell *= bs[d] + 2 * ghost;
    m_data = std::make_shared<std::vector<T>>((std::size_t)m_ncell * nvar * noct, T(0));
  }
  template <std::size_t D = dim, std::enable_if_t<D == 2, int> = 0>
  T &
  operator()(int i, int j, int var, int oct) const
  {
    const int nx = m_bs[0] + 2 * m_g;
    return (*m_data)[(std::size_t)(i + m_g) + nx * (j + m_g) + (std::size_t)m_ncell * (var + (std::size_t)m_nvar * oct)];
  }
  template <std::size_t D = dim, std::enable_if_t<D == 3, int> = 0>
  T &
  operator()(int i, int j, int k, int var, int oct) const
  {
    const int nx = m_bs[0] + 2 * m_g, ny = m_bs[1] + 2 * m_g;
    return (*m_data)[(std::size_t)(i + m_g) + nx * ((j + m_g) + (std::size_t)ny * (k + m_g)) +
                     (std::size_t)m_ncell * (var + (std::size_t)m_nvar * oct)];
  }
  int32_t num_cells() const { return m_ncell; }
  int32_t num_vars() const { return m_nvar; }
  int32_t num_quadrants() const { return m_noct; }
  int32_t shift() const { return m_g; }
  block_size_t<dim> block_size() const { return m_bs; }
  block_size_t<dim> shape() const { return m_bs; }
  block_size_t<dim>
  ghosted_block_size() const
  {
    block_size_t<dim> g;
    for (std::size_t d = 0; d < dim; ++d)
      g[d] = m_bs[d] + 2 * m_g;
    return g;
  }
  // element (cell, var, oct) of an unghosted block
  T &
  operator()(int cell, int var, int oct) const
  {
    return (*m_data)[(std::size_t)cell + (std::size_t)m_ncell * (var + (std::size_t)m_nvar * oct)];
  }
  T * data() const { return m_data->data(); }

private:
  block_size_t<dim>               m_bs{};
  int                             m_g = 0, m_nvar = 0, m_noct = 0, m_ncell = 0;
  std::shared_ptr<std::vector<T>> m_data;
};

template <std::size_t dim, typename T, typename device_t>
using DataArrayBlock = DataArrayGhostedBlock<dim, T, device_t>;
// Face-centred B of n octants: per octant Bx on (bx+1) x by [x bz], By on bx x (by+1) [x bz], and Bz on
// bx x by x (bz+1) (3D) or cell-centred (2D), each x fastest, components concatenated (the layout of
// the C ABI's face arrays). Element (i, j[, k], comp, oct).
template <std::size_t dim, typename T, typename device_t>
class FaceDataArrayBlock
{
public:
  FaceDataArrayBlock() = default;
  // shift: ghost width (element (0, ...) is the first face of the inner block)
  FaceDataArrayBlock(block_size_t<dim> cells, int noct, int shift = 0) : m_cells(cells), m_noct(noct), m_shift(shift)
  {
    int off = 0;
    for (int c = 0; c < 3; ++c)
    {
      int n = 1;
      for (std::size_t d = 0; d < dim; ++d)
        n *= cells[d] + ((int)d == c ? 1 : 0);
      m_off[c] = off;
      off += n;
    }
    m_per = off;
    m_data = std::make_shared<std::vector<T>>((std::size_t)m_per * noct, T(0));
  }
  template <std::size_t D = dim, std::enable_if_t<D == 2, int> = 0>
  T &
  operator()(int i, int j, int c, int oct) const
  {
    const int nx = m_cells[0] + (c == 0);
    i += m_shift;
    j += m_shift;
    return (*m_data)[(std::size_t)m_per * oct + m_off[c] + i + (std::size_t)nx * j];
  }
  template <std::size_t D = dim, std::enable_if_t<D == 3, int> = 0>
  T &
  operator()(int i, int j, int k, int c, int oct) const
  {
    const int nx = m_cells[0] + (c == 0), ny = m_cells[1] + (c == 1);
    i += m_shift;
    j += m_shift;
    k += m_shift;
    return (*m_data)[(std::size_t)m_per * oct + m_off[c] + i + (std::size_t)nx * (j + (std::size_t)ny * k)];
  }
  block_size_t<dim>       cell_block_size() const { return m_cells; }
  // extents of face component c (2D c = 2: the cell-centred Bz)
  block_size_t<dim>
  face_block_size(int c) const
  {
    block_size_t<dim> s = m_cells;
    if (c < (int)dim)
      s[c] += 1;
    return s;
  }
  int32_t                 num_elements_per_octant() const { return m_per; }
  Kokkos::Array<int32_t, 3> offsets() const
  {
    Kokkos::Array<int32_t, 3> o;
    for (int c = 0; c < 3; ++c)
      o[c] = m_off[c];
    return o;
  }
  int32_t shift() const { return m_shift; }
  T *     data() const { return m_data->data(); }

private:
  block_size_t<dim>               m_cells{};
  int                             m_noct = 0, m_shift = 0, m_per = 0, m_off[3] = {0, 0, 0};
  std::shared_ptr<std::vector<T>> m_data;
};
} // namespace kalypsso

// ---- block index helpers (kalypsso-core utils) ----
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
// (i, j[, k]) of cell `cell_index` of an unghosted block of `shape` (x fastest)
template <std::size_t dim>
KOKKOS_INLINE_FUNCTION Kokkos::Array<int32_t, dim>
cellindex_to_coord(int32_t cell_index, block_size_t<dim> shape)
{
  return cellindex_to_coord<dim>(cell_index, shape, 0);
}
// flat index of cell c of an unghosted block of size b (x fastest)
template <std::size_t dim>
KOKKOS_INLINE_FUNCTION int32_t
coord_to_cellindex(coord_t<dim> const & c, block_size_t<dim> const & b)
{
  int32_t i = c[dim - 1];
  for (int a = (int)dim - 2; a >= 0; --a)
    i = i * b[a] + c[a];
  return i;
}
// (i, j[, k], comp) of element `flat` of one octant's face array (components at offsets[comp], each
// x fastest; 2D comp 2 is the cell-centred Bz) of an unghosted face array (shift 0, as the outside
// fill reads it)
template <std::size_t dim>
KOKKOS_INLINE_FUNCTION Kokkos::Array<int32_t, dim + 1>
face_flat_index_unravel(int32_t flat, block_size_t<dim> const & cells, Kokkos::Array<int32_t, 3> const & offsets,
                        int32_t shift)
{
  const int comp = flat < offsets[1] ? 0 : (flat < offsets[2] ? 1 : 2);
  int32_t   r = flat - offsets[comp];
  Kokkos::Array<int32_t, dim + 1> out;
  for (std::size_t d = 0; d < dim; ++d)
  {
    const int32_t n = cells[d] + ((int)d == comp ? 1 : 0);
    out[d] = r % n;
    r /= n;
  }
  (void)shift;
  out[dim] = comp;
  return out;
}
template <std::size_t dim>
KOKKOS_INLINE_FUNCTION Kokkos::Array<int32_t, dim>
cell_index_unravel(int32_t cell_index, block_size_t<dim> shape)
{
  return cellindex_to_coord<dim>(cell_index, shape, 0);
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
// (i, j[, k], comp) of face `idx` of a face block (components concatenated at `offsets`)
template <std::size_t dim, typename O>
KOKKOS_INLINE_FUNCTION Kokkos::Array<int32_t, dim + 1>
face_flat_index_unravel(int32_t idx, block_size_t<dim> cells, O const & offsets, int32_t shift)
{
  int c = 2;
  while (c > 0 && idx < offsets[c])
    --c;
  int32_t r = idx - offsets[c];
  Kokkos::Array<int32_t, dim + 1> out;
  for (std::size_t d = 0; d < dim; ++d)
  {
    const int32_t n = cells[d] + ((int)d == c ? 1 : 0);
    out[d] = r % n - shift;
    r /= n;
  }
  out[dim] = c;
  return out;
}
} // namespace kalypsso

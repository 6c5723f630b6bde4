// Stub of kalypsso-core's stencil helper for the functor bridge (test infrastructure). kalypsso-core is
// not in the reference tree; these lookups are restated from their call sites in the reference's
// functors, on the bridge's neighbour tables (amr_hashmap.h), with this build's definitions (the same
// ones the oracle and the GPU kernels use):
//  * getEdgeSiblingLoc(edge, n): the copy of a block-border edge in the region across its first
//    transverse axis (n = 0), its second (n = 1) or both (n = 2): a same-level leaf (the same edge in
//    its index space), a coarser leaf (level only; the edge's position in it), or the finer child that
//    holds the edge's lower end (index 2 i along the edge), invalid where no region exists;
//  * getNeighLocFinerNearer(cell, shift): the finer neighbour cell across the face `shift` of a border
//    cell, the one with the lower index along the face's transverse axes (2 i), and its leaf;
//  * compute_face_siblings_sum(cell, var, fluxes, right): the sum of the 2^(d-1) fine face fluxes
//    covering the coarse face, first transverse axis fastest, starting from 0.
#pragma once
#include <cstdint>

#include <kalypsso/core/kokkos_shared.h>
#include <kalypsso/core/kalypsso_data_container.h>
#include <kalypsso/core/amr_hashmap.h>
#include <kalypsso/core/orchard_key_base.h>
#include <kalypsso/core/EdgeDataArrayBlock_utils.h>

namespace kalypsso
{
struct ParallelEnv
{
  int rank() const { return 0; }
};
enum class face_type_t : int
{
  LEFT = 0,
  RIGHT = 1
};
template <std::size_t dim>
using shift_t = Kokkos::Array<int, dim>;
// a cell seen from one block; dir / side: the face a finer-neighbour lookup crossed
template <std::size_t dim>
struct CellLocation
{
  coord_t<dim>               coords;
  uint64_t                   key;
  int32_t                    iOct;
  bool                       is_ghost;
  int                        dir = -1;
  int                        side = 0;
  KOKKOS_INLINE_FUNCTION int level() const { return (int)key; }
};
template <std::size_t dim, typename device_t>
struct StencilHelper
{
  const BridgeMesh * m = nullptr;
  block_size_t<dim>  b{};

  StencilHelper() = default;
  template <class H, class K, class B, class P>
  StencilHelper(H const & map, K const &, block_size_t<dim> bs, B const &, P const &) : m(map.mesh), b(bs)
  {}

  static int slot(int ox, int oy, int oz) { return (oz + 1) * 9 + (oy + 1) * 3 + (ox + 1); }

  uint64_t key(int32_t iOct) const { return (uint64_t)m->level[iOct]; }

  EdgeLocation<dim>
  getEdgeSiblingLoc(EdgeLocation<dim> const & e, int n) const
  {
    EdgeLocation<dim> out{e.ijk, 0, -1, false, false};
    const int dir = dim == 2 ? 2 : e.ijk[dim];
    const int t0 = dir == 0 ? 1 : 0, t1 = dir == 2 ? 1 : 2;
    int       bs[3] = {b[0], b[1], dim == 3 ? (int)b[2] : 1};
    int       ijk[3] = {e.ijk[0], e.ijk[1], dim == 3 ? (int)e.ijk[2] : 0};
    const int v0 = ijk[t0] == 0 ? -1 : (ijk[t0] == bs[t0] ? 1 : 0);
    const int v1 = (dim == 2 && t1 == 2) ? 0 : (ijk[t1] == 0 ? -1 : (ijk[t1] == bs[t1] ? 1 : 0));
    int       o[3] = {0, 0, 0};
    if (n == 0 || n == 2)
      o[t0] = v0;
    if (n == 1 || n == 2)
      o[t1] = v1;
    const bool exists = (n == 0 && v0 != 0) || (n == 1 && v1 != 0) || (n == 2 && v0 != 0 && v1 != 0);
    if (!exists)
      return out;
    const int32_t s = slot(o[0], o[1], o[2]);
    const int32_t nb = m->neighbor[(int64_t)e.iOct * 27 + s];
    const int     lv = m->level[e.iOct];
    if (nb >= 0)
    {
      out.iOct = nb;
      out.key = (uint64_t)m->level[nb];
      out.is_valid = true;
      if (m->level[nb] == lv || nb >= m->n_owned)
      {
        for (int a = 0; a < (int)dim; ++a)
          out.ijk[a] = ijk[a] - o[a] * bs[a];
      }
      else
      {
        // coarser leaf: the region is one half of it along each axis (parity of the region's coordinate)
        for (int a = 0; a < (int)dim; ++a)
        {
          const int half = (m->coord[(int64_t)e.iOct * 3 + a] + o[a]) & 1;
          out.ijk[a] = (half * bs[a] + ijk[a] - o[a] * bs[a]) / 2;
        }
      }
      return out;
    }
    if (!m->fine)
      return out;
    int F[3] = {0, 0, 0}, ch[3] = {0, 0, 0};
    for (int a = 0; a < (int)dim; ++a)
    {
      if (o[a] != 0)
      {
        ch[a] = o[a] < 0 ? 1 : 0;
        F[a] = o[a] < 0 ? bs[a] : 0;
      }
      else
      {
        const int x = 2 * ijk[a];
        ch[a] = x >= bs[a] ? 1 : 0;
        F[a] = x - ch[a] * bs[a];
      }
    }
    const int32_t id = m->fine[((int64_t)e.iOct * 27 + s) * 8 + ch[0] + 2 * ch[1] + 4 * ch[2]];
    if (id < 0)
      return out;
    out.iOct = id;
    out.key = (uint64_t)m->level[id];
    out.is_valid = true;
    for (int a = 0; a < (int)dim; ++a)
      out.ijk[a] = F[a];
    return out;
  }

  CellLocation<dim>
  getNeighLocFinerNearer(CellLocation<dim> const & c, shift_t<dim> const & shift) const
  {
    CellLocation<dim> out{c.coords, 0, -1, false};
    int               o[3] = {0, 0, 0}, d = 0;
    for (int a = 0; a < (int)dim; ++a)
      if (shift[a] != 0)
      {
        o[a] = shift[a];
        d = a;
      }
    if (!m->fine)
      return out;
    int ch[3] = {0, 0, 0};
    for (int a = 0; a < (int)dim; ++a)
    {
      if (a == d)
      {
        ch[a] = o[a] < 0 ? 1 : 0;
        out.coords[a] = o[a] < 0 ? b[a] - 1 : 0;
      }
      else
      {
        const int x = 2 * c.coords[a];
        ch[a] = x >= b[a] ? 1 : 0;
        out.coords[a] = x - ch[a] * b[a];
      }
    }
    const int32_t id = m->fine[((int64_t)c.iOct * 27 + slot(o[0], o[1], o[2])) * 8 + ch[0] + 2 * ch[1] + 4 * ch[2]];
    out.iOct = id;
    out.key = id >= 0 ? (uint64_t)m->level[id] : 0;
    out.dir = d;
    out.side = o[d];
    return out;
  }

  template <class A>
  real_t
  compute_face_siblings_sum(CellLocation<dim> const & c, int var, A const & fluxes, bool use_right_flux) const
  {
    const int d = c.dir;
    const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
    real_t    acc = 0;
    if (c.iOct < 0)
      return acc;
    for (int e2 = 0; e2 < (dim == 3 ? 2 : 1); ++e2)
      for (int e1 = 0; e1 < 2; ++e1)
      {
        int f[3] = {c.coords[0], c.coords[1], dim == 3 ? (int)c.coords[2] : 0};
        f[t1] += e1;
        if (dim == 3)
          f[t2] += e2;
        if (use_right_flux)
          f[d] += 1;
        if constexpr (dim == 2)
          acc += fluxes(f[0], f[1], var, c.iOct);
        else
          acc += fluxes(f[0], f[1], f[2], var, c.iOct);
      }
    return acc;
  }
};
} // namespace kalypsso

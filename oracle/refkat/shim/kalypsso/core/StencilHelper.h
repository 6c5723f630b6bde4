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
//    covering the coarse face, first transverse axis fastest, starting from 0;
//  * getNeighLoc(cell, shift): the cell at position cell + shift of the cell's block (at most one block
//    away): in a same-level or outside leaf the cell itself, in a coarser leaf the coarse cell
//    containing it, in a finer region the fine child cell with the even indices 2 q (the first of the
//    2^d cells covering it);
//  * compute_siblings_average(cell, b, var, U): the mean of the 2^d fine cells from that first one, x
//    fastest, summed from 0 then divided by 2^d;
//  * compute_minmod_slopes(c, right, left, var, U, 1): minmod(u - u_left, u_right - u) (0 when they
//    differ in sign), a neighbour location at a finer level read as its sibling average.
#pragma once
#include <cmath>
#include <cstdint>

#include <kalypsso/core/kalypsso_core_base.h>
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
// signed axis ids of unit_shift (+-XDIR ...)
enum : int
{
  XDIR = 1,
  YDIR = 2,
  ZDIR = 3
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
  coord_t<dim>               ijk;
  uint64_t                   key;
  int32_t                    iOct;
  bool                       is_ghost;
  int                        dir = -1;
  int                        side = 0;
  KOKKOS_INLINE_FUNCTION int level() const { return (int)(key & 63); }
  // index of the cell in an unghosted block of size b (x fastest)
  KOKKOS_INLINE_FUNCTION int32_t
  cellindex(block_size_t<dim> const & b) const
  {
    int32_t c = ijk[dim - 1];
    for (int a = (int)dim - 2; a >= 0; --a)
      c = c * b[a] + ijk[a];
    return c;
  }
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
    CellLocation<dim> out{c.ijk, 0, -1, false};
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
        out.ijk[a] = o[a] < 0 ? b[a] - 1 : 0;
      }
      else
      {
        const int x = 2 * c.ijk[a];
        ch[a] = x >= b[a] ? 1 : 0;
        out.ijk[a] = x - ch[a] * b[a];
      }
    }
    const int32_t id = m->fine[((int64_t)c.iOct * 27 + slot(o[0], o[1], o[2])) * 8 + ch[0] + 2 * ch[1] + 4 * ch[2]];
    out.iOct = id;
    out.key = id >= 0 ? (uint64_t)m->level[id] : 0;
    out.dir = d;
    out.side = o[d];
    return out;
  }

  shift_t<dim>
  unit_shift(int s) const
  {
    shift_t<dim> r;
    for (std::size_t a = 0; a < dim; ++a)
      r[a] = 0;
    r[(s < 0 ? -s : s) - 1] = s < 0 ? -1 : 1;
    return r;
  }

  CellLocation<dim>
  getNeighLoc(CellLocation<dim> const & c, shift_t<dim> const & shift) const
  {
    CellLocation<dim> out{c.ijk, 0, -1, false};
    int               o[3] = {0, 0, 0}, q[3] = {0, 0, 0};
    for (int a = 0; a < (int)dim; ++a)
    {
      const int p = c.ijk[a] + shift[a];
      o[a] = p < 0 ? -1 : (p >= b[a] ? 1 : 0);
      q[a] = p - o[a] * b[a];
    }
    const int lv = m->level[c.iOct];
    if (o[0] == 0 && o[1] == 0 && o[2] == 0)
    {
      for (int a = 0; a < (int)dim; ++a)
        out.ijk[a] = q[a];
      out.iOct = c.iOct;
      out.key = (uint64_t)lv;
      return out;
    }
    const int32_t s = slot(o[0], o[1], o[2]);
    const int32_t nb = m->neighbor[(int64_t)c.iOct * 27 + s];
    if (nb >= 0)
    {
      out.iOct = nb;
      out.key = (uint64_t)m->level[nb];
      for (int a = 0; a < (int)dim; ++a)
      {
        if (m->level[nb] == lv || nb >= m->n_owned)
          out.ijk[a] = q[a];
        else
        {
          const int half = (m->coord[(int64_t)c.iOct * 3 + a] + o[a]) & 1;
          out.ijk[a] = (half * b[a] + q[a]) >> 1;
        }
      }
      return out;
    }
    int ch[3] = {0, 0, 0};
    for (int a = 0; a < (int)dim; ++a)
    {
      const int x = 2 * q[a];
      ch[a] = x >= b[a] ? 1 : 0;
      out.ijk[a] = x - ch[a] * b[a];
    }
    const int32_t id = m->fine ? m->fine[((int64_t)c.iOct * 27 + s) * 8 + ch[0] + 2 * ch[1] + 4 * ch[2]] : -1;
    out.iOct = id;
    out.key = id >= 0 ? (uint64_t)m->level[id] : 0;
    return out;
  }

  template <class A>
  real_t
  compute_siblings_average(CellLocation<dim> const & c, block_size_t<dim> const & bs, int var, A const & U) const
  {
    real_t acc = 0;
    for (int ez = 0; ez < (dim == 3 ? 2 : 1); ++ez)
      for (int ey = 0; ey < 2; ++ey)
        for (int ex = 0; ex < 2; ++ex)
        {
          CellLocation<dim> f = c;
          f.ijk[0] += ex;
          f.ijk[1] += ey;
          if constexpr (dim == 3)
            f.ijk[2] += ez;
          acc += U(f.cellindex(bs), var, c.iOct);
        }
    return acc / (real_t)(1 << dim);
  }

  template <class A>
  real_t
  compute_minmod_slopes(CellLocation<dim> const & c, CellLocation<dim> const & right, CellLocation<dim> const & left,
                        int var, A const & U, real_t /*slope_type: 1 at every call site*/) const
  {
    auto val = [&](CellLocation<dim> const & l) {
      return l.level() > c.level() ? compute_siblings_average(l, b, var, U) : U(l.cellindex(b), var, l.iOct);
    };
    const real_t u = U(c.cellindex(b), var, c.iOct);
    const real_t dl = u - val(left), dr = val(right) - u;
    if (dl * dr <= 0.0)
      return 0.0;
    return dl > 0.0 ? std::fmin(dl, dr) : std::fmax(dl, dr);
  }

  // the MPI-mirror path of ConvertToPrimitivesVariablesFunctor looks mirror keys up here (unused on
  // one rank)
  struct MirrorMap
  {
    int      find(uint64_t) const { return -1; }
    bool     valid_at(int) const { return false; }
    int32_t  value_at(int) const { return -1; }
  } m_amr_hashmap_device;

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
        int f[3] = {c.ijk[0], c.ijk[1], dim == 3 ? (int)c.ijk[2] : 0};
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

// Coarse/fine ghost prepass: builds, for every neighbour region of an owned block that lies at
// another level (or whose border faces must come from a finer region), a virtual same-level block
// holding exactly the ghost values the block's stencil reads. The fused step then gathers from it as
// from a same-level neighbour.
//
// Definitions (kalypsso-core's FillBlockGhostFacesFunctor, compute_siblings_average and
// compute_minmod_slopes are not part of the reference tree; these are this library's):
//   * face B: a same-level or outside region copies the neighbour's face; a finer region takes the
//     mean of the 2^(d-1) fine faces covering the face (first transverse axis fastest); a coarser
//     region takes the coarse face containing the face when it lies on a coarse face, else the mean
//     of the two coarse faces bounding the coarse cell along the normal. 2D Bz is cell-centred:
//     mean of the 4 fine cells / the coarse cell. A face on the border between two regions along its
//     normal (the block itself included) comes from the finer of the two, so that every block sees
//     one value for it; a finer face neighbour's virtual block therefore also holds the block's own
//     shared border face;
//   * hydro (ConvertToPrimitivesVariablesFunctor.cpp:217-283, 439-446, 471-635): a finer region
//     gives the mean of the 2^d fine cells (x fastest); a coarser region copies the coarse cell
//     (SIMPLE_COPY, with the coarse cell's own cell-centred B in Bcc, from the coarse block's ghosted
//     faces: a border face shared with a finer region is that region's) or adds 0.25 * (+-1) *
//     minmod(u - u_left, u_right - u) per axis at the coarse level (EXTRAPOLATE_LINEAR_MINMOD).
// Built with --fmad=false: the FP64 path reproduces the CPU restatement bit for bit.
#include <cuda_runtime.h>

#include <cstdint>

#include "launch.cuh"

namespace gmhd
{

struct DRegion
{
  int             kind, id;
  int             sub[3];
  const int32_t * child;
};

__device__ static DRegion
region_of(const GhostArgs & g, int blk, int ox, int oy, int oz)
{
  DRegion r{RK_MISSING, -1, {0, 0, 0}, nullptr};
  if ((ox | oy | oz) == 0)
  {
    r.kind = RK_SAME;
    r.id = blk;
    return r;
  }
  const int64_t s = (int64_t)blk * 27 + nb_slot(ox, oy, oz);
  r.kind = g.kind[s];
  r.id = g.neighbor[s];
  if (r.kind == RK_COARSER)
  {
    const int o[3] = {ox, oy, oz};
    for (int d = 0; d < g.dim; ++d)
      r.sub[d] = (g.coord[(int64_t)blk * 3 + d] + o[d]) & 1;
  }
  else if (r.kind == RK_FINER)
    r.child = g.fine + s * 8;
  return r;
}

__device__ static int
region_level(const DRegion & r)
{
  return r.kind == RK_COARSER ? -1 : (r.kind == RK_FINER ? 1 : (r.kind == RK_MISSING ? -100 : 0));
}

__device__ static inline int
axis_off(int idx, int n)
{
  return idx < 0 ? -1 : (idx >= n ? 1 : 0);
}

__device__ static double
face_at(const GhostArgs & g, int blk, int comp, int i, int j, int k)
{
  const double * Bb = g.B + (int64_t)blk * g.nface;
  if (comp == 0)
    return Bb[i + (int64_t)(g.bx + 1) * (j + (int64_t)g.by * k)];
  if (comp == 1)
    return Bb[g.nfx + i + (int64_t)g.bx * (j + (int64_t)(g.by + 1) * k)];
  return Bb[g.nfx + g.nfy + i + (int64_t)g.bx * (j + (int64_t)g.by * k)];
}

__device__ static double
u_at(const GhostArgs & g, int blk, int v, int i, int j, int k)
{
  return g.U[((int64_t)blk * 5 + v) * g.ncell + i + (int64_t)g.bx * (j + (int64_t)g.by * k)];
}

// Face value of component comp at region-local q of region r; false when a needed leaf is absent.
__device__ static bool
region_face(const GhostArgs & g, const DRegion & r, int comp, const int * q, double & out)
{
  const int  b[3] = {g.bx, g.by, g.bz};
  const bool cellc = g.dim == 2 && comp == 2;
  switch (r.kind)
  {
    case RK_SAME:
    case RK_OUTSIDE:
      out = face_at(g, r.id, comp, q[0], q[1], q[2]);
      return true;
    case RK_FINER:
    {
      double acc = 0.0;
      if (cellc)
      {
        for (int ey = 0; ey < 2; ++ey)
          for (int ex = 0; ex < 2; ++ex)
          {
            const int F0 = 2 * q[0] + ex, F1 = 2 * q[1] + ey;
            const int c0 = F0 >= b[0], c1 = F1 >= b[1];
            const int id = r.child[c0 + 2 * c1];
            if (id < 0)
              return false;
            acc += face_at(g, id, 2, F0 - c0 * b[0], F1 - c1 * b[1], 0);
          }
        out = acc / 4.0;
        return true;
      }
      const int t1 = comp == 0 ? 1 : 0;
      const int t2 = comp == 2 ? 1 : 2;
      for (int e2 = 0; e2 < (g.dim == 3 ? 2 : 1); ++e2)
        for (int e1 = 0; e1 < 2; ++e1)
        {
          int F[3] = {0, 0, 0}, c[3] = {0, 0, 0};
          F[comp] = 2 * q[comp];
          c[comp] = F[comp] >= b[comp];
          F[t1] = 2 * q[t1] + e1;
          c[t1] = F[t1] >= b[t1];
          if (g.dim == 3)
          {
            F[t2] = 2 * q[t2] + e2;
            c[t2] = F[t2] >= b[t2];
          }
          int id = r.child[c[0] + 2 * c[1] + 4 * c[2]];
          if (id < 0 && F[comp] == b[comp])
          {
            // a face between the two children along its normal: the other child holds it too
            c[comp] = 0;
            id = r.child[c[0] + 2 * c[1] + 4 * c[2]];
          }
          if (id < 0)
            return false;
          acc += face_at(g, id, comp, F[0] - c[0] * b[0], F[1] - c[1] * b[1], F[2] - c[2] * b[2]);
        }
      out = acc / (g.dim == 3 ? 4.0 : 2.0);
      return true;
    }
    case RK_COARSER:
    {
      int F[3] = {0, 0, 0};
      for (int d = 0; d < g.dim; ++d)
        F[d] = r.sub[d] * b[d] + q[d];
      if (cellc)
      {
        out = face_at(g, r.id, 2, F[0] >> 1, F[1] >> 1, 0);
        return true;
      }
      int T[3] = {F[0] >> 1, F[1] >> 1, F[2] >> 1};
      if ((F[comp] & 1) == 0)
      {
        T[comp] = F[comp] / 2;
        out = face_at(g, r.id, comp, T[0], T[1], T[2]);
      }
      else
      {
        int T1[3] = {T[0], T[1], T[2]};
        T[comp] = (F[comp] - 1) / 2;
        T1[comp] = (F[comp] + 1) / 2;
        out = 0.5 * (face_at(g, r.id, comp, T[0], T[1], T[2]) + face_at(g, r.id, comp, T1[0], T1[1], T1[2]));
      }
      return true;
    }
    default:
      return false;
  }
}

// Face comp at inner index (i, j, k) of block blk as its ghosted face field holds it: the block's own
// face, except that a border face shared (along its normal) with a finer neighbour region is that
// region's value (false when a needed leaf is absent).
__device__ static bool
own_ghost_face(const GhostArgs & g, int blk, int comp, int i, int j, int k, double & out)
{
  const int b[3] = {g.bx, g.by, g.bz};
  const int idx[3] = {i, j, k};
  if (!(g.dim == 2 && comp == 2) && (idx[comp] == 0 || idx[comp] == b[comp]))
  {
    int o1[3] = {0, 0, 0};
    o1[comp] = idx[comp] == 0 ? -1 : 1;
    const DRegion r1 = region_of(g, blk, o1[0], o1[1], o1[2]);
    if (r1.kind == RK_FINER)
    {
      int q[3] = {i, j, k};
      q[comp] = idx[comp] == 0 ? b[comp] : 0;
      return region_face(g, r1, comp, q, out);
    }
  }
  out = face_at(g, blk, comp, i, j, k);
  return true;
}

// Mean of the 2^d fine cells of variable v covering region-local cell q of a finer region.
__device__ static bool
restrict_cell(const GhostArgs & g, const DRegion & r, const int * q, int v, double & out)
{
  const int b[3] = {g.bx, g.by, g.bz};
  double    acc = 0.0;
  for (int ez = 0; ez < (g.dim == 3 ? 2 : 1); ++ez)
    for (int ey = 0; ey < 2; ++ey)
      for (int ex = 0; ex < 2; ++ex)
      {
        const int F[3] = {2 * q[0] + ex, 2 * q[1] + ey, g.dim == 3 ? 2 * q[2] + ez : 0};
        const int c[3] = {F[0] >= b[0], F[1] >= b[1], F[2] >= b[2]};
        const int id = r.child[c[0] + 2 * c[1] + 4 * c[2]];
        if (id < 0)
          return false;
        acc += u_at(g, id, v, F[0] - c[0] * b[0], F[1] - c[1] * b[1], F[2] - c[2] * b[2]);
      }
  out = acc / (double)(1 << g.dim);
  return true;
}

// Conservative variable v of cell (i, j, k) in block blk's frame at blk's level, at most one block
// away (used for the coarse-level slopes of EXTRAPOLATE_LINEAR_MINMOD).
__device__ static bool
level_cell_value(const GhostArgs & g, int blk, int v, int i, int j, int k, double & out)
{
  const int     b[3] = {g.bx, g.by, g.bz};
  const int     o[3] = {axis_off(i, g.bx), axis_off(j, g.by), g.dim == 3 ? axis_off(k, g.bz) : 0};
  const DRegion r = region_of(g, blk, o[0], o[1], o[2]);
  const int     q[3] = {i - o[0] * b[0], j - o[1] * b[1], k - o[2] * b[2]};
  switch (r.kind)
  {
    case RK_SAME:
    case RK_OUTSIDE:
      out = u_at(g, r.id, v, q[0], q[1], q[2]);
      return true;
    case RK_FINER:
      return restrict_cell(g, r, q, v, out);
    case RK_COARSER:
      out = u_at(g, r.id, v, (r.sub[0] * b[0] + q[0]) >> 1, (r.sub[1] * b[1] + q[1]) >> 1,
                 (r.sub[2] * b[2] + q[2]) >> 1);
      return true;
    default:
      return false;
  }
}

__device__ static double
minmod_slope(double u, double ur, double ul)
{
  const double dl = u - ul, dr = ur - u;
  if (dl * dr <= 0.0)
    return 0.0;
  return dl > 0.0 ? fmin(dl, dr) : fmax(dl, dr);
}

// Cells (or faces, along their normal) of region o that lie within two cells of the block: the
// only ones the fused step reads. o < 0: the last two (faces: b-2 .. b), o > 0: the first two (faces:
// 0 .. 2), o == 0: all.
__device__ static void
near_range(int o, int n, bool normal, int & lo, int & len)
{
  if (o == 0)
  {
    lo = 0;
    len = n + (normal ? 1 : 0);
  }
  else
  {
    lo = o < 0 ? n - 2 : 0;
    len = normal ? 3 : 2;
  }
}

// One warp per virtual block (grid-stride over the warps of all CTAs), its lanes over the cells and
// faces of the region's near layer.
__global__ void __launch_bounds__(256)
ghost_prepass_kernel(const GhostArgs g)
{
  const int b[3] = {g.bx, g.by, g.bz};
  // one warp per virtual block: a region's near layer is a few dozen to a few hundred cells and faces
  const int wpb = blockDim.x >> 5, lane = threadIdx.x & 31;
  for (int v = blockIdx.x * wpb + (threadIdx.x >> 5); v < g.n_virtual; v += gridDim.x * wpb)
  {
    const int     blk = g.vmap[2 * v], slot = g.vmap[2 * v + 1];
    const int     o[3] = {slot % 3 - 1, (slot / 3) % 3 - 1, slot / 9 - 1};
    const DRegion r = region_of(g, blk, o[0], o[1], o[2]);
    // near boxes: cells, then faces of each component
    int lo[4][3], len[4][3], cnt[4];
    for (int c = 0; c < 4; ++c)
    {
      cnt[c] = 1;
      for (int d = 0; d < 3; ++d)
      {
        if (d >= g.dim)
        {
          lo[c][d] = 0;
          len[c][d] = 1;
        }
        else
          near_range(o[d], b[d], c < 3 && c == d && !(g.dim == 2 && c == 2), lo[c][d], len[c][d]);
        cnt[c] *= len[c][d];
      }
    }
    // cnt[3] (cells) first, then faces x, y, z
    const int total = cnt[3] + cnt[0] + cnt[1] + cnt[2];
    for (int it = lane; it < total; it += 32)
    {
      if (it < cnt[3])
      {
        const int     q[3] = {lo[3][0] + it % len[3][0], lo[3][1] + (it / len[3][0]) % len[3][1],
                              lo[3][2] + it / (len[3][0] * len[3][1])};
        const int64_t item = q[0] + (int64_t)g.bx * (q[1] + (int64_t)g.by * q[2]);
        double        u[5] = {0, 0, 0, 0, 0}, bc[3] = {0, 0, 0};
        bool   ok = true;
        switch (r.kind)
        {
          case RK_SAME:
          case RK_OUTSIDE:
            for (int n = 0; n < 5; ++n)
              u[n] = u_at(g, r.id, n, q[0], q[1], q[2]);
            break;
          case RK_FINER:
            for (int n = 0; n < 5 && ok; ++n)
              ok = restrict_cell(g, r, q, n, u[n]);
            break;
          case RK_COARSER:
          {
            const int I[3] = {(r.sub[0] * b[0] + q[0]) >> 1, (r.sub[1] * b[1] + q[1]) >> 1, (r.sub[2] * b[2] + q[2]) >> 1};
            if (g.prolongation == 0)
            {
              // the coarse cell's own cell-centred B, from the coarse block's ghosted faces
              // (ConvertToPrimitivesVariablesFunctor.cpp:175-210 via fill_ghost_copy)
              for (int n = 0; n < 5; ++n)
                u[n] = u_at(g, r.id, n, I[0], I[1], I[2]);
              double fl[3] = {0, 0, 0}, fr[3] = {0, 0, 0};
              for (int c = 0; c < 3 && ok; ++c)
              {
                if (g.dim == 2 && c == 2)
                {
                  fl[2] = fr[2] = face_at(g, r.id, 2, I[0], I[1], 0);
                  continue;
                }
                int I1[3] = {I[0], I[1], I[2]};
                I1[c] += 1;
                ok = own_ghost_face(g, r.id, c, I[0], I[1], I[2], fl[c]) &&
                     own_ghost_face(g, r.id, c, I1[0], I1[1], I1[2], fr[c]);
              }
              bc[0] = 0.5 * (fl[0] + fr[0]);
              bc[1] = 0.5 * (fl[1] + fr[1]);
              bc[2] = 0.5 * (fl[2] + fr[2]);
            }
            else
            {
              const int sgn[3] = {2 * (q[0] & 1) - 1, 2 * (q[1] & 1) - 1, 2 * (q[2] & 1) - 1};
              for (int n = 0; n < 5 && ok; ++n)
              {
                const double uc = u_at(g, r.id, n, I[0], I[1], I[2]);
                double       sl[3] = {0, 0, 0};
                for (int d = 0; d < g.dim && ok; ++d)
                {
                  int    ip[3] = {I[0], I[1], I[2]}, im[3] = {I[0], I[1], I[2]};
                  double ur = 0.0, ul = 0.0;
                  ip[d] += 1;
                  im[d] -= 1;
                  ok = level_cell_value(g, r.id, n, ip[0], ip[1], ip[2], ur) &&
                       level_cell_value(g, r.id, n, im[0], im[1], im[2], ul);
                  sl[d] = minmod_slope(uc, ur, ul);
                }
                double val = uc + 0.25 * (double)sgn[0] * sl[0] + 0.25 * (double)sgn[1] * sl[1];
                if (g.dim == 3)
                  val = val + 0.25 * (double)sgn[2] * sl[2];
                u[n] = val;
              }
            }
            break;
          }
          default:
            ok = false;
        }
        if (!ok)
        {
          atomicOr(g.health, (unsigned)HEALTH_MISSING_NEIGHBOR);
          continue;
        }
        for (int n = 0; n < 5; ++n)
          g.Uv[((int64_t)v * 5 + n) * g.ncell + item] = u[n];
        for (int n = 0; n < 3; ++n)
          g.Bccv[((int64_t)v * 3 + n) * g.ncell + item] = bc[n];
        continue;
      }
      int comp = 0, f = it - cnt[3];
      while (f >= cnt[comp])
        f -= cnt[comp++];
      int q[3] = {lo[comp][0] + f % len[comp][0], lo[comp][1] + (f / len[comp][0]) % len[comp][1],
                  lo[comp][2] + f / (len[comp][0] * len[comp][1])};
      int64_t fi;
      if (comp == 0)
        fi = q[0] + (int64_t)(g.bx + 1) * (q[1] + (int64_t)g.by * q[2]);
      else if (comp == 1)
        fi = g.nfx + q[0] + (int64_t)g.bx * (q[1] + (int64_t)(g.by + 1) * q[2]);
      else
        fi = g.nfx + g.nfy + q[0] + (int64_t)g.bx * (q[1] + (int64_t)g.by * q[2]);
      const bool cellc = g.dim == 2 && comp == 2;
      // block-frame index and the region the block's gather assigns this face to
      int  idx[3] = {0, 0, 0};
      bool mine = true;
      for (int d = 0; d < g.dim; ++d)
      {
        idx[d] = o[d] * b[d] + q[d];
        const bool normal = d == comp && !cellc;
        if (idx[d] < -2 || idx[d] > (normal ? b[d] + 2 : b[d] + 1))
          mine = false;
        const int od = normal ? (idx[d] < 0 ? -1 : (idx[d] > b[d] ? 1 : 0)) : axis_off(idx[d], b[d]);
        if (od != o[d])
          mine = false;
      }
      // the block's own border face shared with a finer face neighbour is read from here too
      if (!mine && !cellc && r.kind == RK_FINER && o[comp] != 0 &&
          (o[0] != 0) + (o[1] != 0) + (o[2] != 0) == 1 && q[comp] == (o[comp] < 0 ? b[comp] : 0))
        mine = true;
      if (!mine)
        continue;
      DRegion rf = r;
      if (!cellc && (idx[comp] == 0 || idx[comp] == b[comp]))
      {
        int o1[3] = {o[0], o[1], o[2]};
        o1[comp] = idx[comp] == 0 ? -1 : 1;
        const DRegion r1 = region_of(g, blk, o1[0], o1[1], o1[2]);
        if (region_level(r1) > region_level(rf))
        {
          rf = r1;
          q[comp] = idx[comp] == 0 ? b[comp] : 0;
        }
      }
      double val = 0.0;
      if (!region_face(g, rf, comp, q, val))
      {
        atomicOr(g.health, (unsigned)HEALTH_MISSING_NEIGHBOR);
        continue;
      }
      g.Bv[(int64_t)v * g.nface + fi] = val;
    }
  }
}

int
launch_ghost_prepass(const GhostArgs & g, cudaStream_t stream)
{
  if (g.n_virtual <= 0)
    return 0;
  const int want = (g.n_virtual + 7) / 8; // 8 warps (virtual blocks) per CTA
  const int grid = want < 152 * 16 ? want : 152 * 16;
  ghost_prepass_kernel<<<grid, 256, 0, stream>>>(g);
  return (int)cudaGetLastError();
}

} // namespace gmhd

// ---- regrid: refinement indicator and remap ---------------------------------------------------
// Definitions as in the CPU restatement (kalypsso-core's ComputeRefineFlags / UserDataRemapper are not
// in the reference tree): indicator per cell and axis on rho and/or the pressure, neighbours clamped to
// the block, SIMPLE_GRADIENT max(|q+ - q|, |q - q-|) / max(|q|, DBL_MIN) or LOHNER_UNSPLIT
// |dp - dm| / (|dp| + |dm| + eps (|q+| + 2|q| + |q-|)); block error = max over cells.
namespace gmhd
{

// quantity 0 (rho) or 1 (pressure) of every owned cell, into q[var][block][cell]
__global__ void __launch_bounds__(256)
refine_quantity_kernel(const double * __restrict__ U, const double * __restrict__ B, int n_owned, int dim, int bx,
                       int by, int bz, int64_t ncell, int64_t nfx, int64_t nfy, int64_t nface, double gamma0,
                       double smallr, double smallp, int use_rho, int use_pressure, double * __restrict__ q)
{
  const int64_t total = (int64_t)n_owned * ncell;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x)
  {
    const int64_t blk = g / ncell, c = g - blk * ncell;
    const double *Ub = U + blk * 5 * ncell, *Bb = B + blk * nface;
    if (use_rho)
      q[g] = Ub[c];
    if (use_pressure)
    {
      const int    i = (int)(c % bx), j = (int)((c / bx) % by), k = (int)(c / ((int64_t)bx * by));
      const double Bxc = 0.5 * (Bb[i + (int64_t)(bx + 1) * (j + (int64_t)by * k)] + Bb[i + 1 + (int64_t)(bx + 1) * (j + (int64_t)by * k)]);
      const double Byc = 0.5 * (Bb[nfx + i + (int64_t)bx * (j + (int64_t)(by + 1) * k)] +
                                Bb[nfx + i + (int64_t)bx * (j + 1 + (int64_t)(by + 1) * k)]);
      const double Bzc = dim == 3 ? 0.5 * (Bb[nfx + nfy + c] + Bb[nfx + nfy + c + (int64_t)bx * by])
                                  : 0.5 * (Bb[nfx + nfy + c] + Bb[nfx + nfy + c]);
      // compute_primitives (models/mhd_utils.h:449-515), cIso == 0
      const double r = fmax(Ub[c], smallr);
      const double vx = Ub[2 * ncell + c] / r, vy = Ub[3 * ncell + c] / r, vz = Ub[4 * ncell + c] / r;
      const double eken = 0.5 * (vx * vx + vy * vy + vz * vz);
      const double emag = 0.5 * (Bxc * Bxc + Byc * Byc + Bzc * Bzc);
      const double eint = (Ub[ncell + c] - emag) / r - eken;
      q[total * (use_rho ? 1 : 0) + g] = fmax((gamma0 - 1.0) * r * eint, r * smallp);
    }
  }
}

__global__ void __launch_bounds__(256)
refine_flags_kernel(const double * __restrict__ q, int nvar, const int32_t * __restrict__ level, int n_owned, int dim,
                    int bx, int by, int bz, int64_t ncell, int criterion, int level_min, int level_max,
                    double eps_refine, double eps_coarsen, double eps_lohner, int8_t * __restrict__ flags)
{
  __shared__ double red[8];
  const int blk = blockIdx.x;
  const int b[3] = {bx, by, bz};
  double    err = 0.0;
  for (int var = 0; var < nvar; ++var)
  {
    const double * Q = q + ((int64_t)var * n_owned + blk) * ncell;
    for (int64_t c = threadIdx.x; c < ncell; c += blockDim.x)
    {
      const int    idx[3] = {(int)(c % bx), (int)((c / bx) % by), (int)(c / ((int64_t)bx * by))};
      const double v = Q[c];
      for (int d = 0; d < dim; ++d)
      {
        const int64_t st = d == 0 ? 1 : (d == 1 ? bx : (int64_t)bx * by);
        const double  qm = idx[d] > 0 ? Q[c - st] : v;
        const double  qp = idx[d] < b[d] - 1 ? Q[c + st] : v;
        double        e;
        if (criterion == 0)
          e = fmax(fabs(qp - v), fabs(v - qm)) / fmax(fabs(v), 2.2250738585072014e-308);
        else
        {
          const double dp = qp - v, dm = v - qm;
          const double den = fabs(dp) + fabs(dm) + eps_lohner * (fabs(qp) + 2.0 * fabs(v) + fabs(qm));
          e = den > 0.0 ? fabs(dp - dm) / den : 0.0;
        }
        err = fmax(err, e);
      }
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    err = fmax(err, __shfl_xor_sync(0xffffffffu, err, off));
  if ((threadIdx.x & 31) == 0)
    red[threadIdx.x >> 5] = err;
  __syncthreads();
  if (threadIdx.x == 0)
  {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      err = fmax(err, red[w]);
    const int lv = level[blk];
    flags[blk] = (err > eps_refine && lv < level_max) ? 1 : ((err < eps_coarsen && lv > level_min) ? -1 : 0);
  }
}

int
launch_refine_flags(const double * U, const double * B, const int32_t * level, int n_owned, int dim, int bx, int by,
                    int bz, int64_t ncell, int64_t nfx, int64_t nfy, int64_t nface, double gamma0, double smallr,
                    double smallp, int criterion, int level_min, int level_max, int use_rho, int use_pressure,
                    double eps_refine, double eps_coarsen, double eps_lohner, double * scratch, int8_t * flags,
                    cudaStream_t stream)
{
  if (n_owned <= 0)
    return 0;
  const int64_t total = (int64_t)n_owned * ncell;
  const int64_t want = (total + 255) / 256;
  refine_quantity_kernel<<<(int)(want < 152 * 64 ? want : 152 * 64), 256, 0, stream>>>(
    U, B, n_owned, dim, bx, by, bz, ncell, nfx, nfy, nface, gamma0, smallr, smallp, use_rho, use_pressure, scratch);
  refine_flags_kernel<<<n_owned, 256, 0, stream>>>(scratch, (use_rho ? 1 : 0) + (use_pressure ? 1 : 0), level, n_owned,
                                                   dim, bx, by, bz, ncell, criterion, level_min, level_max, eps_refine,
                                                   eps_coarsen, eps_lohner, flags);
  return (int)cudaGetLastError();
}

// Face of refined-leaf child rm (remap row) of the new mesh at block-local idx: the ghost prolongation
// of the parent, faces shared with a kept leaf copied from it, then the divergence corrections of the
// borders in the order -x, +x, -y, +y, -z, +z (the CPU restatement's prolonged_face).
__device__ static double
prolonged_face(const GhostArgs & g, const int32_t * rm, int comp, const int * idx)
{
  const int b[3] = {g.bx, g.by, g.bz};
  DRegion   r{RK_COARSER, rm[1], {rm[2] & 1, (rm[2] >> 1) & 1, (rm[2] >> 2) & 1}, nullptr};
  auto      base = [&](int c, const int * q) {
    double v = 0.0;
    region_face(g, r, c, q, v);
    return v;
  };
  auto border = [&](int c, const int * q, double & v) -> bool {
    if (g.dim == 2 && c == 2)
      return false;
    for (int sd = 0; sd < 2; ++sd)
    {
      const int nb = rm[9 + 2 * c + sd];
      if (nb < 0 || q[c] != (sd == 0 ? 0 : b[c]))
        continue;
      int qq[3] = {q[0], q[1], q[2]};
      qq[c] = sd == 0 ? b[c] : 0;
      v = face_at(g, nb, c, qq[0], qq[1], qq[2]);
      return true;
    }
    return false;
  };
  double val;
  if (!border(comp, idx, val))
    val = base(comp, idx);
  if (g.dim == 2 && comp == 2)
    return val;
  for (int n = 0; n < g.dim; ++n)
    for (int sd = 0; sd < 2; ++sd)
    {
      const int nb = rm[9 + 2 * n + sd];
      if (nb < 0 || comp == n)
        continue;
      const int p = sd == 0 ? 0 : b[n] - 1;
      if (idx[n] != p || (idx[comp] & 1) == 0)
        continue;
      const double sgn = sd == 0 ? 1.0 : -1.0;
      const int    t1 = n == 0 ? 1 : 0, t2 = n == 2 ? 1 : 2;
      const int    A = idx[t1] >> 1, Cc = g.dim == 3 ? (idx[t2] >> 1) : 0;
      double       d[2][2] = {{0, 0}, {0, 0}};
      for (int a = 0; a < 2; ++a)
        for (int c2 = 0; c2 < (g.dim == 3 ? 2 : 1); ++c2)
        {
          int q[3] = {0, 0, 0};
          q[n] = sd == 0 ? 0 : b[n];
          q[t1] = 2 * A + a;
          if (g.dim == 3)
            q[t2] = 2 * Cc + c2;
          double bv = 0.0;
          border(n, q, bv);
          d[a][c2] = bv - base(n, q);
        }
      if (g.dim == 2)
      {
        val += sgn * d[0][0];
        continue;
      }
      const double F = 0.5 * (d[0][0] + d[0][1]);
      if (comp == t1)
        val += sgn * F;
      else
      {
        const int a = idx[t1] & 1;
        val += sgn * (a == 0 ? d[0][0] - F : d[1][0] + F);
      }
    }
  return val;
}

// one CTA per new owned block
__global__ void __launch_bounds__(256)
remap_kernel(const GhostArgs g, const int32_t * __restrict__ remap, double * __restrict__ Un,
             double * __restrict__ Bn)
{
  const int       n = blockIdx.x;
  const int32_t * rm = remap + (int64_t)n * 15;
  const int       b[3] = {g.bx, g.by, g.bz};
  double *        Ub = Un + (int64_t)n * 5 * g.ncell;
  double *        Bb = Bn + (int64_t)n * g.nface;
  const int       kind = rm[0];
  if (kind == 0)
  {
    const double * Us = g.U + (int64_t)rm[1] * 5 * g.ncell;
    const double * Bs = g.B + (int64_t)rm[1] * g.nface;
    for (int64_t i = threadIdx.x; i < 5 * g.ncell; i += blockDim.x)
      Ub[i] = Us[i];
    for (int64_t i = threadIdx.x; i < g.nface; i += blockDim.x)
      Bb[i] = Bs[i];
    return;
  }
  const DRegion fine{RK_FINER, -1, {0, 0, 0}, rm + 1};
  for (int64_t c = threadIdx.x; c < g.ncell; c += blockDim.x)
  {
    const int q[3] = {(int)(c % g.bx), (int)((c / g.bx) % g.by), (int)(c / ((int64_t)g.bx * g.by))};
    for (int v = 0; v < 5; ++v)
    {
      double val = 0.0;
      if (kind == 2)
      {
        if (!restrict_cell(g, fine, q, v, val))
          atomicOr(g.health, (unsigned)HEALTH_MISSING_NEIGHBOR);
      }
      else
      {
        const int ch = rm[2];
        val = u_at(g, rm[1], v, ((ch & 1) * b[0] + q[0]) >> 1, (((ch >> 1) & 1) * b[1] + q[1]) >> 1,
                   g.dim == 3 ? ((((ch >> 2) & 1) * b[2] + q[2]) >> 1) : 0);
      }
      Ub[(int64_t)v * g.ncell + c] = val;
    }
  }
  for (int64_t fi = threadIdx.x; fi < g.nface; fi += blockDim.x)
  {
    int     comp, nx, ny;
    int64_t rr;
    if (fi < g.nfx)
    {
      comp = 0; rr = fi; nx = g.bx + 1; ny = g.by;
    }
    else if (fi < g.nfx + g.nfy)
    {
      comp = 1; rr = fi - g.nfx; nx = g.bx; ny = g.by + 1;
    }
    else
    {
      comp = 2; rr = fi - g.nfx - g.nfy; nx = g.bx; ny = g.by;
    }
    const int idx[3] = {(int)(rr % nx), (int)((rr / nx) % ny), (int)(rr / ((int64_t)nx * ny))};
    double    val = 0.0;
    if (kind == 2)
    {
      const int sd = (g.dim == 2 && comp == 2) ? -1 : (idx[comp] == 0 ? 0 : (idx[comp] == b[comp] ? 1 : -1));
      if (sd >= 0 && rm[9 + 2 * comp + sd] >= 0)
      {
        int qq[3] = {idx[0], idx[1], idx[2]};
        qq[comp] = sd == 0 ? b[comp] : 0;
        val = face_at(g, rm[9 + 2 * comp + sd], comp, qq[0], qq[1], qq[2]);
      }
      else if (!region_face(g, fine, comp, idx, val))
        atomicOr(g.health, (unsigned)HEALTH_MISSING_NEIGHBOR);
    }
    else
      val = prolonged_face(g, rm, comp, idx);
    Bb[fi] = val;
  }
}

int
launch_remap(const GhostArgs & g, const int32_t * remap, int n_new, double * Un, double * Bn, cudaStream_t stream)
{
  if (n_new <= 0)
    return 0;
  remap_kernel<<<n_new, 256, 0, stream>>>(g, remap, Un, Bn);
  return (int)cudaGetLastError();
}

} // namespace gmhd

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
//     (SIMPLE_COPY, with the coarse cell's own cell-centred B in Bcc) or adds 0.25 * (+-1) *
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
          const int id = r.child[c[0] + 2 * c[1] + 4 * c[2]];
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

// One CTA per virtual block (grid-stride), its threads over the cells and faces of the region's
// near layer.
__global__ void __launch_bounds__(256)
ghost_prepass_kernel(const GhostArgs g)
{
  const int b[3] = {g.bx, g.by, g.bz};
  for (int v = blockIdx.x; v < g.n_virtual; v += gridDim.x)
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
    for (int it = threadIdx.x; it < total; it += blockDim.x)
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
              for (int n = 0; n < 5; ++n)
                u[n] = u_at(g, r.id, n, I[0], I[1], I[2]);
              bc[0] = 0.5 * (face_at(g, r.id, 0, I[0], I[1], I[2]) + face_at(g, r.id, 0, I[0] + 1, I[1], I[2]));
              bc[1] = 0.5 * (face_at(g, r.id, 1, I[0], I[1], I[2]) + face_at(g, r.id, 1, I[0], I[1] + 1, I[2]));
              bc[2] = g.dim == 3
                        ? 0.5 * (face_at(g, r.id, 2, I[0], I[1], I[2]) + face_at(g, r.id, 2, I[0], I[1], I[2] + 1))
                        : 0.5 * (face_at(g, r.id, 2, I[0], I[1], 0) + face_at(g, r.id, 2, I[0], I[1], 0));
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
  const int grid = g.n_virtual < 152 * 32 ? g.n_virtual : 152 * 32;
  ghost_prepass_kernel<<<grid, 256, 0, stream>>>(g);
  return (int)cudaGetLastError();
}

} // namespace gmhd

// Oracle — test infrastructure only. Nothing in the product links, includes or calls this file;
// tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it as the checker.
//
// FP64 CPU restatement of godunov_mhd_ct's MUSCL-Hancock + constrained-transport stage
// (scheme/GodunovImplemV0.cpp:101-207) over a block mesh described by a neighbour table. It keeps
// the reference's stage order, per-stage arrays and summation order:
//   face-B ghost fill        scheme/GodunovImplemV0.cpp:211-237 (core FillBlockGhostFaces)
//   primitives + ghosts      scheme/ConvertToPrimitivesVariablesFunctor.cpp:173-719
//   limited slopes           scheme/ComputeLimitedSlopesFunctor.cpp:121-314
//   Hancock predictor        scheme/ComputeUpdatedPrimitiveVariablesFunctor.cpp:284-546
//   edge electric field      scheme/ComputeElectricFieldFunctor.cpp:97-235
//   face-B source term       scheme/ComputeSourceFaceMagFunctor.cpp:114-203
//   face fluxes + update     scheme/ComputeHydroFluxesAndStoreFunctor.cpp:118-503,
//                            scheme/ReadFluxesAndConservativeUpdateFunctor.cpp:103-436
//   edge EMFs                scheme/ComputeEmfAndStoreFunctor.cpp:103-590
//   EMF border correction    scheme/CorrectEmfAtBlockBorderFunctor.cpp:94-360
//   CT face-B update         scheme/ReadEmfAndUpdateFunctor.cpp:58-163
//   CFL                      scheme/ComputeDtMHDFunctor.cpp:86-151
//   outside-block fill       border_conditions/FillOutside.cpp:97-395
//
// Definitions where the reference relies on kalypsso-core (absent, so these are unpinned). The mesh
// is a 2:1-balanced (face, edge and corner) forest of equal-size blocks; the neighbour region of block
// b in direction o in {-1,0,1}^3 is the level-L(b) block-sized region next to b, and it is either a
// leaf at L (same), part of a leaf at L-1 (coarser), split into 2^d leaves at L+1 (finer), or an
// outside block at L (non-periodic borders).
//   * face-B ghost layer (core FillBlockGhostFacesFunctor): faces with normal index 0..b and
//     transverse cells inside the block are the block's own, except that a face shared with a finer
//     region takes that region's value (below); a same-level or outside region copies
//     the neighbour's face; a finer region takes the mean of the 2^(d-1) fine faces covering the face
//     (sum with the first transverse axis fastest, then divide); a coarser region takes the coarse
//     face containing the face when the face lies on a coarse face, else the mean of the two coarse
//     faces bounding the coarse cell along the normal. 2D Bz is cell-centred: mean of the 4 fine
//     cells (x fastest) / the coarse cell value. A face on the border between two regions along its
//     normal is taken from the finer one, so that all blocks see one value for every face;
//   * cell-centred hydro ghosts follow ConvertToPrimitivesVariablesFunctor.cpp:217-283, 471-719:
//     same level copies U and takes B_cc from the ghost faces (equal to the neighbour's faces when
//     shared faces agree), an outside block from its own faces (get_conservative_vars of the outside
//     cell); finer takes the mean of the 2^d fine cells (core compute_siblings_average:
//     x fastest, sum then divide) with B_cc from the ghost faces; coarser SIMPLE_COPY copies the
//     coarse cell's U and its B_cc from the coarse block's ghosted faces; EXTRAPOLATE_LINEAR_MINMOD adds
//     0.25 * (+-1) * minmod slope per axis (core compute_minmod_slopes: minmod(u - u_left,
//     u_right - u); neighbours at the coarse level, a refined one read as the mean of its fine cells,
//     a coarser one as its containing cell) with B_cc from the ghost faces;
//   * a coarse cell next to a finer face takes the sum of the 2^(d-1) fine face fluxes (core
//     compute_face_siblings_sum: first transverse axis fastest, from 0) / 2^d
//     (ReadFluxesAndConservativeUpdateFunctor.cpp:141-172);
//   * an edge on a block border has as siblings (core getEdgeSiblingLoc) the regions across its two
//     transverse block borders and across both: one across a block face, three around a block edge
//     (2D: block corner). Outside blocks count as valid siblings but are not averaged in, as in the
//     reference. A finer sibling's edge is the fine edge at the same place in the child touching it
//     (3D: the two fine sub-edges along the edge);
//   * dx = (1 / (bx * 2^level)) * scaling_factor.
//
// Compile with -ffp-contract=off.
#include "oracle_models.h"

#include <algorithm>
#include <cstring>
#include <vector>

namespace oracle
{

struct Mesh
{
  int             dim;
  int             bx, by, bz; // bz == 1 in 2D
  int             n_blocks;   // owned + outside
  int             n_owned;    // blocks [0, n_owned) are updated
  const int32_t * level;      // [n_blocks]
  const int32_t * neighbor;   // [n_blocks * 27]: same-level, coarser or outside block; -1 otherwise
  const int32_t * coord;      // [n_blocks * 3] block coordinates at the block's level, or null
  const int32_t * fine;       // [n_blocks * 27 * 8] children of a refined neighbour region, or null
  int             prolongation; // 0 SIMPLE_COPY, 1 EXTRAPOLATE_LINEAR_MINMOD
  double          scaling_factor;
};

static inline int
nb_slot(int ox, int oy, int oz)
{
  return (oz + 1) * 9 + (oy + 1) * 3 + (ox + 1);
}

// Sizes of the per-block SoA arrays (the C-ABI layout).
struct BlockLayout
{
  int64_t ncell;  // bx*by*bz
  int64_t nfx, nfy, nfz; // face counts per component (2D: nfz = ncell, cell-centred Bz)
  int64_t nface;  // nfx + nfy + nfz
};

static BlockLayout
block_layout(const Mesh & m)
{
  BlockLayout L;
  L.ncell = (int64_t)m.bx * m.by * m.bz;
  L.nfx = (int64_t)(m.bx + 1) * m.by * m.bz;
  L.nfy = (int64_t)m.bx * (m.by + 1) * m.bz;
  L.nfz = m.dim == 3 ? (int64_t)m.bx * m.by * (m.bz + 1) : L.ncell;
  L.nface = L.nfx + L.nfy + L.nfz;
  return L;
}

// Accessors to the caller's arrays. U: [block][var 0..4][k][j][i]; B: [block][Bx | By | Bz].
struct Fields
{
  const Mesh *  m;
  BlockLayout   L;
  const double *U;
  const double *B;

  double
  u(int blk, int var, int i, int j, int k) const
  {
    return U[(int64_t)blk * 5 * L.ncell + (int64_t)var * L.ncell + i + (int64_t)m->bx * (j + (int64_t)m->by * k)];
  }
  double
  bx(int blk, int i, int j, int k) const
  {
    return B[(int64_t)blk * L.nface + i + (int64_t)(m->bx + 1) * (j + (int64_t)m->by * k)];
  }
  double
  by(int blk, int i, int j, int k) const
  {
    return B[(int64_t)blk * L.nface + L.nfx + i + (int64_t)m->bx * (j + (int64_t)(m->by + 1) * k)];
  }
  double
  bz(int blk, int i, int j, int k) const
  {
    return B[(int64_t)blk * L.nface + L.nfx + L.nfy + i + (int64_t)m->bx * (j + (int64_t)m->by * k)];
  }
  double
  face(int blk, int comp, int i, int j, int k) const
  {
    return comp == 0 ? bx(blk, i, j, k) : (comp == 1 ? by(blk, i, j, k) : bz(blk, i, j, k));
  }
};

// A ghosted 3D index space [lo, lo + n) per axis, var-slowest.
struct Box
{
  int lo[3];
  int n[3];
  int nvar;
  std::vector<double> a;

  void
  init(int lx, int nx, int ly, int ny, int lz, int nz, int nv)
  {
    lo[0] = lx; n[0] = nx;
    lo[1] = ly; n[1] = ny;
    lo[2] = lz; n[2] = nz;
    nvar = nv;
    a.assign((size_t)nx * ny * nz * nv, 0.0);
  }
  double &
  operator()(int i, int j, int k, int v)
  {
    return a[(((size_t)v * n[2] + (k - lo[2])) * n[1] + (j - lo[1])) * n[0] + (i - lo[0])];
  }
};

// Neighbour-region classification (see the definitions at the top of this file).
enum RegionKind
{
  RK_MISSING = 0,
  RK_SAME = 1,
  RK_COARSER = 2,
  RK_FINER = 3,
  RK_OUTSIDE = 4
};

struct Region
{
  int             kind;
  int             id;     // same, outside, coarser: the block holding the region
  int             sub[3]; // coarser: position of the region inside the coarse block (0 or 1 per axis)
  const int32_t * child;  // finer: 8 children, x fastest (-1 where not a leaf)
};

static Region
region_of(const Mesh & m, int blk, int ox, int oy, int oz)
{
  Region r{RK_MISSING, -1, {0, 0, 0}, nullptr};
  if (ox == 0 && oy == 0 && oz == 0)
  {
    r.kind = RK_SAME;
    r.id = blk;
    return r;
  }
  const int64_t s = (int64_t)blk * 27 + nb_slot(ox, oy, oz);
  const int     id = m.neighbor[s];
  if (id >= 0)
  {
    r.id = id;
    if (id >= m.n_owned)
      r.kind = RK_OUTSIDE;
    else if (m.level[id] == m.level[blk])
      r.kind = RK_SAME;
    else if (m.level[id] == m.level[blk] - 1 && m.coord)
    {
      r.kind = RK_COARSER;
      const int o[3] = {ox, oy, oz};
      for (int d = 0; d < m.dim; ++d)
        r.sub[d] = (m.coord[(int64_t)blk * 3 + d] + o[d]) & 1;
    }
    return r;
  }
  if (m.fine)
  {
    const int32_t * ch = m.fine + s * 8;
    for (int c = 0; c < (1 << m.dim); ++c)
      if (ch[c] >= 0)
      {
        r.kind = RK_FINER;
        r.child = ch;
        break;
      }
  }
  return r;
}

static inline int
region_axis(int idx, int n)
{
  return idx < 0 ? -1 : (idx >= n ? 1 : 0);
}

struct StepWork
{
  // per block, per thread
  Box Bgx, Bgy, Bgz; // ghosted faces (2D: Bgz is cell-centred Bz)
  Box Q;             // 11 vars on [-2, b+2)
  Box Sx, Sy, Sz;    // slopes, 8 vars on [-1, b+1)
  Box Q2;            // 8 vars on [-1, b+1)
  Box E;             // 3 (2D: 1) comps on [-2, b+2)
  Box SF;            // 3 (2D: 2) comps on [-1, b+1)
};

static double
slope_scalar(double q, double qp, double qm, const Settings & s)
{
  // slope_unsplit_scalar (scheme/ComputeLimitedSlopesFunctor.cpp:121-144)
  const double slope_type = s.slope_type;
  double       dq = 0;
  if (slope_type == 1 or slope_type == 2)
  {
    const double dlft = slope_type * (q - qm);
    const double drgt = slope_type * (qp - q);
    const double dcen = 0.5 * (qp - qm);
    const double dsgn = (dcen >= 0.0) ? 1.0 : -1.0;
    const double slop = std::fmin(std::fabs(dlft), std::fabs(drgt));
    const double dlim = (dlft * drgt) <= 0.0 ? 0.0 : slop;
    dq = dsgn * std::fmin(dlim, std::fabs(dcen));
  }
  return dq;
}

// Level of a neighbour region relative to the block (missing regions rank below everything).
static int
region_level(const Region & r)
{
  return r.kind == RK_COARSER ? -1 : (r.kind == RK_FINER ? 1 : (r.kind == RK_MISSING ? -100 : 0));
}

// Face value of component comp at q (region-local indices) of neighbour region r.
static bool
region_face(const Mesh & m, const Fields & f, const Region & r, int comp, const int * q, double & out)
{
  const int  b[3] = {m.bx, m.by, m.bz};
  const bool cellc = m.dim == 2 && comp == 2;
  switch (r.kind)
  {
    case RK_SAME:
    case RK_OUTSIDE:
      out = f.face(r.id, comp, q[0], q[1], q[2]);
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
            acc += f.bz(id, F0 - c0 * b[0], F1 - c1 * b[1], 0);
          }
        out = acc / 4.0;
        return true;
      }
      const int t1 = comp == 0 ? 1 : 0;
      const int t2 = comp == 2 ? 1 : 2;
      const int n2 = m.dim == 3 ? 2 : 1;
      for (int e2 = 0; e2 < n2; ++e2)
        for (int e1 = 0; e1 < 2; ++e1)
        {
          int F[3] = {0, 0, 0}, c[3] = {0, 0, 0};
          F[comp] = 2 * q[comp];
          c[comp] = F[comp] >= b[comp];
          F[t1] = 2 * q[t1] + e1;
          c[t1] = F[t1] >= b[t1];
          if (m.dim == 3)
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
          acc += f.face(id, comp, F[0] - c[0] * b[0], F[1] - c[1] * b[1], F[2] - c[2] * b[2]);
        }
      out = acc / (m.dim == 3 ? 4.0 : 2.0);
      return true;
    }
    case RK_COARSER:
    {
      int F[3] = {0, 0, 0};
      for (int d = 0; d < m.dim; ++d)
        F[d] = r.sub[d] * b[d] + q[d];
      if (cellc)
      {
        out = f.bz(r.id, F[0] >> 1, F[1] >> 1, 0);
        return true;
      }
      int T[3] = {F[0] >> 1, F[1] >> 1, F[2] >> 1};
      if ((F[comp] & 1) == 0)
      {
        T[comp] = F[comp] / 2;
        out = f.face(r.id, comp, T[0], T[1], T[2]);
      }
      else
      {
        int T1[3] = {T[0], T[1], T[2]};
        T[comp] = (F[comp] - 1) / 2;
        T1[comp] = (F[comp] + 1) / 2;
        out = 0.5 * (f.face(r.id, comp, T[0], T[1], T[2]) + f.face(r.id, comp, T1[0], T1[1], T1[2]));
      }
      return true;
    }
    default:
      return false;
  }
}

// Value of face component comp at (i, j, k) of block blk's ghosted face space (2D comp 2: the
// cell-centred Bz), following the face-B ghost definition at the top of this file. A face lying on
// the border between two regions along its normal (the block itself included) is taken from the
// finer of the two (the first when they are at the same level), so every block sees the same value
// for it. Returns false when the neighbour region is missing.
static bool
ghost_face(const Mesh & m, const Fields & f, int blk, int comp, int i, int j, int k, double & out)
{
  const int  b[3] = {m.bx, m.by, m.bz};
  const bool cellc = m.dim == 2 && comp == 2;
  const int  idx[3] = {i, j, k};
  int        o[3] = {0, 0, 0};
  for (int d = 0; d < m.dim; ++d)
    o[d] = (d == comp && !cellc) ? (idx[d] < 0 ? -1 : (idx[d] > b[d] ? 1 : 0)) : region_axis(idx[d], b[d]);
  Region r = region_of(m, blk, o[0], o[1], o[2]);
  int    q[3] = {idx[0] - o[0] * b[0], idx[1] - o[1] * b[1], idx[2] - o[2] * b[2]};
  if (!cellc && (idx[comp] == 0 || idx[comp] == b[comp]))
  {
    int o1[3] = {o[0], o[1], o[2]};
    o1[comp] = idx[comp] == 0 ? -1 : 1;
    const Region r1 = region_of(m, blk, o1[0], o1[1], o1[2]);
    if (region_level(r1) > region_level(r))
    {
      r = r1;
      q[comp] = idx[comp] == 0 ? b[comp] : 0;
    }
  }
  return region_face(m, f, r, comp, q, out);
}

// Fill ghosted face-B for block blk (GodunovImplemV0.cpp:211-237). Returns 0 or -1 when a needed
// neighbour is missing.
static int
fill_bface_ghosted(const Mesh & m, const Fields & f, int blk, StepWork & w)
{
  const int g = 2;
  const int gz = m.dim == 3 ? 2 : 0;
  w.Bgx.init(-g, m.bx + 2 * g + 1, -g, m.by + 2 * g, -gz, m.bz + 2 * gz, 1);
  w.Bgy.init(-g, m.bx + 2 * g, -g, m.by + 2 * g + 1, -gz, m.bz + 2 * gz, 1);
  if (m.dim == 3)
    w.Bgz.init(-g, m.bx + 2 * g, -g, m.by + 2 * g, -gz, m.bz + 2 * gz + 1, 1);
  else
    w.Bgz.init(-g, m.bx + 2 * g, -g, m.by + 2 * g, 0, 1, 1);
  Box * box[3] = {&w.Bgx, &w.Bgy, &w.Bgz};
  for (int c = 0; c < 3; ++c)
  {
    Box & bb = *box[c];
    for (int k = bb.lo[2]; k < bb.lo[2] + bb.n[2]; ++k)
      for (int j = bb.lo[1]; j < bb.lo[1] + bb.n[1]; ++j)
        for (int i = bb.lo[0]; i < bb.lo[0] + bb.n[0]; ++i)
          if (!ghost_face(m, f, blk, c, i, j, k, bb(i, j, k, 0)))
            return -1;
  }
  return 0;
}

// Mean of the 2^d fine cells of variable v covering cell q of a finer region (core
// compute_siblings_average: x fastest, sum then divide).
static bool
restrict_cell(const Mesh & m, const Fields & f, const Region & r, const int * q, int v, double & out)
{
  const int b[3] = {m.bx, m.by, m.bz};
  double    acc = 0.0;
  for (int ez = 0; ez < (m.dim == 3 ? 2 : 1); ++ez)
    for (int ey = 0; ey < 2; ++ey)
      for (int ex = 0; ex < 2; ++ex)
      {
        const int F[3] = {2 * q[0] + ex, 2 * q[1] + ey, m.dim == 3 ? 2 * q[2] + ez : 0};
        const int c[3] = {F[0] >= b[0], F[1] >= b[1], F[2] >= b[2]};
        const int id = r.child[c[0] + 2 * c[1] + 4 * c[2]];
        if (id < 0)
          return false;
        acc += f.u(id, v, F[0] - c[0] * b[0], F[1] - c[1] * b[1], F[2] - c[2] * b[2]);
      }
  out = acc / (double)(1 << m.dim);
  return true;
}

// Conservative variable v of cell (i, j, k) at block blk's level, at most one block away: same
// level or outside reads the cell, a refined region its fine-cell mean, a coarser one its containing
// cell.
static bool
level_cell_value(const Mesh & m, const Fields & f, int blk, int v, int i, int j, int k, double & out)
{
  const int    b[3] = {m.bx, m.by, m.bz};
  const int    o[3] = {region_axis(i, m.bx), region_axis(j, m.by), m.dim == 3 ? region_axis(k, m.bz) : 0};
  const Region r = region_of(m, blk, o[0], o[1], o[2]);
  const int    q[3] = {i - o[0] * b[0], j - o[1] * b[1], k - o[2] * b[2]};
  switch (r.kind)
  {
    case RK_SAME:
    case RK_OUTSIDE:
      out = f.u(r.id, v, q[0], q[1], q[2]);
      return true;
    case RK_FINER:
      return restrict_cell(m, f, r, q, v, out);
    case RK_COARSER:
      out = f.u(r.id, v, (r.sub[0] * b[0] + q[0]) >> 1, (r.sub[1] * b[1] + q[1]) >> 1,
                (r.sub[2] * b[2] + q[2]) >> 1);
      return true;
    default:
      return false;
  }
}

// core compute_minmod_slopes with slope_type 1
static double
minmod_slope(double u, double ur, double ul)
{
  const double dl = u - ul, dr = ur - u;
  if (dl * dr <= 0.0)
    return 0.0;
  return dl > 0.0 ? std::fmin(dl, dr) : std::fmax(dl, dr);
}

// Primitive variables on the (b+4)^d ghosted block (ConvertToPrimitivesVariablesFunctor).
static int
convert_to_primitives(const Mesh & m, const Fields & f, const Settings & s, int blk, StepWork & w)
{
  const int g = 2;
  const int gz = m.dim == 3 ? 2 : 0;
  w.Q.init(-g, m.bx + 2 * g, -g, m.by + 2 * g, -gz, m.bz + 2 * gz, 11);
  for (int k = -gz; k < m.bz + gz; ++k)
    for (int j = -g; j < m.by + g; ++j)
      for (int i = -g; i < m.bx + g; ++i)
      {
        const int    o[3] = {region_axis(i, m.bx), region_axis(j, m.by), m.dim == 3 ? region_axis(k, m.bz) : 0};
        const Region r = region_of(m, blk, o[0], o[1], o[2]);
        const int    qc[3] = {i - o[0] * m.bx, j - o[1] * m.by, k - o[2] * m.bz};
        const int *  q = qc;
        double       u[8];
        bool         bcc_from_ghost_faces = true;
        switch (r.kind)
        {
          case RK_SAME:
          case RK_OUTSIDE:
            // fill_inner / fill_ghost_copy at the same level (.cpp:373-468)
            for (int v = 0; v < 5; ++v)
              u[v] = f.u(r.id, v, q[0], q[1], q[2]);
            if (r.kind == RK_OUTSIDE)
            {
              // get_conservative_vars(cell_loc_in) reads B_cc from the outside block's own faces, whose
              // copy of the shared border face is FillOutside's (a WALL copies the same face index)
              u[IA] = 0.5 * (f.bx(r.id, q[0], q[1], q[2]) + f.bx(r.id, q[0] + 1, q[1], q[2]));
              u[IB] = 0.5 * (f.by(r.id, q[0], q[1], q[2]) + f.by(r.id, q[0], q[1] + 1, q[2]));
              if (m.dim == 3)
                u[IC] = 0.5 * (f.bz(r.id, q[0], q[1], q[2]) + f.bz(r.id, q[0], q[1], q[2] + 1));
              else
                u[IC] = 0.5 * (f.bz(r.id, q[0], q[1], 0) + f.bz(r.id, q[0], q[1], 0));
              bcc_from_ghost_faces = false;
            }
            break;
          case RK_FINER:
            // get_conservative_vars_restriction (.cpp:217-283)
            for (int v = 0; v < 5; ++v)
              if (!restrict_cell(m, f, r, q, v, u[v]))
                return -1;
            break;
          case RK_COARSER:
          {
            const int I[3] = {(r.sub[0] * m.bx + q[0]) >> 1, (r.sub[1] * m.by + q[1]) >> 1,
                              (r.sub[2] * m.bz + q[2]) >> 1};
            if (m.prolongation == 0)
            {
              // SIMPLE_COPY: fill_ghost_copy of the coarse cell with its own B_cc (.cpp:439-446), read
              // from the coarse block's ghosted faces (a border face shared with a finer region is
              // that region's)
              for (int v = 0; v < 5; ++v)
                u[v] = f.u(r.id, v, I[0], I[1], I[2]);
              double fl[3], fr[3];
              for (int c = 0; c < 3; ++c)
              {
                if (m.dim == 2 && c == 2)
                {
                  if (!ghost_face(m, f, r.id, 2, I[0], I[1], 0, fl[2]))
                    return -1;
                  fr[2] = fl[2];
                  continue;
                }
                int I1[3] = {I[0], I[1], I[2]};
                I1[c] += 1;
                if (!ghost_face(m, f, r.id, c, I[0], I[1], I[2], fl[c]) ||
                    !ghost_face(m, f, r.id, c, I1[0], I1[1], I1[2], fr[c]))
                  return -1;
              }
              u[IA] = 0.5 * (fl[0] + fr[0]);
              u[IB] = 0.5 * (fl[1] + fr[1]);
              u[IC] = 0.5 * (fl[2] + fr[2]);
              bcc_from_ghost_faces = false;
            }
            else
            {
              // EXTRAPOLATE_LINEAR_MINMOD (.cpp:471-635): position of this cell inside the coarse
              // cell in {-1, +1} per axis, slopes at the coarse level
              const int sgn[3] = {2 * (q[0] & 1) - 1, 2 * (q[1] & 1) - 1, 2 * (q[2] & 1) - 1};
              for (int v = 0; v < 5; ++v)
              {
                const double uc = f.u(r.id, v, I[0], I[1], I[2]);
                double       sl[3] = {0, 0, 0};
                for (int d = 0; d < m.dim; ++d)
                {
                  int    ip[3] = {I[0], I[1], I[2]}, im[3] = {I[0], I[1], I[2]};
                  double ur, ul;
                  ip[d] += 1;
                  im[d] -= 1;
                  if (!level_cell_value(m, f, r.id, v, ip[0], ip[1], ip[2], ur) ||
                      !level_cell_value(m, f, r.id, v, im[0], im[1], im[2], ul))
                    return -1;
                  sl[d] = minmod_slope(uc, ur, ul);
                }
                double val = uc + 0.25 * (double)sgn[0] * sl[0] + 0.25 * (double)sgn[1] * sl[1];
                if (m.dim == 3)
                  val = val + 0.25 * (double)sgn[2] * sl[2];
                u[v] = val;
              }
            }
            break;
          }
          default:
            return -1;
        }
        if (bcc_from_ghost_faces)
        {
          // cell-centred B from face values (get_conservative_vars, .cpp:175-210)
          u[IA] = 0.5 * (w.Bgx(i, j, k, 0) + w.Bgx(i + 1, j, k, 0));
          u[IB] = 0.5 * (w.Bgy(i, j, k, 0) + w.Bgy(i, j + 1, k, 0));
          if (m.dim == 3)
            u[IC] = 0.5 * (w.Bgz(i, j, k, 0) + w.Bgz(i, j, k + 1, 0));
          else
            u[IC] = 0.5 * (w.Bgz(i, j, 0, 0) + w.Bgz(i, j, 0, 0));
        }
        double qp[8];
        compute_primitives(u, qp, nullptr, s);
        w.Q(i, j, k, ID) = qp[ID];
        w.Q(i, j, k, IP) = qp[IP];
        w.Q(i, j, k, IU) = qp[IU];
        w.Q(i, j, k, IV) = qp[IV];
        w.Q(i, j, k, IW) = qp[IW];
        // face values (get_face_mag, .cpp:287-369)
        w.Q(i, j, k, IA) = w.Bgx(i, j, k, 0);
        w.Q(i, j, k, IAR) = w.Bgx(i + 1, j, k, 0);
        w.Q(i, j, k, IB) = w.Bgy(i, j, k, 0);
        w.Q(i, j, k, IBR) = w.Bgy(i, j + 1, k, 0);
        if (m.dim == 3)
        {
          w.Q(i, j, k, IC) = w.Bgz(i, j, k, 0);
          w.Q(i, j, k, ICR) = w.Bgz(i, j, k + 1, 0);
        }
        else
        {
          w.Q(i, j, k, IC) = w.Bgz(i, j, 0, 0);
          w.Q(i, j, k, ICR) = w.Bgz(i, j, 0, 0);
        }
      }
  return 0;
}

// slope_unsplit_scalar_mag (scheme/ComputeLimitedSlopesFunctor.cpp:148-221)
static double
slope_mag(StepWork & w, int i, int j, int k, int dir, int v1, int v2, const Settings & s)
{
  const bool normal = (v1 == IA && dir == 0) || (v1 == IB && dir == 1) || (v1 == IC && dir == 2);
  if (normal)
    return w.Q(i, j, k, v2) - w.Q(i, j, k, v1);
  const int di = dir == 0, dj = dir == 1, dk = dir == 2;
  const double datac = (w.Q(i, j, k, v1) + w.Q(i, j, k, v2)) * 0.5;
  const double datap = (w.Q(i + di, j + dj, k + dk, v1) + w.Q(i + di, j + dj, k + dk, v2)) * 0.5;
  const double datam = (w.Q(i - di, j - dj, k - dk, v1) + w.Q(i - di, j - dj, k - dk, v2)) * 0.5;
  return slope_scalar(datac, datap, datam, s);
}

static void
compute_slopes(const Mesh & m, const Settings & s, StepWork & w)
{
  const int g = 1;
  const int gz = m.dim == 3 ? 1 : 0;
  w.Sx.init(-g, m.bx + 2 * g, -g, m.by + 2 * g, -gz, m.bz + 2 * gz, 8);
  w.Sy.init(-g, m.bx + 2 * g, -g, m.by + 2 * g, -gz, m.bz + 2 * gz, 8);
  w.Sz.init(-g, m.bx + 2 * g, -g, m.by + 2 * g, -gz, m.bz + 2 * gz, 8);
  const int nhydro = m.dim == 3 ? 5 : 4; // nbvar_hydro_only<dim>() (models/MHDState.h:36-43)
  for (int k = -gz; k < m.bz + gz; ++k)
    for (int j = -g; j < m.by + g; ++j)
      for (int i = -g; i < m.bx + g; ++i)
      {
        for (int v = 0; v < nhydro; ++v)
        {
          w.Sx(i, j, k, v) = slope_scalar(w.Q(i, j, k, v), w.Q(i + 1, j, k, v), w.Q(i - 1, j, k, v), s);
          w.Sy(i, j, k, v) = slope_scalar(w.Q(i, j, k, v), w.Q(i, j + 1, k, v), w.Q(i, j - 1, k, v), s);
          if (m.dim == 3)
            w.Sz(i, j, k, v) =
              slope_scalar(w.Q(i, j, k, v), w.Q(i, j, k + 1, v), w.Q(i, j, k - 1, v), s);
        }
        w.Sx(i, j, k, IA) = slope_mag(w, i, j, k, 0, IA, IAR, s);
        w.Sy(i, j, k, IA) = slope_mag(w, i, j, k, 1, IA, IAR, s);
        w.Sx(i, j, k, IB) = slope_mag(w, i, j, k, 0, IB, IBR, s);
        w.Sy(i, j, k, IB) = slope_mag(w, i, j, k, 1, IB, IBR, s);
        w.Sx(i, j, k, IC) = slope_mag(w, i, j, k, 0, IC, ICR, s);
        w.Sy(i, j, k, IC) = slope_mag(w, i, j, k, 1, IC, ICR, s);
        if (m.dim == 3)
        {
          w.Sz(i, j, k, IA) = slope_mag(w, i, j, k, 2, IA, IAR, s);
          w.Sz(i, j, k, IB) = slope_mag(w, i, j, k, 2, IB, IBR, s);
          w.Sz(i, j, k, IC) = slope_mag(w, i, j, k, 2, IC, ICR, s);
        }
      }
}

// update_primitive_variables, Hancock branch (scheme/ComputeUpdatedPrimitiveVariablesFunctor.cpp:284-546)
// Viscous force predictor (ComputeUpdatedPrimitiveVariablesFunctor.cpp:174-280): velocity component
// `var` at cell (i, j, k) gets half a step of nu * Laplacian, one axis after the other; nu = mu / rho
// of the cell's primitive density.
static double
viscous_predictor(const Mesh & m, const Settings & s, StepWork & w, int i, int j, int k, int var, double dtdx,
                  double dx, double vel)
{
  const double nu = s.mu / w.Q(i, j, k, ID);
  const double q0 = w.Q(i, j, k, var);
  const double d2x = w.Q(i + 1, j, k, var) + w.Q(i - 1, j, k, var) - 2 * q0;
  vel += 0.5 * nu * d2x / dx * dtdx;
  const double d2y = w.Q(i, j + 1, k, var) + w.Q(i, j - 1, k, var) - 2 * q0;
  vel += 0.5 * nu * d2y / dx * dtdx;
  if (m.dim == 3)
  {
    const double d2z = w.Q(i, j, k + 1, var) + w.Q(i, j, k - 1, var) - 2 * q0;
    vel += 0.5 * nu * d2z / dx * dtdx;
  }
  return vel;
}

static void
compute_predictor(const Mesh & m, const Settings & s, double dt, double dtdx, double dx, StepWork & w)
{
  const int g = 1;
  const int gz = m.dim == 3 ? 1 : 0;
  w.Q2.init(-g, m.bx + 2 * g, -g, m.by + 2 * g, -gz, m.bz + 2 * gz, 8);
  const double gamma = s.gamma0;
  const double dtdy = dtdx, dtdz = dtdx;
  for (int k = -gz; k < m.bz + gz; ++k)
    for (int j = -g; j < m.by + g; ++j)
      for (int i = -g; i < m.bx + g; ++i)
      {
        const double r = w.Q(i, j, k, ID);
        const double p = w.Q(i, j, k, IP);
        double       u = w.Q(i, j, k, IU);
        double       v = w.Q(i, j, k, IV);
        double       ww = w.Q(i, j, k, IW);
        const double A = (w.Q(i, j, k, IA) + w.Q(i, j, k, IAR)) * 0.5;
        const double B = (w.Q(i, j, k, IB) + w.Q(i, j, k, IBR)) * 0.5;
        const double C = (w.Q(i, j, k, IC) + w.Q(i, j, k, ICR)) * 0.5;
        const double drx = w.Sx(i, j, k, ID), dpx = w.Sx(i, j, k, IP), dux = w.Sx(i, j, k, IU),
                     dvx = w.Sx(i, j, k, IV), dwx = w.Sx(i, j, k, IW), dAx = w.Sx(i, j, k, IA),
                     dBx = w.Sx(i, j, k, IB), dCx = w.Sx(i, j, k, IC);
        const double dry = w.Sy(i, j, k, ID), dpy = w.Sy(i, j, k, IP), duy = w.Sy(i, j, k, IU),
                     dvy = w.Sy(i, j, k, IV), dwy = w.Sy(i, j, k, IW), dAy = w.Sy(i, j, k, IA),
                     dBy = w.Sy(i, j, k, IB), dCy = w.Sy(i, j, k, IC);
        double sr0, su0, sv0, sw0, sp0, sA0, sB0, sC0;
        if (m.dim == 2)
        {
          sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy;
          su0 = (-u * dux - dpx / r - B * dBx / r - C * dCx / r) * dtdx + (-v * duy + B * dAy / r) * dtdy;
          sv0 = (-u * dvx + A * dBx / r) * dtdx + (-v * dvy - dpy / r - A * dAy / r - C * dCy / r) * dtdy;
          sw0 = (-u * dwx + A * dCx / r) * dtdx + (-v * dwy + B * dCy / r) * dtdy;
          sp0 = (-u * dpx - dux * gamma * p) * dtdx + (-v * dpy - dvy * gamma * p) * dtdy;
          sA0 = (u * dBy + B * duy - v * dAy - A * dvy) * dtdy;
          sB0 = (-u * dBx - B * dux + v * dAx + A * dvx) * dtdx;
          sC0 = (ww * dAx + A * dwx - u * dCx - C * dux) * dtdx + (-v * dCy - C * dvy + ww * dBy + B * dwy) * dtdy;
        }
        else
        {
          const double drz = w.Sz(i, j, k, ID), dpz = w.Sz(i, j, k, IP), duz = w.Sz(i, j, k, IU),
                       dvz = w.Sz(i, j, k, IV), dwz = w.Sz(i, j, k, IW), dAz = w.Sz(i, j, k, IA),
                       dBz = w.Sz(i, j, k, IB), dCz = w.Sz(i, j, k, IC);
          sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy + (-ww * drz - dwz * r) * dtdz;
          su0 = (-u * dux - (dpx + B * dBx + C * dCx) / r) * dtdx + (-v * duy + B * dAy / r) * dtdy +
                (-ww * duz + C * dAz / r) * dtdz;
          sv0 = (-u * dvx + A * dBx / r) * dtdx + (-v * dvy - (dpy + A * dAy + C * dCy) / r) * dtdy +
                (-ww * dvz + C * dBz / r) * dtdz;
          sw0 = (-u * dwx + A * dCx / r) * dtdx + (-v * dwy + B * dCy / r) * dtdy +
                (-ww * dwz - (dpz + A * dAz + B * dBz) / r) * dtdz;
          sp0 = (-u * dpx - dux * gamma * p) * dtdx + (-v * dpy - dvy * gamma * p) * dtdy +
                (-ww * dpz - dwz * gamma * p) * dtdz;
          sA0 = (u * dBy + B * duy - v * dAy - A * dvy) * dtdy + (u * dCz + C * duz - ww * dAz - A * dwz) * dtdz;
          sB0 = (v * dAx + A * dvx - u * dBx - B * dux) * dtdx + (v * dCz + C * dvz - ww * dBz - B * dwz) * dtdz;
          sC0 = (ww * dAx + A * dwx - u * dCx - C * dux) * dtdx + (ww * dBy + B * dwy - v * dCy - C * dvy) * dtdy;
        }
        if (s.rk2)
        {
          // RK2_SSP: no Hancock half step (ComputeUpdatedPrimitiveVariablesFunctor.cpp:396-407, 531-542)
          w.Q2(i, j, k, ID) = r;
          w.Q2(i, j, k, IU) = u;
          w.Q2(i, j, k, IV) = v;
          w.Q2(i, j, k, IW) = ww;
          w.Q2(i, j, k, IP) = p;
          w.Q2(i, j, k, IA) = A;
          w.Q2(i, j, k, IB) = B;
          w.Q2(i, j, k, IC) = C;
          continue;
        }
        // half-step gravity kick and viscous predictor on the velocity, after the sources
        // (ComputeUpdatedPrimitiveVariablesFunctor.cpp:372-383, 505-517)
        if (s.gravity)
        {
          u += s.grav[0] * 0.5 * dt;
          v += s.grav[1] * 0.5 * dt;
          if (m.dim == 3)
            ww += s.grav[2] * 0.5 * dt;
        }
        if (s.viscosity && s.visc_predictor)
        {
          u = viscous_predictor(m, s, w, i, j, k, IU, dtdx, dx, u);
          v = viscous_predictor(m, s, w, i, j, k, IV, dtdx, dx, v);
          if (m.dim == 3)
            ww = viscous_predictor(m, s, w, i, j, k, IW, dtdx, dx, ww);
        }
        w.Q2(i, j, k, ID) = r + 0.5 * sr0;
        w.Q2(i, j, k, IU) = u + 0.5 * su0;
        w.Q2(i, j, k, IV) = v + 0.5 * sv0;
        w.Q2(i, j, k, IW) = ww + 0.5 * sw0;
        w.Q2(i, j, k, IP) = p + 0.5 * sp0;
        w.Q2(i, j, k, IA) = A + 0.5 * sA0;
        w.Q2(i, j, k, IB) = B + 0.5 * sB0;
        w.Q2(i, j, k, IC) = C + 0.5 * sC0;
      }
}

// compute_elec_field (scheme/ComputeElectricFieldFunctor.cpp:97-235)
static void
compute_elec_field(const Mesh & m, StepWork & w)
{
  const int g = 2;
  const int gz = m.dim == 3 ? 2 : 0;
  w.E.init(-g, m.bx + 2 * g, -g, m.by + 2 * g, -gz, m.bz + 2 * gz, m.dim == 3 ? 3 : 1);
  Box & q = w.Q;
  for (int k = -gz; k < m.bz + gz; ++k)
    for (int j = -g; j < m.by + g; ++j)
      for (int i = -g; i < m.bx + g; ++i)
      {
        if (m.dim == 2)
        {
          if (i > -2 && j > -2)
          {
            const double u = 0.25 * (q(i - 1, j - 1, 0, IU) + q(i - 1, j, 0, IU) + q(i, j - 1, 0, IU) + q(i, j, 0, IU));
            const double v = 0.25 * (q(i - 1, j - 1, 0, IV) + q(i - 1, j, 0, IV) + q(i, j - 1, 0, IV) + q(i, j, 0, IV));
            const double A = 0.5 * (q(i, j - 1, 0, IA) + q(i, j, 0, IA));
            const double B = 0.5 * (q(i - 1, j, 0, IB) + q(i, j, 0, IB));
            w.E(i, j, 0, 0) = u * B - v * A;
          }
        }
        else if (i > -2 && j > -2 && k > -2)
        {
          {
            const double v = 0.25 * (q(i, j - 1, k - 1, IV) + q(i, j - 1, k, IV) + q(i, j, k - 1, IV) + q(i, j, k, IV));
            const double ww = 0.25 * (q(i, j - 1, k - 1, IW) + q(i, j - 1, k, IW) + q(i, j, k - 1, IW) + q(i, j, k, IW));
            const double B = 0.5 * (q(i, j, k - 1, IB) + q(i, j, k, IB));
            const double C = 0.5 * (q(i, j - 1, k, IC) + q(i, j, k, IC));
            w.E(i, j, k, 0) = v * C - ww * B;
          }
          {
            const double u = 0.25 * (q(i - 1, j, k - 1, IU) + q(i - 1, j, k, IU) + q(i, j, k - 1, IU) + q(i, j, k, IU));
            const double ww = 0.25 * (q(i - 1, j, k - 1, IW) + q(i - 1, j, k, IW) + q(i, j, k - 1, IW) + q(i, j, k, IW));
            const double A = 0.5 * (q(i, j, k - 1, IA) + q(i, j, k, IA));
            const double C = 0.5 * (q(i - 1, j, k, IC) + q(i, j, k, IC));
            w.E(i, j, k, 1) = ww * A - u * C;
          }
          {
            const double u = 0.25 * (q(i - 1, j - 1, k, IU) + q(i - 1, j, k, IU) + q(i, j - 1, k, IU) + q(i, j, k, IU));
            const double v = 0.25 * (q(i - 1, j - 1, k, IV) + q(i - 1, j, k, IV) + q(i, j - 1, k, IV) + q(i, j, k, IV));
            const double A = 0.5 * (q(i, j - 1, k, IA) + q(i, j, k, IA));
            const double B = 0.5 * (q(i - 1, j, k, IB) + q(i, j, k, IB));
            w.E(i, j, k, 2) = u * B - v * A;
          }
        }
      }
}

// compute_sFaceMag (scheme/ComputeSourceFaceMagFunctor.cpp:114-203)
static void
compute_sfacemag(const Mesh & m, double dtdx, StepWork & w)
{
  const int g = 1;
  const int gz = m.dim == 3 ? 1 : 0;
  w.SF.init(-g, m.bx + 2 * g, -g, m.by + 2 * g, -gz, m.bz + 2 * gz, m.dim == 3 ? 3 : 2);
  const double dtdy = dtdx, dtdz = dtdx;
  Box & e = w.E;
  for (int k = -gz; k < m.bz + gz; ++k)
    for (int j = -g; j < m.by + g; ++j)
      for (int i = -g; i < m.bx + g; ++i)
      {
        if (m.dim == 2)
        {
          w.SF(i, j, 0, 0) = (e(i, j + 1, 0, 0) - e(i, j, 0, 0)) * 0.5 * dtdy;
          w.SF(i, j, 0, 1) = -(e(i + 1, j, 0, 0) - e(i, j, 0, 0)) * 0.5 * dtdx;
        }
        else
        {
          w.SF(i, j, k, 0) = (e(i, j + 1, k, 2) - e(i, j, k, 2)) * 0.5 * dtdy -
                             (e(i, j, k + 1, 1) - e(i, j, k, 1)) * 0.5 * dtdz;
          w.SF(i, j, k, 1) = -(e(i + 1, j, k, 2) - e(i, j, k, 2)) * 0.5 * dtdx +
                             (e(i, j, k + 1, 0) - e(i, j, k, 0)) * 0.5 * dtdz;
          w.SF(i, j, k, 2) = (e(i + 1, j, k, 1) - e(i, j, k, 1)) * 0.5 * dtdx -
                             (e(i, j + 1, k, 0) - e(i, j, k, 0)) * 0.5 * dtdy;
        }
      }
}

static Box &
slopes_dir(StepWork & w, int dir)
{
  return dir == 0 ? w.Sx : (dir == 1 ? w.Sy : w.Sz);
}

// reconstruct_state_{2d,3d} (scheme/ComputeHydroFluxesAndStoreFunctor.cpp:118-214)
static void
reconstruct_face(StepWork & w, const Settings & s, int i, int j, int k, int dir, double offset, double * qr)
{
  Box & S = slopes_dir(w, dir);
  for (int v = 0; v < 8; ++v)
    qr[v] = w.Q2(i, j, k, v) + offset * S(i, j, k, v);
  qr[ID] = std::fmax(s.smallr, qr[ID]);
  qr[IP] = std::fmax(s.smallp * qr[ID], qr[IP]);
}

// Per-block face fluxes of all directions: [dir][var 0..7][face], faces of direction d indexed
// i + nx * (j + ny * k) with nx = bx + (d == 0) etc.
struct FluxLayout
{
  int64_t n[3];   // faces per direction (0 for z in 2D)
  int64_t off[3]; // offset of direction d (times 8 vars)
  int64_t total;
};

static FluxLayout
flux_layout(const Mesh & m)
{
  FluxLayout F;
  F.n[0] = (int64_t)(m.bx + 1) * m.by * m.bz;
  F.n[1] = (int64_t)m.bx * (m.by + 1) * m.bz;
  F.n[2] = m.dim == 3 ? (int64_t)m.bx * m.by * (m.bz + 1) : 0;
  F.off[0] = 0;
  F.off[1] = 8 * F.n[0];
  F.off[2] = F.off[1] + 8 * F.n[1];
  F.total = F.off[2] + 8 * F.n[2];
  return F;
}

// compute_fluxes_and_store_{2d,3d} (scheme/ComputeHydroFluxesAndStoreFunctor.cpp:216-503) for one
// direction: flux * dt/dx into Fblk (FluxLayout).
static int
compute_fluxes(const Mesh & m, const Settings & s, double dtdx, int dir, StepWork & w, double * Fblk)
{
  const FluxLayout FL = flux_layout(m);
  const int nx = m.bx + (dir == 0), ny = m.by + (dir == 1), nz = m.bz + (dir == 2 && m.dim == 3);
  const int di = dir == 0, dj = dir == 1, dk = dir == 2;
  // normal-B slot and the velocity / B component swapped with x for this direction
  const int ivel = dir == 0 ? IU : (dir == 1 ? IV : IW);
  const int imag = dir == 0 ? IA : (dir == 1 ? IB : IC);
  double *  Fd = Fblk + FL.off[dir];
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
      {
        double qL[8], qR[8], flux[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        reconstruct_face(w, s, i - di, j - dj, k - dk, dir, 0.5, qL);
        reconstruct_face(w, s, i, j, k, dir, -0.5, qR);
        const double bn = w.Q(i, j, k, imag) + w.SF(i, j, k, dir);
        qR[imag] = bn;
        qL[imag] = bn;
        if (dir != 0)
        {
          std::swap(qL[IU], qL[ivel]);
          std::swap(qR[IU], qR[ivel]);
          std::swap(qL[IA], qL[imag]);
          std::swap(qR[IA], qR[imag]);
        }
        if (riemann_mhd(qL, qR, flux, s) != 0)
          return -3;
        if (dir != 0)
        {
          std::swap(flux[IU], flux[ivel]);
          std::swap(flux[IA], flux[imag]);
        }
        const int64_t fi = i + (int64_t)nx * (j + (int64_t)ny * k);
        for (int v = 0; v < 8; ++v)
          Fd[v * FL.n[dir] + fi] = flux[v] * dtdx;
      }
  return 0;
}

// get_flux_from_fine_neighbor (scheme/ReadFluxesAndConservativeUpdateFunctor.h:233-270): sum of the
// 2^(d-1) fine fluxes through the face of cell q on side `side` (-1 left, +1 right) along dir.
// Viscous face fluxes along dir (ComputeViscousFluxesAndStoreFunctor.cpp:168-344): at the left face
// of cell (i, j, k), the velocity gradient is a backward difference from the cell (normal: across the
// face; transverse: inside the cell's row), the stress tensor uses it with the cell's velocity; the
// flux (times dt/dx) goes to E and the momenta, zero for rho and B. Same layout as compute_fluxes.
static void
compute_viscous_fluxes(const Mesh & m, const Settings & s, double dtdx, double dx, int dir, StepWork & w,
                       double * Fblk)
{
  const FluxLayout FL = flux_layout(m);
  const int        nx = m.bx + (dir == 0), ny = m.by + (dir == 1), nz = m.bz + (dir == 2);
  const double     mu = s.mu;
  const int        nv = m.dim;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
      {
        double vel[3] = {0.0, 0.0, 0.0}, g[3][3] = {}; // g[c][d]: d(velocity c)/d(axis d)
        for (int c = 0; c < nv; ++c)
        {
          const int    var = IU + c;
          const double qr = w.Q(i, j, k, var);
          vel[c] = qr;
          g[c][0] = (qr - w.Q(i - 1, j, k, var)) / dx;
          g[c][1] = (qr - w.Q(i, j - 1, k, var)) / dx;
          if (m.dim == 3)
            g[c][2] = (qr - w.Q(i, j, k - 1, var)) / dx;
        }
        double fu, fv, fw = 0.0, fe;
        if (m.dim == 2)
        {
          const double div = g[0][0] + g[1][1];
          const double txy = mu * (g[1][0] + g[0][1]);
          if (dir == 0)
          {
            const double txx = 2 * mu * (g[0][0] - 0.5 * div);
            fu = -txx;
            fv = -txy;
            fe = -vel[0] * txx - vel[1] * txy;
          }
          else
          {
            const double tyy = 2 * mu * (g[1][1] - 0.5 * div);
            fu = -txy;
            fv = -tyy;
            fe = -vel[0] * txy - vel[1] * tyy;
          }
        }
        else
        {
          const double third = 1.0 / 3.0;
          const double div = g[0][0] + g[1][1] + g[2][2];
          double       t0, t1, t2;
          if (dir == 0)
          {
            t0 = 2 * mu * (g[0][0] - third * div);
            t1 = mu * (g[1][0] + g[0][1]);
            t2 = mu * (g[2][0] + g[0][2]);
          }
          else if (dir == 1)
          {
            t0 = mu * (g[0][1] + g[1][0]);
            t1 = 2 * mu * (g[1][1] - third * div);
            t2 = mu * (g[2][1] + g[1][2]);
          }
          else
          {
            t0 = mu * (g[0][2] + g[2][0]);
            t1 = mu * (g[1][2] + g[2][1]);
            t2 = 2 * mu * (g[2][2] - third * div);
          }
          fu = -t0;
          fv = -t1;
          fw = -t2;
          fe = -vel[0] * t0 - vel[1] * t1 - vel[2] * t2;
        }
        const int64_t f = i + (int64_t)nx * (j + (int64_t)ny * k);
        double *      F = Fblk + FL.off[dir];
        F[ID * FL.n[dir] + f] = 0.0 * dtdx;
        F[IP * FL.n[dir] + f] = fe * dtdx; // energy (IE == IP)
        F[IU * FL.n[dir] + f] = fu * dtdx;
        F[IV * FL.n[dir] + f] = fv * dtdx;
        F[IW * FL.n[dir] + f] = fw * dtdx;
        if (m.dim == 2)
          F[IC * FL.n[dir] + f] = 0.0 * dtdx;
      }
}

// AddGravitySourceTerm (scheme/AddGravitySourceTerm.cpp:47-99) on one owned block: momentum gets
// dt g times the mean of the old and new densities, the energy the resulting change of kinetic energy.
static void
add_gravity_source(const Mesh & m, const Settings & s, double dt, const double * Ublk, double * U2blk, int64_t ncell)
{
  for (int64_t c = 0; c < ncell; ++c)
  {
    const double rho_old = Ublk[ID * ncell + c];
    const double rho_new = U2blk[ID * ncell + c];
    double       ru = U2blk[IU * ncell + c], rv = U2blk[IV * ncell + c], rw = 0.0;
    if (m.dim == 3)
      rw = U2blk[IW * ncell + c];
    double ekin_old = 0.5 * (ru * ru + rv * rv) / rho_new;
    if (m.dim == 3)
      ekin_old += 0.5 * (rw * rw) / rho_new;
    ru += dt * s.grav[0] * (rho_old + rho_new) / 2;
    rv += dt * s.grav[1] * (rho_old + rho_new) / 2;
    if (m.dim == 3)
      rw += dt * s.grav[2] * (rho_old + rho_new) / 2;
    U2blk[IU * ncell + c] = ru;
    U2blk[IV * ncell + c] = rv;
    if (m.dim == 3)
      U2blk[IW * ncell + c] = rw;
    double ekin_new = 0.5 * (ru * ru + rv * rv) / rho_new;
    if (m.dim == 3)
      ekin_new += 0.5 * (rw * rw) / rho_new;
    U2blk[IP * ncell + c] += (ekin_new - ekin_old); // total energy (IE == IP)
  }
}

static bool
fine_flux_sum(const Mesh & m, const std::vector<std::vector<double>> & flux_all, const Region & r, int dir,
              int side, const int * q, int v, double & out)
{
  const FluxLayout FL = flux_layout(m);
  const int        b[3] = {m.bx, m.by, m.bz};
  const int        t1 = dir == 0 ? 1 : 0;
  const int        t2 = dir == 2 ? 1 : 2;
  double           acc = 0.0;
  for (int e2 = 0; e2 < (m.dim == 3 ? 2 : 1); ++e2)
    for (int e1 = 0; e1 < 2; ++e1)
    {
      int F[3] = {0, 0, 0}, c[3] = {0, 0, 0};
      c[dir] = side < 0 ? 1 : 0;
      F[dir] = side < 0 ? b[dir] : 0; // right flux of the last fine cell / left flux of the first
      F[t1] = 2 * q[t1] + e1;
      c[t1] = F[t1] >= b[t1];
      F[t1] -= c[t1] * b[t1];
      if (m.dim == 3)
      {
        F[t2] = 2 * q[t2] + e2;
        c[t2] = F[t2] >= b[t2];
        F[t2] -= c[t2] * b[t2];
      }
      const int id = r.child[c[0] + 2 * c[1] + 4 * c[2]];
      if (id < 0 || id >= m.n_owned)
        return false;
      const int nx = m.bx + (dir == 0), ny = m.by + (dir == 1);
      acc += flux_all[id][FL.off[dir] + v * FL.n[dir] + F[0] + (int64_t)nx * (F[1] + (int64_t)ny * F[2])];
    }
  out = acc;
  return true;
}

// read_fluxes_and_update_{2d,3d} (scheme/ReadFluxesAndConservativeUpdateFunctor.cpp:103-436): per
// direction accum = 0 + F(i) - F(i+1), a face with finer neighbours taking their flux sum / 2^d, then
// U2 += accum (2D: Bz too).
static int
update_u(const Mesh & m, int blk, const std::vector<std::vector<double>> & flux_all, double * U2blk,
         double * Bz2blk)
{
  const FluxLayout FL = flux_layout(m);
  const int        b[3] = {m.bx, m.by, m.bz};
  const int64_t    ncell = (int64_t)m.bx * m.by * m.bz;
  const double     vr = (double)(1 << m.dim);
  const std::vector<double> & Fb = flux_all[blk];
  const int nvar = m.dim == 2 ? 6 : 5;
  for (int dir = 0; dir < m.dim; ++dir)
  {
    int olo[3] = {0, 0, 0}, ohi[3] = {0, 0, 0};
    olo[dir] = -1;
    ohi[dir] = 1;
    const Region rlo = region_of(m, blk, olo[0], olo[1], olo[2]);
    const Region rhi = region_of(m, blk, ohi[0], ohi[1], ohi[2]);
    const int    nx = m.bx + (dir == 0), ny = m.by + (dir == 1);
    const int    di = dir == 0, dj = dir == 1, dk = dir == 2;
    for (int k = 0; k < m.bz; ++k)
      for (int j = 0; j < m.by; ++j)
        for (int i = 0; i < m.bx; ++i)
        {
          const int     q[3] = {i, j, k};
          const int64_t c = i + (int64_t)m.bx * (j + (int64_t)m.by * k);
          const int64_t fl = i + (int64_t)nx * (j + (int64_t)ny * k);
          const int64_t fr = (i + di) + (int64_t)nx * ((j + dj) + (int64_t)ny * (k + dk));
          for (int n = 0; n < nvar; ++n)
          {
            const int v = n < 5 ? n : IC;
            double    acc = 0.0;
            if (q[dir] == 0 && rlo.kind == RK_FINER)
            {
              double sum;
              if (!fine_flux_sum(m, flux_all, rlo, dir, -1, q, v, sum))
                return -1;
              acc = acc + sum / vr;
            }
            else
              acc = acc + Fb[FL.off[dir] + v * FL.n[dir] + fl];
            if (q[dir] == b[dir] - 1 && rhi.kind == RK_FINER)
            {
              double sum;
              if (!fine_flux_sum(m, flux_all, rhi, dir, 1, q, v, sum))
                return -1;
              acc = acc - sum / vr;
            }
            else
              acc = acc - Fb[FL.off[dir] + v * FL.n[dir] + fr];
            if (n < 5)
              U2blk[v * ncell + c] += acc;
            else
              Bz2blk[c] += acc;
          }
        }
  }
  return 0;
}

// compute_limited_slope of a face-B value (scheme/ComputeEmfAndStoreFunctor.h:365-419)
static double
face_slope(StepWork & w, const Settings & s, int i, int j, int k, int var, int dir)
{
  const int di = dir == 0, dj = dir == 1, dk = dir == 2;
  return slope_scalar(w.Q(i, j, k, var), w.Q(i + di, j + dj, k + dk, var), w.Q(i - di, j - dj, k - dk, var), s);
}

enum EdgeLoc
{
  LB,
  RT,
  RB,
  LT
};

// reconstruct_state_2d_at_edge (scheme/ComputeEmfAndStoreFunctor.cpp:103-214)
static void
reconstruct_edge_2d(StepWork & w, const Settings & s, int is, int js, EdgeLoc loc, double * q)
{
  for (int v = 0; v < 8; ++v)
    q[v] = w.Q2(is, js, 0, v);
  int sx, sy, ia, ja, ib, jb, sa, sb;
  switch (loc)
  {
    case LB: ia = is; ja = js; ib = is; jb = js; sx = -1; sy = -1; sa = -1; sb = -1; break;
    case RT: ia = is + 1; ja = js; ib = is; jb = js + 1; sx = 1; sy = 1; sa = 1; sb = 1; break;
    case RB: ia = is + 1; ja = js; ib = is; jb = js; sx = 1; sy = -1; sa = -1; sb = 1; break;
    default: ia = is; ja = js; ib = is; jb = js + 1; sx = -1; sy = 1; sa = 1; sb = -1; break;
  }
  double A = w.Q(ia, ja, 0, IA);
  double B = w.Q(ib, jb, 0, IB);
  if (!s.rk2) // the half-step face source only with HANCOCK (ComputeEmfAndStoreFunctor.cpp:189-193)
  {
    A += w.SF(ia, ja, 0, 0);
    B += w.SF(ib, jb, 0, 1);
  }
  const double dAy = face_slope(w, s, ia, ja, 0, IA, 1);
  const double dBx = face_slope(w, s, ib, jb, 0, IB, 0);
  const double fx = (double)sx, fy = (double)sy;
  for (int v : {ID, IP, IU, IV, IW})
    q[v] += 0.5 * (fx * w.Sx(is, js, 0, v) + fy * w.Sy(is, js, 0, v));
  q[IA] = A + 0.5 * ((double)sa * dAy);
  q[IB] = B + 0.5 * ((double)sb * dBx);
  q[IC] += 0.5 * (fx * w.Sx(is, js, 0, IC) + fy * w.Sy(is, js, 0, IC));
  q[ID] = std::fmax(s.smallr, q[ID]);
  q[IP] = std::fmax(s.smallp * q[ID], q[IP]);
}

// reconstruct_state_3d_at_edge (scheme/ComputeEmfAndStoreFunctor.cpp:218-367). The branch order
// below is the reference's; for (dir0,dir1) = (IY,IZ) and (IX,IZ) the cell-centred By term is
// added on top of the face value / twice, exactly as the reference does.
static void
reconstruct_edge_3d(StepWork & w, const Settings & s, int is, int js, int ks, EdgeLoc loc, int dir0, int dir1,
                    double * q)
{
  for (int v = 0; v < 8; ++v)
    q[v] = w.Q2(is, js, ks, v);
  int sd0 = 1, sd1 = 1, sb0 = 1, sb1 = 1;
  int ijk0[3] = {is, js, ks};
  int ijk1[3] = {is, js, ks};
  switch (loc)
  {
    case LB: sd0 = -1; sd1 = -1; sb0 = -1; sb1 = -1; break;
    case RT: ijk0[dir0] += 1; ijk1[dir1] += 1; sd0 = 1; sd1 = 1; sb0 = 1; sb1 = 1; break;
    case RB: ijk0[dir0] += 1; sd0 = 1; sd1 = -1; sb0 = -1; sb1 = 1; break;
    default: ijk1[dir1] += 1; sd0 = -1; sd1 = 1; sb0 = 1; sb1 = -1; break;
  }
  double B0 = w.Q(ijk0[0], ijk0[1], ijk0[2], IA + dir0);
  double B1 = w.Q(ijk1[0], ijk1[1], ijk1[2], IA + dir1);
  if (!s.rk2) // the half-step face source only with HANCOCK (ComputeEmfAndStoreFunctor.cpp:297-301)
  {
    B0 += w.SF(ijk0[0], ijk0[1], ijk0[2], dir0);
    B1 += w.SF(ijk1[0], ijk1[1], ijk1[2], dir1);
  }
  const double dB0d1 = face_slope(w, s, ijk0[0], ijk0[1], ijk0[2], IA + dir0, dir1);
  const double dB1d0 = face_slope(w, s, ijk1[0], ijk1[1], ijk1[2], IA + dir1, dir0);
  Box &        S0 = slopes_dir(w, dir0);
  Box &        S1 = slopes_dir(w, dir1);
  const double f0 = (double)sd0, f1 = (double)sd1;
  auto         h = [&](int v) { return 0.5 * (f0 * S0(is, js, ks, v) + f1 * S1(is, js, ks, v)); };
  q[ID] += h(ID);
  q[IP] += h(IP);
  q[IU] += h(IU);
  q[IV] += h(IV);
  q[IW] += h(IW);
  if (dir0 == 0)
    q[IA] = B0 + 0.5 * ((double)sb0 * dB0d1);
  else
    q[IA] += h(IA);
  if (dir0 == 1)
    q[IB] = B0 + 0.5 * ((double)sb0 * dB0d1);
  else
    q[IB] += h(IB);
  if (dir1 == 1)
    q[IB] = B1 + 0.5 * ((double)sb1 * dB1d0);
  else
    q[IB] += h(IB);
  if (dir1 == 2)
    q[IC] = B1 + 0.5 * ((double)sb1 * dB1d0);
  else
    q[IC] += h(IC);
  q[ID] = std::fmax(s.smallr, q[ID]);
  q[IP] = std::fmax(s.smallp * q[ID], q[IP]);
}

// compute_emf_and_store_{2d,3d} (scheme/ComputeEmfAndStoreFunctor.cpp:371-590). emf has
// (b+1)^d edges per component, component-slowest.
static void
compute_emfs(const Mesh & m, const Settings & s, double dtdx, StepWork & w, double * emf)
{
  const int ex = m.bx + 1, ey = m.by + 1, ez = m.dim == 3 ? m.bz + 1 : 1;
  const int64_t ne = (int64_t)ex * ey * ez;
  double        qe[4][8];
  for (int k = 0; k < ez; ++k)
    for (int j = 0; j < ey; ++j)
      for (int i = 0; i < ex; ++i)
      {
        const int64_t e = i + (int64_t)ex * (j + (int64_t)ey * k);
        if (m.dim == 2)
        {
          reconstruct_edge_2d(w, s, i, j, LB, qe[ELB]);
          reconstruct_edge_2d(w, s, i - 1, j - 1, RT, qe[ERT]);
          reconstruct_edge_2d(w, s, i - 1, j, RB, qe[ERB]);
          reconstruct_edge_2d(w, s, i, j - 1, LT, qe[ELT]);
          emf[e] = compute_emf(qe, 2, s) * dtdx;
          continue;
        }
        if (k < m.bz)
        {
          reconstruct_edge_3d(w, s, i, j, k, LB, 0, 1, qe[ELB]);
          reconstruct_edge_3d(w, s, i - 1, j - 1, k, RT, 0, 1, qe[ERT]);
          reconstruct_edge_3d(w, s, i - 1, j, k, RB, 0, 1, qe[ERB]);
          reconstruct_edge_3d(w, s, i, j - 1, k, LT, 0, 1, qe[ELT]);
          emf[2 * ne + e] = compute_emf(qe, 2, s) * dtdx;
        }
        if (j < m.by)
        {
          reconstruct_edge_3d(w, s, i, j, k, LB, 0, 2, qe[ELB]);
          reconstruct_edge_3d(w, s, i - 1, j, k - 1, RT, 0, 2, qe[ERT]);
          reconstruct_edge_3d(w, s, i - 1, j, k, RB, 0, 2, qe[ERB]);
          reconstruct_edge_3d(w, s, i, j, k - 1, LT, 0, 2, qe[ELT]);
          for (int v = 0; v < 8; ++v)
            std::swap(qe[ERB][v], qe[ELT][v]);
          emf[1 * ne + e] = compute_emf(qe, 1, s) * dtdx;
        }
        if (i < m.bx)
        {
          reconstruct_edge_3d(w, s, i, j, k, LB, 1, 2, qe[ELB]);
          reconstruct_edge_3d(w, s, i, j - 1, k - 1, RT, 1, 2, qe[ERT]);
          reconstruct_edge_3d(w, s, i, j - 1, k, RB, 1, 2, qe[ERB]);
          reconstruct_edge_3d(w, s, i, j, k - 1, LT, 1, 2, qe[ELT]);
          emf[0 * ne + e] = compute_emf(qe, 0, s) * dtdx;
        }
      }
}

static int64_t
emf_count(const Mesh & m)
{
  return (int64_t)(m.bx + 1) * (m.by + 1) * (m.dim == 3 ? m.bz + 1 : 1);
}

// read_emf_and_update_{2d,3d} (scheme/ReadEmfAndUpdateFunctor.cpp:58-163): B of one block (faces,
// C ABI layout) += curl of the block's edge EMFs emf2 [ncomp][(b+1)^d] (2D: the z component only).
static void
read_emf_and_update(const Mesh & m, const double * emf2, double * B2blk)
{
  const int     ex = m.bx + 1, ey = m.by + 1;
  const int64_t ne = emf_count(m);
  const BlockLayout L = block_layout(m);
  double *          Bx = B2blk;
  double *          By = B2blk + L.nfx;
  double *          Bz = B2blk + L.nfx + L.nfy;
  auto              E = [&](int c, int i, int j, int k) { return emf2[c * ne + i + (int64_t)ex * (j + (int64_t)ey * k)]; };
  if (m.dim == 2)
  {
    for (int j = 0; j < m.by; ++j)
      for (int i = 0; i <= m.bx; ++i)
        Bx[i + (int64_t)(m.bx + 1) * j] += (E(0, i, j + 1, 0) - E(0, i, j, 0));
    for (int j = 0; j <= m.by; ++j)
      for (int i = 0; i < m.bx; ++i)
        By[i + (int64_t)m.bx * j] -= (E(0, i + 1, j, 0) - E(0, i, j, 0));
    return;
  }
  for (int k = 0; k < m.bz; ++k)
    for (int j = 0; j < m.by; ++j)
      for (int i = 0; i <= m.bx; ++i)
      {
        double d = 0;
        d += (E(2, i, j + 1, k) - E(2, i, j, k));
        d -= (E(1, i, j, k + 1) - E(1, i, j, k));
        Bx[i + (int64_t)(m.bx + 1) * (j + (int64_t)m.by * k)] += d;
      }
  for (int k = 0; k < m.bz; ++k)
    for (int j = 0; j <= m.by; ++j)
      for (int i = 0; i < m.bx; ++i)
      {
        double d = 0;
        d += (E(0, i, j, k + 1) - E(0, i, j, k));
        d -= (E(2, i + 1, j, k) - E(2, i, j, k));
        By[i + (int64_t)m.bx * (j + (int64_t)(m.by + 1) * k)] += d;
      }
  for (int k = 0; k <= m.bz; ++k)
    for (int j = 0; j < m.by; ++j)
      for (int i = 0; i < m.bx; ++i)
      {
        double d = 0;
        d += (E(1, i + 1, j, k) - E(1, i, j, k));
        d -= (E(0, i, j + 1, k) - E(0, i, j, k));
        Bz[i + (int64_t)m.bx * (j + (int64_t)m.by * k)] += d;
      }
}

// correct_emf, uniform-level branch (scheme/CorrectEmfAtBlockBorderFunctor.cpp:94-360) followed by
// read_emf_and_update_{2d,3d} (scheme/ReadEmfAndUpdateFunctor.cpp:58-163) for block blk.
// CorrectEmfAtBlockBorderFunctor::correct_emf (CorrectEmfAtBlockBorderFunctor.cpp:94-360) over the edges
// of block blk: emf2 receives the block's EMFs (deep_copy(emf2, emf), GodunovImplemV0.cpp:606) with its
// border edges corrected from the sibling copies in emf_all. Returns 0 or -1 (a finer sibling that is
// not an owned block).
static int
correct_emf(const Mesh & m, int blk, const std::vector<double> & emf_all, std::vector<double> & emf2)
{
  const int     ex = m.bx + 1, ey = m.by + 1, ez = m.dim == 3 ? m.bz + 1 : 1;
  const int64_t ne = emf_count(m);
  const int     ncomp = m.dim == 3 ? 3 : 1;
  const double *emf_self = &emf_all[(size_t)blk * ncomp * ne];
  emf2.assign(emf_self, emf_self + ncomp * ne);
  const int bsz[3] = {m.bx, m.by, m.bz};
  for (int c = 0; c < ncomp; ++c)
  {
    const int edir = m.dim == 3 ? c : 2;
    // transverse directions of this edge direction
    const int t0 = edir == 0 ? 1 : 0;
    const int t1 = edir == 2 ? 1 : 2;
    for (int k = 0; k < ez; ++k)
      for (int j = 0; j < ey; ++j)
        for (int i = 0; i < ex; ++i)
        {
          int idx[3] = {i, j, k};
          // only edges that exist for this component
          if (m.dim == 3 && idx[edir] >= bsz[edir])
            continue;
          const int a0 = idx[t0], a1 = (m.dim == 3 || t1 < 2) ? idx[t1] : 0;
          const int v0 = a0 == 0 ? -1 : (a0 == bsz[t0] ? 1 : 0);
          const int v1 = (m.dim == 2 && t1 == 2) ? 0 : (a1 == 0 ? -1 : (a1 == bsz[t1] ? 1 : 0));
          if (v0 == 0 && v1 == 0)
            continue;
          // sibling edges (core getEdgeSiblingLoc): across t0, across t1, across both
          // (CorrectEmfAtBlockBorderFunctor.cpp:94-360)
          Region rs[3];
          bool   valid[3];
          int    lev[3]; // sibling level - own level
          int    sidx[3][3];
          int    so[3][3];
          for (int n = 0; n < 3; ++n)
          {
            int o[3] = {0, 0, 0};
            if (n == 0 || n == 2)
              o[t0] = v0;
            if (n == 1 || n == 2)
              o[t1] = v1;
            const bool exists = (n == 0 && v0 != 0) || (n == 1 && v1 != 0) || (n == 2 && v0 != 0 && v1 != 0);
            rs[n] = exists ? region_of(m, blk, o[0], o[1], o[2]) : Region{RK_MISSING, -1, {0, 0, 0}, nullptr};
            valid[n] = rs[n].kind != RK_MISSING;
            lev[n] = rs[n].kind == RK_COARSER ? -1 : (rs[n].kind == RK_FINER ? 1 : 0);
            for (int d = 0; d < 3; ++d)
            {
              so[n][d] = o[d];
              sidx[n][d] = idx[d] - o[d] * bsz[d];
            }
          }
          const bool coarser = (valid[0] && lev[0] < 0) || (valid[1] && lev[1] < 0) || (valid[2] && lev[2] < 0);
          const bool finer = (valid[0] && lev[0] > 0) || (valid[1] && lev[1] > 0) || (valid[2] && lev[2] > 0);
          const bool all_same = valid[0] && lev[0] == 0 && valid[1] && lev[1] == 0 && valid[2] && lev[2] == 0;
          const int64_t e = i + (int64_t)ex * (j + (int64_t)ey * k);
          auto          sib_emf = [&](int id, const int * ix) {
            const int64_t es = ix[0] + (int64_t)ex * (ix[1] + (int64_t)ey * ix[2]);
            return emf_all[(size_t)id * ncomp * ne + c * ne + es];
          };
          if (coarser)
          {
            // average with the same-level siblings
            double acc = emf_self[c * ne + e];
            int    count = 1;
            for (int n = 0; n < 3; ++n)
              if (valid[n] && lev[n] == 0 && rs[n].kind != RK_OUTSIDE)
              {
                acc += sib_emf(rs[n].id, sidx[n]);
                count++;
              }
            emf2[c * ne + e] = acc / (double)count;
          }
          else if (finer)
          {
            // average over the finer siblings' edges (3D: both sub-edges along the edge)
            double acc = 0.0;
            int    count = 0;
            for (int n = 0; n < 3; ++n)
            {
              if (!(valid[n] && lev[n] > 0))
                continue;
              int F[3] = {0, 0, 0}, ch[3] = {0, 0, 0};
              for (int d = 0; d < m.dim; ++d)
              {
                if (so[n][d] != 0)
                {
                  ch[d] = so[n][d] < 0 ? 1 : 0;
                  F[d] = so[n][d] < 0 ? bsz[d] : 0;
                }
                else
                {
                  const int x = 2 * idx[d];
                  ch[d] = x >= bsz[d];
                  F[d] = x - ch[d] * bsz[d];
                }
              }
              const int id = rs[n].child[ch[0] + 2 * ch[1] + 4 * ch[2]];
              if (id < 0 || id >= m.n_owned)
                return -1;
              acc += sib_emf(id, F);
              if (m.dim == 3)
              {
                int F1[3] = {F[0], F[1], F[2]};
                F1[edir] += 1;
                acc += sib_emf(id, F1);
              }
              count++;
            }
            emf2[c * ne + e] = acc / (double)count / (double)(1 << (m.dim - 1));
          }
          if (all_same)
          {
            double acc = 0.0;
            int    count = 1;
            acc += emf_self[c * ne + e];
            for (int n = 0; n < 3; ++n)
              if (rs[n].kind != RK_OUTSIDE)
              {
                acc += sib_emf(rs[n].id, sidx[n]);
                count++;
              }
            emf2[c * ne + e] = acc / (double)count;
          }
        }
  }
  return 0;
}

// border EMF correction, then the CT update of block blk's faces
static int
correct_emf_and_update_b(const Mesh & m, int blk, const std::vector<double> & emf_all, double * B2blk)
{
  std::vector<double> emf2;
  const int           st = correct_emf(m, blk, emf_all, emf2);
  if (st != 0)
    return st;
  read_emf_and_update(m, emf2.data(), B2blk);
  return 0;
}

static double
cell_length(const Mesh & m, int level)
{
  return (1.0 / (double)((int64_t)m.bx << level)) * m.scaling_factor;
}


// ---- regrid: refinement indicator and remap (SolverGodunovMHD.cpp:263-319, 1092-1262) --------
// kalypsso-core's ComputeRefineFlags and UserDataRemapper are not in the reference tree; these are
// this restatement's definitions (mirrored by the GPU kernels in amr.cu):
//   * indicator per cell and axis on rho and/or the pressure (compute_primitives with the cell-centred
//     B of the faces), neighbours clamped to the block: SIMPLE_GRADIENT
//     max(|q+ - q|, |q - q-|) / max(|q|, DBL_MIN); LOHNER_UNSPLIT |dp - dm| / (|dp| + |dm| +
//     eps_lohner (|q+| + 2|q| + |q-|)) with dp = q+ - q, dm = q - q-; block error = max; flag +1
//     if error > epsilon_refine and level < level_max, -1 if error < epsilon_coarsen and level >
//     level_min;
//   * remap: kept leaves copy; a coarsened leaf takes the mean of its children (cells and faces, as
//     the ghost restriction; a face shared with a kept leaf of its level copies that leaf's face);
//     a refined leaf copies the parent cell (SIMPLE_COPY) and prolongs faces
//     as the ghost prolongation, except that faces shared with a leaf that stays at the child's level
//     copy that leaf's faces, the resulting divergence of each adjacent fine cell being cancelled on
//     the faces inside its coarse cell (2D: + or - d0 on the middle face; 3D: F = (d00 + d01)/2 on
//     the two faces normal to the first transverse axis, d00 - F and d10 + F on those normal to the
//     second), borders applied in the order -x, +x, -y, +y, -z, +z.
struct RefineParams
{
  int32_t criterion; // 0 SIMPLE_GRADIENT, 1 LOHNER_UNSPLIT
  int32_t level_min, level_max;
  int32_t use_rho, use_pressure;
  double  eps_refine, eps_coarsen, eps_lohner;
};

static double
refine_quantity(const Mesh & m, const Fields & f, const Settings & s, int blk, int var, int i, int j, int k)
{
  if (var == 0)
    return f.u(blk, ID, i, j, k);
  double u[8], q[8];
  for (int n = 0; n < 5; ++n)
    u[n] = f.u(blk, n, i, j, k);
  u[IA] = 0.5 * (f.bx(blk, i, j, k) + f.bx(blk, i + 1, j, k));
  u[IB] = 0.5 * (f.by(blk, i, j, k) + f.by(blk, i, j + 1, k));
  if (m.dim == 3)
    u[IC] = 0.5 * (f.bz(blk, i, j, k) + f.bz(blk, i, j, k + 1));
  else
    u[IC] = 0.5 * (f.bz(blk, i, j, 0) + f.bz(blk, i, j, 0));
  compute_primitives(u, q, nullptr, s);
  return q[IP];
}

static double
block_refine_error(const Mesh & m, const Fields & f, const Settings & s, const RefineParams & rp, int blk)
{
  const int b[3] = {m.bx, m.by, m.bz};
  double    err = 0.0;
  for (int var = 0; var < 2; ++var)
  {
    if ((var == 0 && !rp.use_rho) || (var == 1 && !rp.use_pressure))
      continue;
    for (int k = 0; k < m.bz; ++k)
      for (int j = 0; j < m.by; ++j)
        for (int i = 0; i < m.bx; ++i)
        {
          const double q = refine_quantity(m, f, s, blk, var, i, j, k);
          for (int d = 0; d < m.dim; ++d)
          {
            int im[3] = {i, j, k}, ip[3] = {i, j, k};
            im[d] = std::max(im[d] - 1, 0);
            ip[d] = std::min(ip[d] + 1, b[d] - 1);
            const double qm = refine_quantity(m, f, s, blk, var, im[0], im[1], im[2]);
            const double qp = refine_quantity(m, f, s, blk, var, ip[0], ip[1], ip[2]);
            double       e;
            if (rp.criterion == 0)
              e = std::fmax(std::fabs(qp - q), std::fabs(q - qm)) / std::fmax(std::fabs(q), 2.2250738585072014e-308);
            else
            {
              const double dp = qp - q, dm = q - qm;
              const double den = std::fabs(dp) + std::fabs(dm) +
                                 rp.eps_lohner * (std::fabs(qp) + 2.0 * std::fabs(q) + std::fabs(qm));
              e = den > 0.0 ? std::fabs(dp - dm) / den : 0.0;
            }
            err = std::fmax(err, e);
          }
        }
  }
  return err;
}

// Face value (component comp, block-local idx) of refined-leaf child n of the new mesh: the ghost
// prolongation of the parent, faces shared with a kept leaf copied from it, then the divergence
// corrections of the borders in order.
static double
prolonged_face(const Mesh & mo, const Fields & fo, const int32_t * rm, int comp, const int * idx)
{
  const int b[3] = {mo.bx, mo.by, mo.bz};
  const int parent = rm[1], child = rm[2];
  Region    r{RK_COARSER, parent, {child & 1, (child >> 1) & 1, (child >> 2) & 1}, nullptr};
  auto      base = [&](int c, const int * q) {
    double v = 0.0;
    region_face(mo, fo, r, c, q, v);
    return v;
  };
  const bool cellc = mo.dim == 2 && comp == 2;
  // border replacement
  auto border = [&](int c, const int * q, double & v) {
    if (mo.dim == 2 && c == 2)
      return false;
    for (int sd = 0; sd < 2; ++sd)
    {
      const int nb = rm[9 + 2 * c + sd];
      if (nb < 0 || q[c] != (sd == 0 ? 0 : b[c]))
        continue;
      int qq[3] = {q[0], q[1], q[2]};
      qq[c] = sd == 0 ? b[c] : 0;
      v = fo.face(nb, c, qq[0], qq[1], qq[2]);
      return true;
    }
    return false;
  };
  double val;
  if (!border(comp, idx, val))
    val = base(comp, idx);
  if (cellc)
    return val;
  for (int n = 0; n < mo.dim; ++n)
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
      // deltas of the border faces of this coarse cell, d[a][c] at (t1: 2A + a, t2: 2C + c)
      const int A = idx[t1] >> 1, Cc = mo.dim == 3 ? (idx[t2] >> 1) : 0;
      double    d[2][2] = {{0, 0}, {0, 0}};
      for (int a = 0; a < 2; ++a)
        for (int c2 = 0; c2 < (mo.dim == 3 ? 2 : 1); ++c2)
        {
          int q[3] = {0, 0, 0};
          q[n] = sd == 0 ? 0 : b[n];
          q[t1] = 2 * A + a;
          if (mo.dim == 3)
            q[t2] = 2 * Cc + c2;
          double bv = 0.0;
          border(n, q, bv);
          d[a][c2] = bv - base(n, q);
        }
      if (mo.dim == 2)
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

} // namespace oracle

using namespace oracle;

extern "C" {

struct oracle_mesh
{
  int32_t         dim, bx, by, bz, n_blocks, n_owned;
  const int32_t * level;
  const int32_t * neighbor;
  double          scaling_factor;
  const int32_t * outside_src;    // [n_blocks - n_owned]
  const int32_t * outside_normal; // [3 * (n_blocks - n_owned)], +1 below / -1 above the domain
  int32_t         bc[6];          // BC_MHD values for XMIN..ZMAX (FillOutside.h:55-61)
  const int32_t * coord;          // [3 * n_blocks] block coordinates at the block's level, or null
  const int32_t * fine_neighbor;  // [27 * 8 * n_blocks] children of refined neighbour regions, or null
  int32_t         prolongation;   // [amr] cell_centered_prolongation_type: 0 SIMPLE_COPY, 1 LINEAR_MINMOD
};

struct oracle_settings
{
  double  gamma0, cfl, slope_type, smallr, smallc;
  int32_t riemann;
  int32_t time_integrator; // [amr] time_integrator: 0 HANCOCK, 1 RK2_SSP
  int32_t gravity_enabled; // [gravity] enabled
  double  gravity[3];      // [gravity] uniform_gx, uniform_gy, uniform_gz
  int32_t viscosity_enabled; // [viscosity] enabled
  double  viscosity_mu;      // [viscosity] mu
  int32_t viscous_predictor; // [viscosity] hancock_predictor_enabled
};

static Mesh
to_mesh(const oracle_mesh * om)
{
  Mesh m;
  m.dim = om->dim;
  m.bx = om->bx;
  m.by = om->by;
  m.bz = om->dim == 3 ? om->bz : 1;
  m.n_blocks = om->n_blocks;
  m.n_owned = om->n_owned;
  m.level = om->level;
  m.neighbor = om->neighbor;
  m.coord = om->coord;
  m.fine = om->fine_neighbor;
  m.prolongation = om->prolongation;
  m.scaling_factor = om->scaling_factor;
  return m;
}

static Settings
to_settings(const oracle_settings * os)
{
  Settings st = make_settings(os->gamma0, os->cfl, os->slope_type, os->smallr, os->smallc, os->riemann);
  st.rk2 = os->time_integrator == 1;
  st.gravity = os->gravity_enabled != 0;
  for (int d = 0; d < 3; ++d)
    st.grav[d] = os->gravity[d];
  st.viscosity = os->viscosity_enabled != 0;
  st.mu = os->viscosity_mu;
  st.visc_predictor = os->viscous_predictor != 0;
  return st;
}

// One do_time_step: U2 and B2 must equal U and B on entry (SolverGodunovMHD.cpp:166-167, 545-548).
// Returns 0, -1 (missing neighbour), -2 (level jump), -3 (unknown Riemann solver).
static double * g_flux_sink = nullptr; // oracle_step_fluxes: copy of the per-block face fluxes

int
oracle_step(const oracle_mesh * om, const oracle_settings * os, const double * U, double * U2,
            const double * B, double * B2, double dt)
{
  const Mesh     m = to_mesh(om);
  const Settings s = to_settings(os);
  for (int b = 0; b < m.n_owned; ++b)
    for (int sl = 0; sl < 27; ++sl)
    {
      const int id = m.neighbor[(int64_t)b * 27 + sl];
      if (id >= 0 && id < m.n_owned && m.level[id] != m.level[b] && (m.level[id] != m.level[b] - 1 || !m.coord))
        return -2;
    }
  Fields f;
  f.m = &m;
  f.L = block_layout(m);
  f.U = U;
  f.B = B;
  const int64_t                    ne = emf_count(m) * (m.dim == 3 ? 3 : 1);
  const FluxLayout                 FL = flux_layout(m);
  std::vector<double>              emf_all((size_t)m.n_owned * ne, 0.0);
  std::vector<std::vector<double>> flux_all((size_t)m.n_owned);
  std::vector<std::vector<double>> visc_all(s.viscosity ? (size_t)m.n_owned : 0);
  int                              status = 0;
  // stages K2-K11 per block: everything up to the face fluxes and the raw edge EMFs
#pragma omp parallel
  {
    StepWork w;
#pragma omp for schedule(dynamic, 1)
    for (int blk = 0; blk < m.n_owned; ++blk)
    {
      const double dx = cell_length(m, m.level[blk]);
      const double dtdx = dt / dx;
      flux_all[blk].assign((size_t)FL.total, 0.0);
      int st = fill_bface_ghosted(m, f, blk, w);
      if (st == 0)
        st = convert_to_primitives(m, f, s, blk, w);
      if (st == 0)
      {
        compute_slopes(m, s, w);
        compute_predictor(m, s, dt, dtdx, dx, w);
        compute_elec_field(m, w);
        compute_sfacemag(m, dtdx, w);
        for (int dir = 0; dir < m.dim && st == 0; ++dir)
          st = compute_fluxes(m, s, dtdx, dir, w, flux_all[blk].data());
        if (s.viscosity)
        {
          visc_all[blk].assign((size_t)FL.total, 0.0);
          for (int dir = 0; dir < m.dim; ++dir)
            compute_viscous_fluxes(m, s, dtdx, dx, dir, w, visc_all[blk].data());
        }
        if (st == 0)
          compute_emfs(m, s, dtdx, w, &emf_all[(size_t)blk * ne]);
      }
      if (st != 0)
      {
#pragma omp critical
        status = st;
      }
    }
  }
  if (status != 0)
    return status;
  if (g_flux_sink)
    for (int blk = 0; blk < m.n_owned; ++blk)
      std::memcpy(g_flux_sink + (size_t)blk * FL.total, flux_all[blk].data(), sizeof(double) * FL.total);
  // conservative update with the coarse/fine flux correction, then EMF correction + CT
#pragma omp parallel for schedule(dynamic, 1)
  for (int blk = 0; blk < m.n_owned; ++blk)
  {
    double * U2blk = U2 + (int64_t)blk * 5 * f.L.ncell;
    double * B2blk = B2 + (int64_t)blk * f.L.nface;
    int      st = update_u(m, blk, flux_all, U2blk, B2blk + f.L.nfx + f.L.nfy);
    // viscous fluxes through the same update, after the three hydro directions
    // (GodunovImplemV0.cpp:179-192)
    if (st == 0 && s.viscosity)
      st = update_u(m, blk, visc_all, U2blk, B2blk + f.L.nfx + f.L.nfy);
    if (st == 0)
      st = correct_emf_and_update_b(m, blk, emf_all, B2blk);
    if (st == 0 && s.gravity)
      add_gravity_source(m, s, dt, U + (int64_t)blk * 5 * f.L.ncell, U2blk, f.L.ncell);
    if (st != 0)
    {
#pragma omp critical
      status = st;
    }
  }
  return status;
}

// The per-block stage arrays of oracle_step for block blk (for checks against the reference's own
// stage functors): ghosted primitives q [11][(b+4)^d], slopes [dim][8][(b+2)^d], predictor
// q2 [8][(b+2)^d], edge electric field e [1|3][(b+4)^d], face source sf [2|3][(b+2)^d]; each array
// variable-major, x fastest (2D: one z layer). Returns 0 or the stage error.
int
oracle_block_stages(const oracle_mesh * om, const oracle_settings * os, const double * U, const double * B, double dt,
                    int blk, double * q, double * slopes, double * q2, double * e, double * sf)
{
  const Mesh     m = to_mesh(om);
  const Settings s = to_settings(os);
  if (blk < 0 || blk >= m.n_owned)
    return -1;
  Fields f;
  f.m = &m;
  f.L = block_layout(m);
  f.U = U;
  f.B = B;
  StepWork     w;
  const double dx = cell_length(m, m.level[blk]);
  const double dtdx = dt / dx;
  int          st = fill_bface_ghosted(m, f, blk, w);
  if (st == 0)
    st = convert_to_primitives(m, f, s, blk, w);
  if (st != 0)
    return st;
  compute_slopes(m, s, w);
  compute_predictor(m, s, dt, dtdx, dx, w);
  compute_elec_field(m, w);
  compute_sfacemag(m, dtdx, w);
  auto put = [](double * dst, const Box & bx) {
    if (dst)
      std::memcpy(dst, bx.a.data(), sizeof(double) * bx.a.size());
  };
  put(q, w.Q);
  if (slopes)
  {
    const size_t ns = w.Sx.a.size();
    std::memcpy(slopes, w.Sx.a.data(), sizeof(double) * ns);
    std::memcpy(slopes + ns, w.Sy.a.data(), sizeof(double) * ns);
    if (m.dim == 3)
      std::memcpy(slopes + 2 * ns, w.Sz.a.data(), sizeof(double) * ns);
  }
  put(q2, w.Q2);
  put(e, w.E);
  put(sf, w.SF);
  return 0;
}

// The ghosted face field of block blk (the face-B ghost layer oracle_step builds, fill_bface_ghosted):
// Bx on faces [-2, bx+2] x cells [-2, b+2) of the other axes, By and Bz likewise (2D: the cell-centred Bz
// on [-2, b+2)^2), x fastest, components concatenated. Returns 0 or -1 (missing neighbour).
int
oracle_block_ghost_faces(const oracle_mesh * om, const double * U, const double * B, int blk, double * out)
{
  const Mesh m = to_mesh(om);
  if (blk < 0 || blk >= m.n_owned)
    return -1;
  Fields f;
  f.m = &m;
  f.L = block_layout(m);
  f.U = U;
  f.B = B;
  StepWork w;
  if (fill_bface_ghosted(m, f, blk, w) != 0)
    return -1;
  size_t off = 0;
  for (const Box * bb : {&w.Bgx, &w.Bgy, &w.Bgz})
  {
    std::memcpy(out + off, bb->a.data(), sizeof(double) * bb->a.size());
    off += bb->a.size();
  }
  return 0;
}

// Face fluxes [dir][8][faces] (times dt/dx) and raw edge EMFs [1|3][(b+1)^d] (times dt/dx, before the
// border correction) of block blk, as oracle_step computes them.
int
oracle_block_fluxes_emf(const oracle_mesh * om, const oracle_settings * os, const double * U, const double * B,
                        double dt, int blk, double * fluxes, double * emf)
{
  const Mesh     m = to_mesh(om);
  const Settings s = to_settings(os);
  if (blk < 0 || blk >= m.n_owned)
    return -1;
  Fields f;
  f.m = &m;
  f.L = block_layout(m);
  f.U = U;
  f.B = B;
  StepWork     w;
  const double dx = cell_length(m, m.level[blk]);
  const double dtdx = dt / dx;
  int          st = fill_bface_ghosted(m, f, blk, w);
  if (st == 0)
    st = convert_to_primitives(m, f, s, blk, w);
  if (st != 0)
    return st;
  compute_slopes(m, s, w);
  compute_predictor(m, s, dt, dtdx, dx, w);
  compute_elec_field(m, w);
  compute_sfacemag(m, dtdx, w);
  const FluxLayout FL = flux_layout(m);
  std::vector<double> F((size_t)FL.total, 0.0);
  for (int dir = 0; dir < m.dim && st == 0; ++dir)
    st = compute_fluxes(m, s, dtdx, dir, w, F.data());
  if (st != 0)
    return st;
  std::memcpy(fluxes, F.data(), sizeof(double) * F.size());
  compute_emfs(m, s, dtdx, w, emf);
  return 0;
}

// Viscous face fluxes of one owned block (compute_viscous_fluxes on the block's t^n primitives),
// times dt/dx, per direction [8][faces] concatenated.
int
oracle_block_viscous_fluxes(const oracle_mesh * om, const oracle_settings * os, const double * U, const double * B,
                            double dt, int blk, double * fluxes)
{
  const Mesh     m = to_mesh(om);
  const Settings s = to_settings(os);
  if (blk < 0 || blk >= m.n_owned)
    return -1;
  Fields f;
  f.m = &m;
  f.L = block_layout(m);
  f.U = U;
  f.B = B;
  StepWork     w;
  const double dx = cell_length(m, m.level[blk]);
  int          st = fill_bface_ghosted(m, f, blk, w);
  if (st == 0)
    st = convert_to_primitives(m, f, s, blk, w);
  if (st != 0)
    return st;
  const FluxLayout    FL = flux_layout(m);
  std::vector<double> F((size_t)FL.total, 0.0);
  for (int dir = 0; dir < m.dim; ++dir)
    compute_viscous_fluxes(m, s, dt / dx, dx, dir, w, F.data());
  std::memcpy(fluxes, F.data(), sizeof(double) * F.size());
  return 0;
}

// oracle_step that also copies the per-block face fluxes (flux * dt/dx, [block][dir][var][face]) to
// fluxes_out, for checks of the coarse/fine flux correction.
int
oracle_step_fluxes(const oracle_mesh * om, const oracle_settings * os, const double * U, double * U2,
                   const double * B, double * B2, double dt, double * fluxes_out)
{
  g_flux_sink = fluxes_out;
  const int st = oracle_step(om, os, U, U2, B, B2, dt);
  g_flux_sink = nullptr;
  return st;
}

// One cell's 1/dt (ComputeDtMHDFunctor.cpp:86-151; with gravity :155-249): the fast speeds v over dx,
// with gravity corrected by k / (sqrt(1 + 2k) - 1), k = sum|g| dx / |v|^2 (floored at 1e-4); with
// viscosity at least 4 nu / dx^2, nu = mu / rho (conservative density).
static double
cfl_inv_dt(const Mesh & m, const Settings & s, const double * v, double dx, double rho)
{
  double val;
  if (s.gravity)
  {
    double v2 = v[0] * v[0] + v[1] * v[1];
    if (m.dim == 3)
      v2 += v[2] * v[2];
    double k = std::fabs(s.grav[0]) + std::fabs(s.grav[1]);
    if (m.dim == 3)
      k += std::fabs(s.grav[2]);
    k *= dx / v2;
    k = std::fmax(k, 1e-4);
    const double factor = k / (std::sqrt(1.0 + 2.0 * k) - 1.0);
    val = 0.0;
    val += (v[0] * factor) / dx;
    val += (v[1] * factor) / dx;
    if (m.dim == 3)
      val += (v[2] * factor) / dx;
  }
  else
    val = m.dim == 3 ? v[0] / dx + v[1] / dx + v[2] / dx : v[0] / dx + v[1] / dx;
  if (s.viscosity)
  {
    const double nu = s.mu / rho;
    val = std::fmax(val, 4 * nu / (dx * dx));
  }
  return val;
}

// AddGravitySourceTerm alone on n_blocks blocks of size b: Unew [n][5][cells] updated in place from
// Uold (same layout), with gravity g[3] and time step dt.
int
oracle_gravity_source(int dim, const int * b, int n_blocks, const double * g, double dt, const double * Uold,
                      double * Unew)
{
  if (dim != 2 && dim != 3)
    return -1;
  Mesh m{};
  m.dim = dim;
  m.bx = b[0];
  m.by = b[1];
  m.bz = dim == 3 ? b[2] : 1;
  Settings s{};
  s.gravity = 1;
  for (int d = 0; d < 3; ++d)
    s.grav[d] = g[d];
  const int64_t ncell = block_layout(m).ncell;
  for (int n = 0; n < n_blocks; ++n)
    add_gravity_source(m, s, dt, Uold + (size_t)n * 5 * ncell, Unew + (size_t)n * 5 * ncell, ncell);
  return 0;
}

// Conservative update alone (update_u) of owned block blk with its face fluxes `fluxes` (per
// direction [8][faces] concatenated, times dt/dx): U2blk [5][cells] and the block's faces B2blk (2D:
// the cell-centred Bz) updated in place. Blocks with finer neighbours need their fluxes too: -1.
int
oracle_block_update(const oracle_mesh * om, int blk, const double * fluxes, double * U2blk, double * B2blk)
{
  const Mesh m = to_mesh(om);
  if (blk < 0 || blk >= m.n_owned)
    return -1;
  const FluxLayout                 FL = flux_layout(m);
  const BlockLayout                L = block_layout(m);
  std::vector<std::vector<double>> flux_all((size_t)m.n_blocks);
  flux_all[blk].assign(fluxes, fluxes + FL.total);
  return update_u(m, blk, flux_all, U2blk, B2blk + L.nfx + L.nfy);
}

// CT update alone on n_blocks blocks of size b (read_emf_and_update): B [n][faces] updated in place by
// emf [n][ncomp][(b+1)^d] (ncomp 3 in 3D, 1 in 2D).
// The border EMF correction alone over the owned blocks: emf_in [n_owned][1|3][(b+1)^d] raw EMFs (as
// oracle_block_fluxes_emf returns them), emf_out the same layout after correct_emf. Returns 0 or the
// first error.
int
oracle_correct_emf(const oracle_mesh * om, const double * emf_in, double * emf_out)
{
  const Mesh          m = to_mesh(om);
  const int64_t       ne = emf_count(m) * (m.dim == 3 ? 3 : 1);
  std::vector<double> emf_all(emf_in, emf_in + (size_t)m.n_owned * ne);
  int                 status = 0;
  for (int blk = 0; blk < m.n_owned && status == 0; ++blk)
  {
    std::vector<double> emf2;
    status = correct_emf(m, blk, emf_all, emf2);
    if (status == 0)
      std::memcpy(emf_out + (size_t)blk * ne, emf2.data(), sizeof(double) * ne);
  }
  return status;
}

// The conservative update alone over the owned blocks, coarse/fine flux sums included: fluxes
// [n_owned][dir][var][face] (flux * dt/dx, as oracle_step_fluxes writes them), U2 [n_owned][5][cells] and
// the faces B2 (2D: the cell-centred Bz) updated in place. Returns 0 or the first error.
int
oracle_update_all(const oracle_mesh * om, const double * fluxes, double * U2, double * B2)
{
  const Mesh        m = to_mesh(om);
  const BlockLayout L = block_layout(m);
  const FluxLayout  FL = flux_layout(m);
  std::vector<std::vector<double>> flux_all((size_t)m.n_owned);
  for (int blk = 0; blk < m.n_owned; ++blk)
    flux_all[blk].assign(fluxes + (size_t)blk * FL.total, fluxes + (size_t)(blk + 1) * FL.total);
  int status = 0;
  for (int blk = 0; blk < m.n_owned && status == 0; ++blk)
    status = update_u(m, blk, flux_all, U2 + (int64_t)blk * 5 * L.ncell, B2 + (int64_t)blk * L.nface + L.nfx + L.nfy);
  return status;
}

int
oracle_ct_update(int dim, const int * b, int n_blocks, const double * emf, double * B)
{
  if (dim != 2 && dim != 3)
    return -1;
  Mesh m{};
  m.dim = dim;
  m.bx = b[0];
  m.by = b[1];
  m.bz = dim == 3 ? b[2] : 1;
  const BlockLayout L = block_layout(m);
  const int64_t     ne = emf_count(m) * (dim == 3 ? 3 : 1);
  for (int n = 0; n < n_blocks; ++n)
    read_emf_and_update(m, emf + (size_t)n * ne, B + (size_t)n * L.nface);
  return 0;
}

// ComputeDtMHDFunctor::apply over owned blocks; returns invDt (max over cells).
double
oracle_inv_dt(const oracle_mesh * om, const oracle_settings * os, const double * U, const double * B)
{
  const Mesh     m = to_mesh(om);
  const Settings s = to_settings(os);
  Fields         f;
  f.m = &m;
  f.L = block_layout(m);
  f.U = U;
  f.B = B;
  double inv_dt = 0.0;
#pragma omp parallel for reduction(max : inv_dt) schedule(static)
  for (int blk = 0; blk < m.n_owned; ++blk)
  {
    const double dx = cell_length(m, m.level[blk]);
    for (int k = 0; k < m.bz; ++k)
      for (int j = 0; j < m.by; ++j)
        for (int i = 0; i < m.bx; ++i)
        {
          double u[8], q[8], v[3] = {0.0, 0.0, 0.0};
          for (int n = 0; n < 5; ++n)
            u[n] = f.u(blk, n, i, j, k);
          u[IA] = 0.5 * (f.bx(blk, i, j, k) + f.bx(blk, i + 1, j, k));
          u[IB] = 0.5 * (f.by(blk, i, j, k) + f.by(blk, i, j + 1, k));
          if (m.dim == 3)
            u[IC] = 0.5 * (f.bz(blk, i, j, k) + f.bz(blk, i, j, k + 1));
          else
            u[IC] = 0.5 * (f.bz(blk, i, j, 0) + f.bz(blk, i, j, 0));
          compute_primitives(u, q, nullptr, s);
          find_speed_info(q, m.dim, v, s);
          inv_dt = std::fmax(inv_dt, cfl_inv_dt(m, s, v, dx, u[ID]));
        }
  }
  return inv_dt;
}

// FillOutsideCellFunctor (border_conditions/FillOutside.cpp:97-395) over the outside blocks
// [n_owned, n_blocks). Hydro: for every domain face the inside block touches on the outside block's
// side, ZERO_GRADIENT copies the first/last inside cell along the normal, WALL mirrors it and negates
// the normal velocity (later faces overwrite earlier ones, as in the reference loop). Face B:
// ZERO_GRADIENT clamps the face index to the first/last face along each outside direction; WALL leaves
// the index unchanged (a TODO in the reference) so the same face of the inside block is copied.
void
oracle_fill_outside(const oracle_mesh * om, double * U, double * B)
{
  const Mesh        m = to_mesh(om);
  const BlockLayout L = block_layout(m);
  const int         n_out = m.n_blocks - m.n_owned;
  const int         bs[3] = {m.bx, m.by, m.bz};
  enum
  {
    ZERO_GRADIENT = 2,
    WALL = 3
  };
  for (int o = 0; o < n_out; ++o)
  {
    const int      ob = m.n_owned + o, ib = om->outside_src[o];
    const int32_t *nrm = om->outside_normal + 3 * o;
    for (int k = 0; k < m.bz; ++k)
      for (int j = 0; j < m.by; ++j)
        for (int i = 0; i < m.bx; ++i)
        {
          const int     co[3] = {i, j, k};
          const int64_t c = i + (int64_t)m.bx * (j + (int64_t)m.by * k);
          for (int face = 0; face < 2 * m.dim; ++face)
          {
            const int  d = face / 2;
            const bool applies = (face % 2 == 0) ? nrm[d] > 0 : nrm[d] < 0;
            if (!applies)
              continue;
            int ci[3] = {co[0], co[1], co[2]};
            if (om->bc[face] == ZERO_GRADIENT)
              ci[d] = (face % 2 == 0) ? 0 : bs[d] - 1;
            else if (om->bc[face] == WALL)
              ci[d] = bs[d] - 1 - co[d];
            else
              continue;
            const int64_t cin = ci[0] + (int64_t)m.bx * (ci[1] + (int64_t)m.by * ci[2]);
            for (int v = 0; v < 5; ++v)
              U[((int64_t)ob * 5 + v) * L.ncell + c] = U[((int64_t)ib * 5 + v) * L.ncell + cin];
            if (om->bc[face] == WALL)
              U[((int64_t)ob * 5 + 2 + d) * L.ncell + c] *= -1;
          }
        }
    for (int64_t f = 0; f < L.nface; ++f)
    {
      int     comp, nx, ny, nz;
      int64_t r, base;
      if (f < L.nfx)
      {
        comp = 0; r = f; nx = m.bx + 1; ny = m.by; nz = m.bz; base = 0;
      }
      else if (f < L.nfx + L.nfy)
      {
        comp = 1; r = f - L.nfx; nx = m.bx; ny = m.by + 1; nz = m.bz; base = L.nfx;
      }
      else
      {
        comp = 2; r = f - L.nfx - L.nfy; nx = m.bx; ny = m.by; nz = m.dim == 3 ? m.bz + 1 : m.bz;
        base = L.nfx + L.nfy;
      }
      int       idx[3] = {(int)(r % nx), (int)((r / nx) % ny), (int)(r / ((int64_t)nx * ny))};
      const int fsz[3] = {nx, ny, nz};
      for (int d = 0; d < m.dim; ++d)
      {
        if (nrm[d] > 0 && om->bc[2 * d] == ZERO_GRADIENT)
          idx[d] = 0;
        else if (nrm[d] < 0 && om->bc[2 * d + 1] == ZERO_GRADIENT)
          idx[d] = fsz[d] - 1;
      }
      (void)comp;
      const int64_t fin = idx[0] + (int64_t)nx * (idx[1] + (int64_t)ny * idx[2]);
      B[(int64_t)ob * L.nface + f] = B[(int64_t)ib * L.nface + base + fin];
    }
  }
}

// nsteps of (dt = cfl / invDt; fill outside blocks; do_time_step; U <- U2, B <- B2) on U/B in place
// (SolverGodunovMHD::next_iteration_impl + godunov_unsplit, SolverGodunovMHD.cpp:407-549). dt_out[n] receives
// the dt of step n. Returns 0 or the first step error.
int
oracle_run_to(const oracle_mesh * om, const oracle_settings * os, double * U, double * B, int nsteps,
              double * dt_out, double * t, double t_end);

int
oracle_run(const oracle_mesh * om, const oracle_settings * os, double * U, double * B, int nsteps,
           double * dt_out)
{
  return oracle_run_to(om, os, U, B, nsteps, dt_out, nullptr, 0.0);
}

// As oracle_run, with the solver's end-time control when t != nullptr: dt = min(cfl/invDt, t_end - t),
// and dt = 0 once t has reached t_end (the state is then carried over unchanged).
int
oracle_run_to(const oracle_mesh * om, const oracle_settings * os, double * U, double * B, int nsteps,
              double * dt_out, double * t, double t_end)
{
  const Mesh        m = to_mesh(om);
  const BlockLayout L = block_layout(m);
  const size_t      nu = (size_t)m.n_blocks * 5 * L.ncell;
  const size_t      nb = (size_t)m.n_blocks * L.nface;
  std::vector<double> U2(U, U + nu), B2(B, B + nb);
  for (int n = 0; n < nsteps; ++n)
  {
    const double inv_dt = oracle_inv_dt(om, os, U, B);
    double       dt = os->cfl / inv_dt;
    if (t)
    {
      const double rem = t_end - *t;
      if (dt > rem)
        dt = rem;
      if (!(rem > 0.0))
        dt = 0.0;
      *t += dt;
    }
    if (m.n_blocks > m.n_owned)
    {
      oracle_fill_outside(om, U, B);
      std::memcpy(U2.data(), U, nu * sizeof(double));
      std::memcpy(B2.data(), B, nb * sizeof(double));
    }
    if (dt_out)
      dt_out[n] = dt;
    if (os->time_integrator == 1)
    {
      // RK2_SSP (SolverGodunovMHD.cpp:551-647): U_RK = U + L(U); U2 = U_RK + L(U_RK);
      // U = 1/2 U + 1/2 U2. The stage-1 combination (core LinearCombination, coefficients 0 and 1)
      // leaves U_RK unchanged.
      std::vector<double> Urk(U, U + nu), Brk(B, B + nb);
      int                 st = oracle_step(om, os, U, Urk.data(), B, Brk.data(), dt);
      if (st != 0)
        return st;
      if (m.n_blocks > m.n_owned)
        oracle_fill_outside(om, Urk.data(), Brk.data());
      std::memcpy(U2.data(), Urk.data(), nu * sizeof(double));
      std::memcpy(B2.data(), Brk.data(), nb * sizeof(double));
      st = oracle_step(om, os, Urk.data(), U2.data(), Brk.data(), B2.data(), dt);
      if (st != 0)
        return st;
      const size_t nuo = (size_t)m.n_owned * 5 * L.ncell, nbo = (size_t)m.n_owned * L.nface;
      for (size_t i = 0; i < nuo; ++i)
        U[i] = 0.5 * U[i] + 0.5 * U2[i];
      for (size_t i = 0; i < nbo; ++i)
        B[i] = 0.5 * B[i] + 0.5 * B2[i];
      continue;
    }
    const int st = oracle_step(om, os, U, U2.data(), B, B2.data(), dt);
    if (st != 0)
      return st;
    std::memcpy(U, U2.data(), nu * sizeof(double));
    std::memcpy(B, B2.data(), nb * sizeof(double));
  }
  return 0;
}

// Refinement flags of the owned blocks (-1 coarsen, 0 keep, +1 refine); see RefineParams.
void
oracle_refine_flags(const oracle_mesh * om, const oracle_settings * os, const double * U, const double * B,
                    const int32_t * params_i, const double * params_d, int8_t * flags)
{
  const Mesh     m = to_mesh(om);
  const Settings s = to_settings(os);
  Fields         f;
  f.m = &m;
  f.L = block_layout(m);
  f.U = U;
  f.B = B;
  RefineParams rp{params_i[0], params_i[1], params_i[2], params_i[3], params_i[4], params_d[0], params_d[1],
                  params_d[2]};
#pragma omp parallel for schedule(dynamic, 1)
  for (int blk = 0; blk < m.n_owned; ++blk)
  {
    const double err = block_refine_error(m, f, s, rp, blk);
    const int    lv = m.level[blk];
    flags[blk] = (err > rp.eps_refine && lv < rp.level_max) ? 1 : ((err < rp.eps_coarsen && lv > rp.level_min) ? -1 : 0);
  }
}

// Remap U, B of the old mesh to the new one (remap rows of BlockMesh.adapt: kind, sources, fine
// face neighbours); owned blocks of the new arrays are written.
int
oracle_remap(const oracle_mesh * om_old, const oracle_mesh * om_new, const int32_t * remap, const double * Uo,
             const double * Bo, double * Un, double * Bn)
{
  const Mesh mo = to_mesh(om_old), mn = to_mesh(om_new);
  Fields     fo;
  fo.m = &mo;
  fo.L = block_layout(mo);
  fo.U = Uo;
  fo.B = Bo;
  const BlockLayout L = fo.L;
  int               status = 0;
#pragma omp parallel for schedule(dynamic, 1)
  for (int n = 0; n < mn.n_owned; ++n)
  {
    const int32_t * rm = remap + (int64_t)n * 15;
    double *        Ub = Un + (int64_t)n * 5 * L.ncell;
    double *        Bb = Bn + (int64_t)n * L.nface;
    if (rm[0] == 0)
    {
      std::memcpy(Ub, Uo + (int64_t)rm[1] * 5 * L.ncell, sizeof(double) * 5 * L.ncell);
      std::memcpy(Bb, Bo + (int64_t)rm[1] * L.nface, sizeof(double) * L.nface);
      continue;
    }
    // cells
    for (int k = 0; k < mo.bz; ++k)
      for (int j = 0; j < mo.by; ++j)
        for (int i = 0; i < mo.bx; ++i)
        {
          const int     q[3] = {i, j, k};
          const int64_t c = i + (int64_t)mo.bx * (j + (int64_t)mo.by * k);
          for (int v = 0; v < 5; ++v)
          {
            double val = 0.0;
            if (rm[0] == 2)
            {
              Region r{RK_FINER, -1, {0, 0, 0}, rm + 1};
              if (!restrict_cell(mo, fo, r, q, v, val))
                status = -1;
            }
            else
            {
              const int ch = rm[2];
              const int I[3] = {((ch & 1) * mo.bx + i) >> 1, (((ch >> 1) & 1) * mo.by + j) >> 1,
                                (mo.dim == 3 ? (((ch >> 2) & 1) * mo.bz + k) >> 1 : 0)};
              val = fo.u(rm[1], v, I[0], I[1], I[2]);
            }
            Ub[v * L.ncell + c] = val;
          }
        }
    // faces
    for (int64_t fi = 0; fi < L.nface; ++fi)
    {
      int     comp, nx, ny;
      int64_t rr;
      if (fi < L.nfx)
      {
        comp = 0; rr = fi; nx = mo.bx + 1; ny = mo.by;
      }
      else if (fi < L.nfx + L.nfy)
      {
        comp = 1; rr = fi - L.nfx; nx = mo.bx; ny = mo.by + 1;
      }
      else
      {
        comp = 2; rr = fi - L.nfx - L.nfy; nx = mo.bx; ny = mo.by;
      }
      const int idx[3] = {(int)(rr % nx), (int)((rr / nx) % ny), (int)(rr / ((int64_t)nx * ny))};
      double    val = 0.0;
      if (rm[0] == 2)
      {
        // mean of the children's faces; a face shared with a kept leaf of the same level is its copy
        Region r{RK_FINER, -1, {0, 0, 0}, rm + 1};
        const int sd = (mo.dim == 2 && comp == 2) ? -1 : (idx[comp] == 0 ? 0 : (idx[comp] == (comp == 0 ? mo.bx : (comp == 1 ? mo.by : mo.bz)) ? 1 : -1));
        if (sd >= 0 && rm[9 + 2 * comp + sd] >= 0)
        {
          int qq[3] = {idx[0], idx[1], idx[2]};
          qq[comp] = sd == 0 ? (comp == 0 ? mo.bx : (comp == 1 ? mo.by : mo.bz)) : 0;
          val = fo.face(rm[9 + 2 * comp + sd], comp, qq[0], qq[1], qq[2]);
        }
        else if (!region_face(mo, fo, r, comp, idx, val))
          status = -1;
      }
      else
        val = prolonged_face(mo, fo, rm, comp, idx);
      Bb[fi] = val;
    }
  }
  return status;
}

// Per-call entry points for the known-answer tests.
void
oracle_riemann(const oracle_settings * os, const double * qL_in, const double * qR_in, double * flux)
{
  const Settings s = to_settings(os);
  double         qL[8], qR[8];
  std::memcpy(qL, qL_in, sizeof qL);
  std::memcpy(qR, qR_in, sizeof qR);
  for (int v = 0; v < 8; ++v)
    flux[v] = 0.0;
  riemann_mhd(qL, qR, flux, s);
}

double
oracle_compute_emf(const oracle_settings * os, const double * q4x8, int emf_dir)
{
  const Settings s = to_settings(os);
  double         qe[4][8];
  std::memcpy(qe, q4x8, sizeof qe);
  return compute_emf(qe, emf_dir, s);
}

void
oracle_compute_primitives(const oracle_settings * os, const double * u, double * q, double * c)
{
  const Settings s = to_settings(os);
  compute_primitives(u, q, c, s);
}

void
oracle_find_speed_info(const oracle_settings * os, const double * q, int dim, double * out)
{
  const Settings s = to_settings(os);
  find_speed_info(q, dim, out, s);
}

double
oracle_find_speed_fast(const oracle_settings * os, const double * q, int dir)
{
  const Settings s = to_settings(os);
  return find_speed_fast(q, dir, s);
}

} // extern "C"

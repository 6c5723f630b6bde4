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
// Assumptions where the reference relies on kalypsso-core (absent, so these are unpinned):
//   * all neighbours are at the same AMR level (uniform meshes); a level jump is rejected;
//   * the face-B ghost layer is a copy of the neighbour's faces; faces on the block border are
//     taken from the block itself (they equal the neighbour's copy whenever shared faces agree);
//   * dx = (1 / (bx * 2^level)) * scaling_factor;
//   * an edge on a block border has as siblings the blocks sharing it: one across a block face,
//     three around a block edge (2D: block corner). Outside blocks count as valid siblings but
//     are not averaged in, as in the reference.
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
  const int32_t * neighbor;   // [n_blocks * 27], -1 when absent
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

// Locate the block and local coordinates holding cell (i,j,k) of block blk. Returns -1 if the
// neighbour does not exist.
static int
locate_cell(const Mesh & m, int blk, int & i, int & j, int & k)
{
  const int ox = i < 0 ? -1 : (i >= m.bx ? 1 : 0);
  const int oy = j < 0 ? -1 : (j >= m.by ? 1 : 0);
  const int oz = m.dim == 3 ? (k < 0 ? -1 : (k >= m.bz ? 1 : 0)) : 0;
  if (ox == 0 && oy == 0 && oz == 0)
    return blk;
  const int nb = m.neighbor[(int64_t)blk * 27 + nb_slot(ox, oy, oz)];
  i -= ox * m.bx;
  j -= oy * m.by;
  k -= oz * m.bz;
  return nb;
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
  Box F;             // flux, 8 vars
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

// Fill ghosted face-B for block blk. Returns 0 or -1 when a needed neighbour is missing.
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

  // x faces: i in [-2, bx+2]
  for (int k = -gz; k < m.bz + gz; ++k)
    for (int j = -g; j < m.by + g; ++j)
      for (int i = -g; i <= m.bx + g; ++i)
      {
        const int ox = i < 0 ? -1 : (i > m.bx ? 1 : 0);
        const int oy = j < 0 ? -1 : (j >= m.by ? 1 : 0);
        const int oz = m.dim == 3 ? (k < 0 ? -1 : (k >= m.bz ? 1 : 0)) : 0;
        int       nb = blk;
        if (ox || oy || oz)
          nb = m.neighbor[(int64_t)blk * 27 + nb_slot(ox, oy, oz)];
        if (nb < 0)
          return -1;
        w.Bgx(i, j, k, 0) = f.bx(nb, i - ox * m.bx, j - oy * m.by, k - oz * m.bz);
      }
  // y faces: j in [-2, by+2]
  for (int k = -gz; k < m.bz + gz; ++k)
    for (int j = -g; j <= m.by + g; ++j)
      for (int i = -g; i < m.bx + g; ++i)
      {
        const int ox = i < 0 ? -1 : (i >= m.bx ? 1 : 0);
        const int oy = j < 0 ? -1 : (j > m.by ? 1 : 0);
        const int oz = m.dim == 3 ? (k < 0 ? -1 : (k >= m.bz ? 1 : 0)) : 0;
        int       nb = blk;
        if (ox || oy || oz)
          nb = m.neighbor[(int64_t)blk * 27 + nb_slot(ox, oy, oz)];
        if (nb < 0)
          return -1;
        w.Bgy(i, j, k, 0) = f.by(nb, i - ox * m.bx, j - oy * m.by, k - oz * m.bz);
      }
  // z faces (3D: k in [-2, bz+2]) or cell-centred Bz (2D)
  if (m.dim == 3)
  {
    for (int k = -gz; k <= m.bz + gz; ++k)
      for (int j = -g; j < m.by + g; ++j)
        for (int i = -g; i < m.bx + g; ++i)
        {
          const int ox = i < 0 ? -1 : (i >= m.bx ? 1 : 0);
          const int oy = j < 0 ? -1 : (j >= m.by ? 1 : 0);
          const int oz = k < 0 ? -1 : (k > m.bz ? 1 : 0);
          int       nb = blk;
          if (ox || oy || oz)
            nb = m.neighbor[(int64_t)blk * 27 + nb_slot(ox, oy, oz)];
          if (nb < 0)
            return -1;
          w.Bgz(i, j, k, 0) = f.bz(nb, i - ox * m.bx, j - oy * m.by, k - oz * m.bz);
        }
  }
  else
  {
    for (int j = -g; j < m.by + g; ++j)
      for (int i = -g; i < m.bx + g; ++i)
      {
        int ii = i, jj = j, kk = 0;
        const int nb = locate_cell(m, blk, ii, jj, kk);
        if (nb < 0)
          return -1;
        w.Bgz(i, j, 0, 0) = f.bz(nb, ii, jj, 0);
      }
  }
  return 0;
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
        int ii = i, jj = j, kk = k;
        const int nb = locate_cell(m, blk, ii, jj, kk);
        if (nb < 0)
          return -1;
        if (m.level[nb] != m.level[blk])
          return -2;
        double u[8];
        u[ID] = f.u(nb, ID, ii, jj, kk);
        u[IP] = f.u(nb, IP, ii, jj, kk);
        u[IU] = f.u(nb, IU, ii, jj, kk);
        u[IV] = f.u(nb, IV, ii, jj, kk);
        u[IW] = f.u(nb, IW, ii, jj, kk);
        // cell-centred B from face values (get_conservative_vars, .cpp:175-210)
        u[IA] = 0.5 * (w.Bgx(i, j, k, 0) + w.Bgx(i + 1, j, k, 0));
        u[IB] = 0.5 * (w.Bgy(i, j, k, 0) + w.Bgy(i, j + 1, k, 0));
        if (m.dim == 3)
          u[IC] = 0.5 * (w.Bgz(i, j, k, 0) + w.Bgz(i, j, k + 1, 0));
        else
          u[IC] = 0.5 * (w.Bgz(i, j, 0, 0) + w.Bgz(i, j, 0, 0));
        double q[8];
        compute_primitives(u, q, nullptr, s);
        w.Q(i, j, k, ID) = q[ID];
        w.Q(i, j, k, IP) = q[IP];
        w.Q(i, j, k, IU) = q[IU];
        w.Q(i, j, k, IV) = q[IV];
        w.Q(i, j, k, IW) = q[IW];
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
static void
compute_predictor(const Mesh & m, const Settings & s, double dtdx, StepWork & w)
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
        const double u = w.Q(i, j, k, IU);
        const double v = w.Q(i, j, k, IV);
        const double ww = w.Q(i, j, k, IW);
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

// compute_fluxes_and_store_{2d,3d} (scheme/ComputeHydroFluxesAndStoreFunctor.cpp:216-503) followed by
// read_fluxes_and_update_{2d,3d} (scheme/ReadFluxesAndConservativeUpdateFunctor.cpp:103-436) for one
// direction; U2 and (2D) Bz of block blk are updated in place.
static int
fluxes_and_update(const Mesh & m, const Settings & s, double dtdx, int dir, StepWork & w, double * U2blk,
                  double * Bz2blk)
{
  const int nx = m.bx + (dir == 0), ny = m.by + (dir == 1), nz = m.bz + (dir == 2 && m.dim == 3);
  w.F.init(0, nx, 0, ny, 0, nz, 8);
  const int di = dir == 0, dj = dir == 1, dk = dir == 2;
  // normal-B slot and the velocity / B component swapped with x for this direction
  const int ivel = dir == 0 ? IU : (dir == 1 ? IV : IW);
  const int imag = dir == 0 ? IA : (dir == 1 ? IB : IC);
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
        for (int v = 0; v < 8; ++v)
          w.F(i, j, k, v) = flux[v] * dtdx;
      }
  const int64_t ncell = (int64_t)m.bx * m.by * m.bz;
  for (int k = 0; k < m.bz; ++k)
    for (int j = 0; j < m.by; ++j)
      for (int i = 0; i < m.bx; ++i)
      {
        const int64_t c = i + (int64_t)m.bx * (j + (int64_t)m.by * k);
        for (int v = 0; v < 5; ++v)
        {
          double acc = 0.0;
          acc = acc + w.F(i, j, k, v);
          acc = acc - w.F(i + di, j + dj, k + dk, v);
          U2blk[v * ncell + c] += acc;
        }
        if (m.dim == 2)
        {
          double acc = 0.0;
          acc = acc + w.F(i, j, k, IC);
          acc = acc - w.F(i + di, j + dj, k + dk, IC);
          Bz2blk[c] += acc;
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
  A += w.SF(ia, ja, 0, 0);
  B += w.SF(ib, jb, 0, 1);
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
  B0 += w.SF(ijk0[0], ijk0[1], ijk0[2], dir0);
  B1 += w.SF(ijk1[0], ijk1[1], ijk1[2], dir1);
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

// correct_emf, uniform-level branch (scheme/CorrectEmfAtBlockBorderFunctor.cpp:94-360) followed by
// read_emf_and_update_{2d,3d} (scheme/ReadEmfAndUpdateFunctor.cpp:58-163) for block blk.
static void
correct_emf_and_update_b(const Mesh & m, int blk, const std::vector<double> & emf_all, double * B2blk)
{
  const int     ex = m.bx + 1, ey = m.by + 1, ez = m.dim == 3 ? m.bz + 1 : 1;
  const int64_t ne = emf_count(m);
  const int     ncomp = m.dim == 3 ? 3 : 1;
  const double *emf_self = &emf_all[(size_t)blk * ncomp * ne];
  std::vector<double> emf2(emf_self, emf_self + ncomp * ne); // deep_copy(emf2, emf)
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
          // sibling edges: across t0, across t1, across both
          int sib[3];
          int sidx[3][3];
          for (int n = 0; n < 3; ++n)
          {
            int o[3] = {0, 0, 0};
            if (n == 0 || n == 2)
              o[t0] = v0;
            if (n == 1 || n == 2)
              o[t1] = v1;
            const bool exists = (n == 0 && v0 != 0) || (n == 1 && v1 != 0) || (n == 2 && v0 != 0 && v1 != 0);
            sib[n] = exists ? m.neighbor[(int64_t)blk * 27 + nb_slot(o[0], o[1], o[2])] : -1;
            for (int d = 0; d < 3; ++d)
              sidx[n][d] = idx[d] - o[d] * bsz[d];
          }
          for (int n = 0; n < 3; ++n)
            if (sib[n] >= 0 && m.level[sib[n]] != m.level[blk])
              sib[n] = -2; // level jump: not supported by this restatement (checked by caller)
          const bool all_same = sib[0] >= 0 && sib[1] >= 0 && sib[2] >= 0;
          if (!all_same)
            continue; // neither coarser nor finer neighbours on uniform meshes: emf2 keeps emf
          const int64_t e = i + (int64_t)ex * (j + (int64_t)ey * k);
          double        acc = 0.0;
          int           count = 1;
          acc += emf_self[c * ne + e];
          for (int n = 0; n < 3; ++n)
          {
            if (sib[n] < m.n_owned)
            {
              const int64_t es = sidx[n][0] + (int64_t)ex * (sidx[n][1] + (int64_t)ey * sidx[n][2]);
              acc += emf_all[(size_t)sib[n] * ncomp * ne + c * ne + es];
              count++;
            }
          }
          emf2[c * ne + e] = acc / (double)count;
        }
  }
  // CT update
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

static bool
mesh_is_uniform(const Mesh & m)
{
  for (int b = 0; b < m.n_blocks; ++b)
    if (m.level[b] != m.level[0])
      return false;
  return true;
}

static double
cell_length(const Mesh & m, int level)
{
  return (1.0 / (double)((int64_t)m.bx << level)) * m.scaling_factor;
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
};

struct oracle_settings
{
  double  gamma0, cfl, slope_type, smallr, smallc;
  int32_t riemann;
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
  m.scaling_factor = om->scaling_factor;
  return m;
}

static Settings
to_settings(const oracle_settings * os)
{
  return make_settings(os->gamma0, os->cfl, os->slope_type, os->smallr, os->smallc, os->riemann);
}

// One do_time_step: U2 and B2 must equal U and B on entry (SolverGodunovMHD.cpp:166-167, 545-548).
// Returns 0, -1 (missing neighbour), -2 (level jump), -3 (unknown Riemann solver).
int
oracle_step(const oracle_mesh * om, const oracle_settings * os, const double * U, double * U2,
            const double * B, double * B2, double dt)
{
  const Mesh     m = to_mesh(om);
  const Settings s = to_settings(os);
  if (!mesh_is_uniform(m))
    return -2;
  Fields f;
  f.m = &m;
  f.L = block_layout(m);
  f.U = U;
  f.B = B;
  const int64_t       ne = emf_count(m) * (m.dim == 3 ? 3 : 1);
  std::vector<double> emf_all((size_t)m.n_owned * ne, 0.0);
  const double        dtdx = dt / cell_length(m, m.level[0]);
  int                 status = 0;
#pragma omp parallel
  {
    StepWork w;
#pragma omp for schedule(dynamic, 1)
    for (int blk = 0; blk < m.n_owned; ++blk)
    {
      int st = fill_bface_ghosted(m, f, blk, w);
      if (st == 0)
        st = convert_to_primitives(m, f, s, blk, w);
      if (st == 0)
      {
        compute_slopes(m, s, w);
        compute_predictor(m, s, dtdx, w);
        compute_elec_field(m, w);
        compute_sfacemag(m, dtdx, w);
        double * U2blk = U2 + (int64_t)blk * 5 * f.L.ncell;
        double * Bz2blk = B2 + (int64_t)blk * f.L.nface + f.L.nfx + f.L.nfy;
        for (int dir = 0; dir < m.dim && st == 0; ++dir)
          st = fluxes_and_update(m, s, dtdx, dir, w, U2blk, Bz2blk);
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
#pragma omp parallel for schedule(dynamic, 1)
  for (int blk = 0; blk < m.n_owned; ++blk)
    correct_emf_and_update_b(m, blk, emf_all, B2 + (int64_t)blk * f.L.nface);
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
          double u[8], q[8], v[3];
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
          double val = m.dim == 3 ? v[0] / dx + v[1] / dx + v[2] / dx : v[0] / dx + v[1] / dx;
          inv_dt = std::fmax(inv_dt, val);
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
    const int st = oracle_step(om, os, U, U2.data(), B, B2.data(), dt);
    if (st != 0)
      return st;
    std::memcpy(U, U2.data(), nu * sizeof(double));
    std::memcpy(B, B2.data(), nb * sizeof(double));
  }
  return 0;
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

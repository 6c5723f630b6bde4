// Fused MUSCL-Hancock + constrained-transport step over one tile of one leaf block per CTA.
//
// One launch replaces the reference's per-stage kernels of GodunovImplemV0::do_time_step
// (scheme/GodunovImplemV0.cpp:101-207): face-B ghost fill, primitive conversion, limited slopes,
// Hancock predictor, edge E, sFaceMag, HLLD face fluxes + conservative update (3 directions),
// 2D-HLLD edge EMFs, border EMF averaging and the CT face-B update. The tile and its 2-cell halo
// are gathered from the block and its neighbours (neighbour table) into shared memory; all
// intermediates stay on chip. Only U, B are read and U2, B2 written in HBM. The next step's CFL
// reduction (scheme/ComputeDtMHDFunctor.cpp:86-151) is fused into the epilogue.
//
// Template Cfg: compute type R (double: the FP64 drop-in, float: the mixed path), dimension,
// tile extents and threads per CTA. EXACT selects the reference's FP64 accumulation order for
// U2 (three rounded per-direction adds); otherwise the face terms are summed error-free in FP32
// (TwoSum: a sum and its rounding error) and both are added to U in FP64.
#pragma once

#include <cstdint>
#include <type_traits>

#include "mhd_math.cuh"

namespace gmhd
{

struct StepArgs
{
  const double * __restrict__ U;
  double * __restrict__ U2;
  const double * __restrict__ B;
  double * __restrict__ B2;
  const int32_t * __restrict__ neighbor; // [n_blocks * 27]
  const int32_t * __restrict__ level;    // [n_blocks]
  const int32_t * __restrict__ problem;  // [n_blocks] problem id, or null (single problem)
  int     n_owned;
  int     bx, by, bz;
  int     tiles_x, tiles_y, tiles_z;
  int64_t ncell, nfx, nfy, nface;
  double  gamma0, smallr, smallc, smallp, slope_type, scaling_factor, cfl;
  // the same in FP32 for the mixed path (converted once on the host: each FP64 conversion in the
  // kernel is an FP64-pipe instruction per warp)
  float   gamma0_f, smallr_f, smallc_f, smallp_f, slope_type_f;
  int     riemann;
  int     rk2;                                  // [amr] time_integrator RK2_SSP: no Hancock half step
  double  dt;                                   // used when dt_dev is null
  const double *             dt_dev;            // per problem dt on the device, or null
  unsigned long long *       invdt_out;         // per problem: fused CFL of U2/B2 (max), or null
  unsigned int *             health;            // OR of HEALTH_* flags
  int                        n_blocks;          // ids >= n_blocks in `neighbor` are virtual blocks
  Sources                    src;               // gravity / viscosity (viscous fluxes need C::VISC)
  int                        tile;              // host dispatch: tile x extent asked for (0: largest that fits)
  // the owned blocks blk_list[0 .. blk_count) only (device array; null: all); conforming meshes (no tile list)
  const int32_t *            blk_list;
  int                        blk_count;

  // ---- coarse/fine meshes (all null / zero when no block has a neighbour at another level) ----
  // Neighbour regions at another level are presented to the gather as virtual same-level blocks
  // (Uv, Bv), built each step by the ghost prepass; Bccv holds the cell-centred B of SIMPLE_COPY
  // ghosts (the coarse cell's own, ConvertToPrimitivesVariablesFunctor.cpp:439-446).
  const int8_t *  kind;       // [n_owned * 27] RegionKind of each neighbour slot
  const int32_t * fine;       // [n_blocks * 27 * 8] children of refined neighbour regions
  const double *  Uv;         // [virtual][5][ncell]
  const double *  Bv;         // [virtual][nface]
  const double *  Bccv;       // [virtual][3][ncell]
  int             prolongation; // 0 SIMPLE_COPY, 1 EXTRAPOLATE_LINEAR_MINMOD
  // Two passes: pass 1 runs every tile that has no finer neighbour (and, side data only, the
  // tiles that have both) and stores the fine-side face fluxes and raw border EMFs that coarse
  // neighbours need; pass 2 runs the tiles next to finer blocks and reads them
  // (ReadFluxesAndConservativeUpdateFunctor.cpp:141-172, CorrectEmfAtBlockBorderFunctor.cpp:94-360).
  const int32_t * tile_list;  // tiles of this launch (coarse/fine passes: ~tile for side-data-only tiles); null: all
  int             n_list;     // entries of tile_list
  int             pass;       // 0 (single pass), 1 or 2
  double *        flux_side;  // [slot][2*dim faces][NFV][flux_face_stride] fluxes * dt/dx
  const int32_t * flux_slot;  // [n_owned] slot of blocks with a coarser face neighbour, else -1
  int             flux_face_stride;
  double *        emf_side;   // [slot][ncomp][(bx+1)(by+1)(bz+1 | 1)] raw EMFs * dt/dx
  const int32_t * emf_slot;   // [n_owned] slot of blocks with any coarser neighbour, else -1
};

// Neighbour-region kinds of a coarse/fine mesh (RK_SAME also for the block itself).
enum : int
{
  RK_MISSING = 0,
  RK_SAME = 1,
  RK_COARSER = 2,
  RK_FINER = 3,
  RK_OUTSIDE = 4
};

enum : unsigned int
{
  HEALTH_MISSING_NEIGHBOR = 1u,
  HEALTH_LEVEL_JUMP = 2u,
  HEALTH_BAD_DENSITY = 4u,
  HEALTH_NONFINITE = 8u,
  HEALTH_LOW_BETA_FP64 = 16u, // informational: FP64 pressure recovery was used (mixed path)
};

template <typename R_, int DIM_, int TX_, int TY_, int TZ_, int NT_, bool EXACT_, bool AMR_ = false,
          bool VISC_ = false>
struct Cfg
{
  using R = R_;
  static constexpr bool AMR = AMR_;   // coarse/fine mesh support compiled in
  static constexpr bool VISC = VISC_; // viscous fluxes compiled in
  // CTAs per SM the register allocation must allow. 2D 16x16 tiles: three on the mixed path (24 warps
  // per SM, 74-76 registers without spills; 3 % faster than four CTAs at 64 registers on the 1024
  // field loops, and four were 20-25 % faster than the two CTAs of an unconstrained allocation), two
  // on the FP64 path (128 registers, a few spilled bytes; 13 % faster than one CTA)
  static constexpr int MINB = (DIM_ == 2 && TX_ == 16 && NT_ == 256) ? (EXACT_ ? 2 : 3) : 1;
  static constexpr int  DIM = DIM_;
  static constexpr int  TX = TX_;
  static constexpr int  TY = TY_;
  static constexpr int  TZ = DIM_ == 3 ? TZ_ : 1;
  static constexpr int  NT = NT_;
  static constexpr bool EXACT = EXACT_;

  static constexpr int D3 = DIM == 3 ? 1 : 0;
  // Q region: cells [-2, T+2)
  static constexpr int QX = TX + 4, QY = TY + 4, QZ = TZ + 4 * D3;
  static constexpr int NQ = QX * QY * QZ;
  // faces (value at t^n): x faces [-2, TX+2], cells [-2, T+2) transverse; 2D Bz is cell-centred
  static constexpr int NFBX = (TX + 5) * QY * QZ;
  static constexpr int NFBY = QX * (TY + 5) * QZ;
  static constexpr int NFBZ = QX * QY * (D3 ? TZ + 5 : 1);
  // S region: cells [-1, T+1) (slopes, predictor, sFaceMag)
  static constexpr int SX = TX + 2, SY = TY + 2, SZ = TZ + 2 * D3;
  static constexpr int NS = SX * SY * SZ;
  static constexpr int NDIR = DIM;
  static constexpr int NSF = DIM == 3 ? 3 : 2;
  // E region: edges [-1, T+2)
  static constexpr int EX = TX + 3, EY = TY + 3, EZ = D3 ? TZ + 3 : 1;
  static constexpr int NE = EX * EY * EZ;
  static constexpr int NECOMP = DIM == 3 ? 3 : 1;
  // EMF region: edges [0, T]
  static constexpr int MX = TX + 1, MY = TY + 1, MZ = D3 ? TZ + 1 : 1;
  static constexpr int NM = MX * MY * MZ;
  // flux buffer (one direction at a time)
  static constexpr int NF_X = (TX + 1) * TY * TZ;
  static constexpr int NF_Y = TX * (TY + 1) * TZ;
  static constexpr int NF_Z = TX * TY * (TZ + 1);
  static constexpr int NF = NF_X > NF_Y ? (NF_X > NF_Z ? NF_X : NF_Z) : (NF_Y > NF_Z ? NF_Y : NF_Z);
  static constexpr int NFV = DIM == 3 ? 5 : 6; // flux vars used by the update (2D adds Bz)
  // vars per face of the coarse/fine flux side buffer: the NFV hydro fluxes, then the viscous fluxes
  // of E, rho u, rho v, rho w
  static constexpr int NFS = NFV + (VISC ? 4 : 0);

  // fluxes of all directions (one list: x faces, then y, then z)
  static constexpr int NFT = NF_X + NF_Y + (DIM == 3 ? NF_Z : 0);
  // updated face B on [0, T] along each normal (for the fused CFL)
  static constexpr int NB2X = (TX + 1) * TY * TZ;
  static constexpr int NB2Y = TX * (TY + 1) * TZ;
  static constexpr int NB2Z = DIM == 3 ? TX * TY * (TZ + 1) : 0;
  static constexpr int NB2 = NB2X + NB2Y + NB2Z;
  // edges of the tile per direction (z edges are the only ones in 2D)
  static constexpr int NEZ = (TX + 1) * (TY + 1) * TZ;
  static constexpr int NEY = DIM == 3 ? (TX + 1) * TY * (TZ + 1) : 0;
  static constexpr int NEX = DIM == 3 ? TX * (TY + 1) * (TZ + 1) : 0;
  static constexpr int NEDGE = NEZ + NEY + NEX;
  static constexpr int RPD = (int)(sizeof(double) / sizeof(R)); // R slots per double

  // shared-memory carve-up, in units of R. The union U1 holds the primitives at t^n and the edge
  // electric field (phases 1-4), then the FP64 EMFs, the face fluxes and the updated faces.
  static constexpr int OFF_FBX = 0;
  static constexpr int OFF_FBY = OFF_FBX + NFBX;
  static constexpr int OFF_FBZ = OFF_FBY + NFBY;
  static constexpr int OFF_SL = OFF_FBZ + NFBZ;
  static constexpr int OFF_Q2 = OFF_SL + NDIR * 8 * NS;
  static constexpr int OFF_SF = OFF_Q2 + 8 * NS;
  // t^n velocities (DIM components) of cells [-1, T] for the viscous fluxes, outside the union below
  static constexpr int VX = TX + 2, VY = TY + 2, VZ = D3 ? TZ + 2 : 1;
  static constexpr int NVEL = VISC ? VX * VY * VZ : 0;
  static constexpr int OFF_VEL = OFF_SF + NSF * NS;
  static constexpr int OFF_U1 = ((OFF_VEL + DIM * NVEL + 1) / 2) * 2; // 8-byte aligned
  static constexpr int U1_EARLY = 5 * NQ + NECOMP * NE;
  static constexpr int OFF_E = OFF_U1 + 5 * NQ;
  static constexpr int OFF_EMFD = OFF_U1;
  static constexpr int OFF_FL = OFF_EMFD + RPD * NECOMP * NM;
  static constexpr int OFF_B2 = OFF_FL + NFV * NFT;
  static constexpr int U1_LATE = RPD * NECOMP * NM + NFV * NFT + NB2;
  static constexpr int TOTAL = OFF_U1 + (U1_EARLY > U1_LATE ? U1_EARLY : U1_LATE);

  // Persistent, software-pipelined variant (mixed precision, 3D, conforming or coarse/fine meshes, with
  // or without viscosity; the FP64 path gains nothing from it, being bound by its FP64 pipe, and the 2D
  // kernels, whose four CTAs per SM already overlap one another's gathers, run 6 % slower with it: both
  // keep one tile per CTA): one CTA per SM loops over tiles (all tiles of the owned blocks, or a pass's tile
  // list); after phase 5 of a tile it stages the next tile's FP64 gather (face B and U of the Q region,
  // in the layout of fbx|fby|fbz and of the primitives) into [OFF_SL, OFF_VEL) with cp.async, and those
  // copies land while phases 6-7 run. The area ends before the viscous variants' t^n velocities, which
  // phase 7 still reads.
  static constexpr int  NFB = NFBX + NFBY + NFBZ;
  static constexpr int  STAGE_DOUBLES = NFB + 5 * NQ;
  static constexpr bool PIPE = !EXACT && DIM == 3 && NFBX % 2 == 0 && NFBY % 2 == 0 && NFBZ % 2 == 0 &&
                               NQ % 2 == 0 && (OFF_SL * sizeof(R)) % 16 == 0 &&
                               (size_t)STAGE_DOUBLES * 8 <= (size_t)(OFF_VEL - OFF_SL) * sizeof(R);
  // after the tile arrays: neighbour tables and region kinds, [32] each, two of each with PIPE
  static constexpr int    NBR_INTS = (PIPE ? 2 : 1) * 32 * (AMR ? 2 : 1) < 64 ? 64 : (PIPE ? 2 : 1) * 32 * (AMR ? 2 : 1);
  static constexpr size_t SMEM_BYTES = sizeof(R) * (size_t)TOTAL + NBR_INTS * sizeof(int);

  static constexpr int NCELL = TX * TY * TZ;
  static constexpr int CPT = (NCELL + NT - 1) / NT;

  __device__ static int qi(int i, int j, int k) { return (i + 2) + QX * ((j + 2) + QY * (k + 2 * D3)); }
  __device__ static int fxi(int i, int j, int k) { return (i + 2) + (TX + 5) * ((j + 2) + QY * (k + 2 * D3)); }
  __device__ static int fyi(int i, int j, int k) { return (i + 2) + QX * ((j + 2) + (TY + 5) * (k + 2 * D3)); }
  __device__ static int fzi(int i, int j, int k) { return (i + 2) + QX * ((j + 2) + QY * (k + 2 * D3)); }
  __device__ static int si(int i, int j, int k) { return (i + 1) + SX * ((j + 1) + SY * (k + D3)); }
  __device__ static int ei(int i, int j, int k) { return (i + 1) + EX * ((j + 1) + EY * (k + D3)); }
  __device__ static int mi(int i, int j, int k) { return i + MX * (j + MY * k); }
  __device__ static int vi(int i, int j, int k) { return (i + 1) + VX * ((j + 1) + VY * (k + D3)); }
};

// Viscous flux (times dt/dx) at the left face along dir of tile cell (i, j, k), from the t^n
// velocities of cells [-1, T] (ComputeViscousFluxesAndStoreFunctor.cpp:168-344): the velocity
// gradient is a backward difference from the cell (across the face along dir, inside the cell's row
// along the others); out = E, rho u, rho v, rho w (rho and B fluxes are zero).
template <class C>
__device__ __forceinline__ void
viscous_face_flux(const typename C::R * vel, int dir, int i, int j, int k, typename C::R mu, typename C::R dx,
                  typename C::R dtdx, typename C::R * out)
{
  using R = typename C::R;
  constexpr int NC = C::DIM;
  R             v[3], g[3][3];
  const int     c0 = C::vi(i, j, k);
  const int     cx = C::vi(i - 1, j, k), cy = C::vi(i, j - 1, k), cz = C::D3 ? C::vi(i, j, k - 1) : c0;
#pragma unroll
  for (int c = 0; c < NC; ++c)
  {
    const R * V = vel + c * C::NVEL;
    const R   qr = V[c0];
    v[c] = qr;
    g[c][0] = (qr - V[cx]) / dx;
    g[c][1] = (qr - V[cy]) / dx;
    if constexpr (C::DIM == 3)
      g[c][2] = (qr - V[cz]) / dx;
  }
  R fu, fv, fw = R(0), fe;
  if constexpr (C::DIM == 2)
  {
    const R div = g[0][0] + g[1][1];
    const R txy = mu * (g[1][0] + g[0][1]);
    if (dir == 0)
    {
      const R txx = R(2) * mu * (g[0][0] - R(0.5) * div);
      fu = -txx;
      fv = -txy;
      fe = -v[0] * txx - v[1] * txy;
    }
    else
    {
      const R tyy = R(2) * mu * (g[1][1] - R(0.5) * div);
      fu = -txy;
      fv = -tyy;
      fe = -v[0] * txy - v[1] * tyy;
    }
  }
  else
  {
    const R third = R(1.0 / 3.0);
    const R div = g[0][0] + g[1][1] + g[2][2];
    R       t0, t1, t2;
    if (dir == 0)
    {
      t0 = R(2) * mu * (g[0][0] - third * div);
      t1 = mu * (g[1][0] + g[0][1]);
      t2 = mu * (g[2][0] + g[0][2]);
    }
    else if (dir == 1)
    {
      t0 = mu * (g[0][1] + g[1][0]);
      t1 = R(2) * mu * (g[1][1] - third * div);
      t2 = mu * (g[2][1] + g[1][2]);
    }
    else
    {
      t0 = mu * (g[0][2] + g[2][0]);
      t1 = mu * (g[1][2] + g[2][1]);
      t2 = R(2) * mu * (g[2][2] - third * div);
    }
    fu = -t0;
    fv = -t1;
    fw = -t2;
    fe = -v[0] * t0 - v[1] * t1 - v[2] * t2;
  }
  out[0] = fe * dtdx;
  out[1] = fu * dtdx;
  out[2] = fv * dtdx;
  out[3] = fw * dtdx;
}

// Sum over the 2^(d-1) fine faces covering coarse face (g1, g2) of this block's border face toward
// neighbour slot `slot` (direction d, side), of flux side variable `var`, divided by 2^d
// (ReadFluxesAndConservativeUpdateFunctor.h:233-270). The fine blocks stored them in pass 1.
template <class C>
__device__ double
fine_face_flux(const StepArgs & a, int blk, int slot, int d, int side, int g1, int g2, int var)
{
  const int bs[3] = {a.bx, a.by, a.bz};
  const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
  const int ff = 2 * d + (side < 0 ? 1 : 0); // the fine block's face toward this block
  double    acc = 0.0;
  for (int e2 = 0; e2 < (C::DIM == 3 ? 2 : 1); ++e2)
    for (int e1 = 0; e1 < 2; ++e1)
    {
      int ch[3] = {0, 0, 0};
      ch[d] = side < 0 ? 1 : 0;
      int F1 = 2 * g1 + e1;
      ch[t1] = F1 >= bs[t1] ? 1 : 0;
      F1 -= ch[t1] * bs[t1];
      int F2 = 0;
      if (C::DIM == 3)
      {
        F2 = 2 * g2 + e2;
        ch[t2] = F2 >= bs[t2] ? 1 : 0;
        F2 -= ch[t2] * bs[t2];
      }
      const int id = a.fine[((int64_t)blk * 27 + slot) * 8 + ch[0] + 2 * ch[1] + 4 * ch[2]];
      const int cs = id >= 0 ? a.flux_slot[id] : -1;
      if (cs >= 0)
        acc += a.flux_side[(((int64_t)cs * 2 * C::DIM + ff) * C::NFS + var) * a.flux_face_stride + F1 +
                           (int64_t)bs[t1] * F2];
    }
  return acc / (double)(1 << C::DIM);
}

// Asynchronous global -> shared copies (cp.async, sm_80+): 8 bytes through L1, 16 bytes bypassing it.
__device__ __forceinline__ void
cp_async8(void * smem_dst, const void * gmem_src)
{
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void
cp_async16(void * smem_dst, const void * gmem_src)
{
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void
cp_async_commit()
{
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void
cp_async_wait_all()
{
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

__device__ __forceinline__ int
nb_slot(int ox, int oy, int oz)
{
  return (oz + 1) * 9 + (oy + 1) * 3 + (ox + 1);
}

__device__ __forceinline__ unsigned long long
atomic_max_pos_double(unsigned long long * addr, double v)
{
  // positive doubles order like their bit patterns
  return atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// ---- phase-5 work: per-direction passes with compile-time strides ------------------------------
// Shared-memory views of one tile, passed to the passes below.
template <class C>
struct TileView
{
  using R = typename C::R;
  const R *   fb[3]; // face B at t^n, components x, y, z (2D z: cell-centred Bz)
  const R *   sl;    // slopes [dir][var][S cell]
  const R *   q2;    // predictor [var][S cell]
  const R *   sf;    // half-step face-B source [comp][S cell]
  double *    emfd;  // EMFs [comp][edge], FP64
  R *         fl;    // fluxes [var][face item]
  const int * s_nbr;
  Phys<R>     ph;
  R           dtdx;
  int         x0, y0, z0, bx, by, bz, n_owned;
  int         rk2;
  // coarse/fine meshes (s_kind null otherwise)
  const int *     s_kind;
  int             blk, pass;
  const int32_t * fine;
  const double *  emf_side;
  const int32_t * emf_slot;
  double *        emf_self; // this block's raw-EMF side slot in pass 1, or null
};

// stride of the S region along direction d
template <class C>
__device__ constexpr int
s_stride(int d)
{
  return d == 0 ? 1 : (d == 1 ? C::SX : C::SX * C::SY);
}
// stride of face array c along direction d
template <class C>
__device__ constexpr int
f_stride(int c, int d)
{
  return d == 0 ? 1
                : (c == 0 ? (d == 1 ? C::TX + 5 : (C::TX + 5) * C::QY)
                          : (c == 1 ? (d == 1 ? C::QX : C::QX * (C::TY + 5)) : (d == 1 ? C::QX : C::QX * C::QY)));
}
template <class C, int CMP>
__device__ __forceinline__ int
f_index(int i, int j, int k)
{
  return CMP == 0 ? C::fxi(i, j, k) : (CMP == 1 ? C::fyi(i, j, k) : C::fzi(i, j, C::D3 ? k : 0));
}

// CorrectEmfAtBlockBorderFunctor::correct_emf (CorrectEmfAtBlockBorderFunctor.cpp:94-360) of a
// block-border edge on a coarse/fine mesh. Siblings are the regions across the two transverse block
// borders (v0 along D0, v1 along D1) and across both. Same-level copies are this tile's own value
// (every block computes a shared edge from identical ghost data); a finer sibling's edge is the
// fine block's raw EMF from pass 1 (3D: its two sub-edges along the edge). In pass 1 the raw value
// is also stored for coarse neighbours.
template <class C, int CD, int D0, int D1>
__device__ __forceinline__ double
amr_border_emf(const TileView<C> & t, const int * gi, int v0, int v1, typename C::R val)
{
  using R = typename C::R;
  constexpr int COMP = C::DIM == 3 ? CD : 0;
  if (v0 == 0 && v1 == 0)
    return to_d<R>(val);
  const int     sx = t.bx + 1, sy = t.by + 1;
  const int64_t ne = (int64_t)sx * sy * (C::DIM == 3 ? t.bz + 1 : 1);
  if (t.emf_self)
    t.emf_self[COMP * ne + gi[0] + (int64_t)sx * (gi[1] + (int64_t)sy * gi[2])] = to_d<R>(val);
  int kd[3], sl[3], so[3][3];
#pragma unroll
  for (int n = 0; n < 3; ++n)
  {
    so[n][0] = so[n][1] = so[n][2] = 0;
    if (n == 0 || n == 2)
      so[n][D0] = v0;
    if (n == 1 || n == 2)
      so[n][D1] = v1;
    const bool exists = (n == 0 && v0 != 0) || (n == 1 && v1 != 0) || (n == 2 && v0 != 0 && v1 != 0);
    sl[n] = nb_slot(so[n][0], so[n][1], so[n][2]);
    kd[n] = exists ? t.s_kind[sl[n]] : (int)RK_MISSING;
  }
  bool coarser = false, finer = false, all_same = true;
#pragma unroll
  for (int n = 0; n < 3; ++n)
  {
    const bool valid = kd[n] != RK_MISSING;
    coarser = coarser || (valid && kd[n] == RK_COARSER);
    finer = finer || (valid && kd[n] == RK_FINER);
    all_same = all_same && valid && kd[n] != RK_COARSER && kd[n] != RK_FINER;
  }
  double out = to_d<R>(val);
  // The averages of copies of the same value: the FP64 path takes them as the reference does, in its
  // order: ((0 + v) + v + v) / 3 can differ from v by one ulp). On the mixed path v is an FP32 value, so
  // k v (k <= 4) is exact in FP64 and the FP64 average is v itself: the value is kept as it is, with no
  // FP64 division, and a fine block's corrected edge equals the raw value its coarse neighbour reads back.
  if (coarser)
  {
    if constexpr (C::EXACT)
    {
      double acc = to_d<R>(val);
      int    count = 1;
#pragma unroll
      for (int n = 0; n < 3; ++n)
        if (kd[n] == RK_SAME)
        {
          acc += to_d<R>(val);
          ++count;
        }
      out = acc / (double)count;
    }
  }
  else if (finer)
  {
    const int bs[3] = {t.bx, t.by, t.bz};
    double    acc = 0.0;
    int       count = 0;
#pragma unroll
    for (int n = 0; n < 3; ++n)
    {
      if (kd[n] != RK_FINER)
        continue;
      int F[3] = {0, 0, 0}, ch[3] = {0, 0, 0};
#pragma unroll
      for (int d = 0; d < C::DIM; ++d)
      {
        if (so[n][d] != 0)
        {
          ch[d] = so[n][d] < 0 ? 1 : 0;
          F[d] = so[n][d] < 0 ? bs[d] : 0;
        }
        else
        {
          const int x = 2 * gi[d];
          ch[d] = x >= bs[d] ? 1 : 0;
          F[d] = x - ch[d] * bs[d];
        }
      }
      const int id = t.fine[((int64_t)t.blk * 27 + sl[n]) * 8 + ch[0] + 2 * ch[1] + 4 * ch[2]];
      const int cs = id >= 0 ? t.emf_slot[id] : -1;
      if (cs < 0)
        continue;
      const double * E = t.emf_side + ((int64_t)cs * C::NECOMP + COMP) * ne;
      const int64_t  e = F[0] + (int64_t)sx * (F[1] + (int64_t)sy * F[2]);
      acc += E[e];
      if constexpr (C::DIM == 3)
        acc += E[e + (CD == 0 ? 1 : (CD == 1 ? (int64_t)sx : (int64_t)sx * sy))];
      ++count;
    }
    out = acc / (double)count / (double)(1 << (C::DIM - 1));
  }
  if (all_same && C::EXACT)
  {
    double acc = 0.0;
    int    count = 1;
    acc += to_d<R>(val);
#pragma unroll
    for (int n = 0; n < 3; ++n)
      if (kd[n] != RK_OUTSIDE)
      {
        acc += to_d<R>(val);
        ++count;
      }
    out = acc / (double)count;
  }
  return out;
}

// Face fluxes on the tile's block-border faces of a coarse/fine mesh
// (ReadFluxesAndConservativeUpdateFunctor.cpp:141-172, .h:233-270): pass 1 stores the fluxes of
// faces whose neighbour is coarser; pass 2 replaces the flux of faces whose neighbour is finer by
// the sum of the 2^(d-1) fine fluxes (first transverse axis fastest) / 2^d.
template <class C>
__device__ __forceinline__ void
amr_border_fluxes(const StepArgs & a, typename C::R * fl, const int * s_kind, int blk, int x0, int y0, int z0, int tid,
                  const typename C::R * vel, typename C::R dx, typename C::R dtdx)
{
  using R = typename C::R;
  const int bs[3] = {a.bx, a.by, a.bz};
  const int org[3] = {x0, y0, z0};
  const int T[3] = {C::TX, C::TY, C::TZ};
  const int my_slot = a.pass == 1 ? a.flux_slot[blk] : -1;
  for (int f = 0; f < 2 * C::DIM; ++f)
  {
    const int d = f >> 1, side = (f & 1) ? 1 : -1;
    if (side < 0 ? org[d] != 0 : org[d] + T[d] != bs[d])
      continue;
    int o[3] = {0, 0, 0};
    o[d] = side;
    const int  slot = nb_slot(o[0], o[1], o[2]);
    const int  kd = s_kind[slot];
    const bool write = a.pass == 1 && kd == RK_COARSER && my_slot >= 0;
    const bool read = a.pass == 2 && kd == RK_FINER;
    if (!write && !read)
      continue;
    const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
    const int n1 = T[t1], n2 = C::DIM == 3 ? T[t2] : 1;
    const int off = d == 0 ? 0 : (d == 1 ? C::NF_X : C::NF_X + C::NF_Y);
    const int nxd = C::TX + (d == 0), nyd = C::TY + (d == 1);
    // pass 1 stores the hydro and viscous fluxes; pass 2 replaces the hydro fluxes here (the viscous
    // ones are read in the update)
    const int nvar = write ? C::NFS : C::NFV;
    for (int m = tid; m < n1 * n2 * nvar; m += C::NT)
    {
      const int v = m / (n1 * n2), r = m - v * (n1 * n2);
      const int u1 = r % n1, u2 = r / n1;
      int       li[3] = {0, 0, 0};
      li[d] = side < 0 ? 0 : T[d];
      li[t1] = u1;
      if (C::DIM == 3)
        li[t2] = u2;
      const int idx = off + li[0] + nxd * (li[1] + nyd * li[2]);
      const int g1 = org[t1] + u1, g2 = C::DIM == 3 ? org[t2] + u2 : 0;
      if (write)
      {
        double val;
        if (v < C::NFV)
          val = to_d<R>(fl[v * C::NFT + idx]);
        else
        {
          R fv[4];
          viscous_face_flux<C>(vel, d, li[0], li[1], li[2], (R)a.src.mu, dx, dtdx, fv);
          val = to_d<R>(fv[v - C::NFV]);
        }
        a.flux_side[(((int64_t)my_slot * 2 * C::DIM + f) * C::NFS + v) * a.flux_face_stride + g1 + (int64_t)bs[t1] * g2] =
          val;
        continue;
      }
      fl[v * C::NFT + idx] = to_r<R>(fine_face_flux<C>(a, blk, slot, d, side, g1, g2, v));
    }
  }
}

// Corner positions of the 4 cells around an edge (the cell itself is LB).
enum : int
{
  LOC_LB = 0,
  LOC_RT = 1,
  LOC_RB = 2,
  LOC_LT = 3
};

// reconstruct_state_{2d,3d}_at_edge (scheme/ComputeEmfAndStoreFunctor.cpp:103-367) of the cell at
// S index sc, whose own faces are fb0 (array D0) and fb1 (array D1); LOC selects which edge of the
// cell. Signs and shifts follow the reference's table of LB/RT/RB/LT.
template <class C, int D0, int D1, int LOC>
__device__ __forceinline__ void
recon_edge(const TileView<C> & t, int sc, int fb0, int fb1, typename C::R * q)
{
  using R = typename C::R;
  constexpr bool sh0 = LOC == LOC_RT || LOC == LOC_RB;
  constexpr bool sh1 = LOC == LOC_RT || LOC == LOC_LT;
  constexpr int  sd0 = (LOC == LOC_RT || LOC == LOC_RB) ? 1 : -1;
  constexpr int  sd1 = (LOC == LOC_RT || LOC == LOC_LT) ? 1 : -1;
  constexpr int  sb0 = (LOC == LOC_RT || LOC == LOC_LT) ? 1 : -1;
  constexpr int  sb1 = (LOC == LOC_RT || LOC == LOC_RB) ? 1 : -1;
  constexpr int  NS = C::NS;
#pragma unroll
  for (int v = 0; v < 8; ++v)
    q[v] = t.q2[v * NS + sc];
  const int f0 = fb0 + (sh0 ? f_stride<C>(D0, D0) : 0);
  const int f1 = fb1 + (sh1 ? f_stride<C>(D1, D1) : 0);
  const R * F0 = t.fb[D0];
  const R * F1 = t.fb[D1];
  R         B0 = F0[f0];
  R         B1 = F1[f1];
  if (!t.rk2) // the half-step face source only with HANCOCK (ComputeEmfAndStoreFunctor.cpp:189-193, 297-301)
  {
    B0 += t.sf[D0 * NS + sc + (sh0 ? s_stride<C>(D0) : 0)];
    B1 += t.sf[D1 * NS + sc + (sh1 ? s_stride<C>(D1) : 0)];
  }
  const R   dB0d1 = slope1<R>(F0[f0], F0[f0 + f_stride<C>(D0, D1)], F0[f0 - f_stride<C>(D0, D1)], t.ph.slope_type);
  const R   dB1d0 = slope1<R>(F1[f1], F1[f1 + f_stride<C>(D1, D0)], F1[f1 - f_stride<C>(D1, D0)], t.ph.slope_type);
  const R * S0 = t.sl + D0 * 8 * NS + sc;
  const R * S1 = t.sl + D1 * 8 * NS + sc;
  const R   g0 = (R)sd0, g1 = (R)sd1;
  auto      h = [&](int v) { return R(0.5) * (g0 * S0[v * NS] + g1 * S1[v * NS]); };
#pragma unroll
  for (int v = 0; v < 5; ++v)
    q[v] += h(v);
  if constexpr (C::DIM == 2)
  {
    q[IA] = B0 + R(0.5) * ((R)sb0 * dB0d1);
    q[IB] = B1 + R(0.5) * ((R)sb1 * dB1d0);
    q[IC] += h(IC);
  }
  else
  {
    // the reference's branch order for IA / IB / IC (ComputeEmfAndStoreFunctor.cpp:324-363)
    if constexpr (D0 == 0)
      q[IA] = B0 + R(0.5) * ((R)sb0 * dB0d1);
    else
      q[IA] += h(IA);
    if constexpr (D0 == 1)
      q[IB] = B0 + R(0.5) * ((R)sb0 * dB0d1);
    else
      q[IB] += h(IB);
    if constexpr (D1 == 1)
      q[IB] = B1 + R(0.5) * ((R)sb1 * dB1d0);
    else
      q[IB] += h(IB);
    if constexpr (D1 == 2)
      q[IC] = B1 + R(0.5) * ((R)sb1 * dB1d0);
    else
      q[IC] += h(IC);
  }
  q[ID] = rmax<R>(t.ph.smallr, q[ID]);
  q[IP] = rmax<R>(t.ph.smallp * q[ID], q[IP]);
}

// EMFs along direction CD on the tile's edges [0, T] (ComputeEmfAndStoreFunctor.cpp:371-590), with
// the border averaging of CorrectEmfAtBlockBorderFunctor (uniform level, .cpp:298-356)
// Face increment of the CT update from two EMF differences: the reference's "d = 0; d += a; d -= b"
// (ReadEmfAndUpdateFunctor.cpp:118-161) on the FP64 path; a - b on the mixed path, the same value
// up to the sign of a zero, one FP64 instruction less per face.
template <bool EXACT>
__device__ __forceinline__ double
curl2(double a, double b)
{
  if constexpr (EXACT)
  {
    double d = 0;
    d += a;
    d -= b;
    return d;
  }
  else
    return a - b;
}

// Items of the phase-5 passes are dealt round-robin to the threads, each pass starting where the
// previous one stopped (START = items dealt before, mod NT), so that no thread gets the remainder
// of every pass.
template <class C>
__device__ __forceinline__ int
first_item(int tid, int start)
{
  const int m0 = tid - start;
  return m0 < 0 ? m0 + C::NT : m0;
}
template <class C, int CD>
__device__ constexpr int
edge_count()
{
  return (CD == 0 ? C::TX : C::TX + 1) * (CD == 1 ? C::TY : C::TY + 1) * (C::DIM == 3 ? (CD == 2 ? C::TZ : C::TZ + 1) : 1);
}
template <class C, int D>
__device__ constexpr int
face_count()
{
  return (C::TX + (D == 0)) * (C::TY + (D == 1)) * (C::TZ + (D == 2 && C::D3));
}

template <class C, int CD, int START>
__device__ __forceinline__ void
edge_pass(const TileView<C> & t, int tid)
{
  using R = typename C::R;
  constexpr int D0 = CD == 0 ? 1 : 0;
  constexpr int D1 = CD == 2 ? 1 : 2;
  constexpr int NX = CD == 0 ? C::TX : C::TX + 1;
  constexpr int NY = CD == 1 ? C::TY : C::TY + 1;
  constexpr int NZ = C::DIM == 3 ? (CD == 2 ? C::TZ : C::TZ + 1) : 1;
  constexpr int s0 = s_stride<C>(D0), s1 = s_stride<C>(D1);
  constexpr int f00 = f_stride<C>(D0, D0), f01 = f_stride<C>(D0, D1);
  constexpr int f10 = f_stride<C>(D1, D0), f11 = f_stride<C>(D1, D1);
  for (int m = first_item<C>(tid, START); m < NX * NY * NZ; m += C::NT)
  {
    const int i = m % NX, j = (m / NX) % NY, k = m / (NX * NY);
    const int sc = C::si(i, j, k);
    const int g0 = f_index<C, D0>(i, j, k);
    const int g1 = f_index<C, D1>(i, j, k);
    R         qe[4][8];
    recon_edge<C, D0, D1, LOC_LB>(t, sc, g0, g1, qe[ELB]);
    recon_edge<C, D0, D1, LOC_RT>(t, sc - s0 - s1, g0 - f00 - f01, g1 - f10 - f11, qe[ERT]);
    // y edges: the reference swaps the RB and LT states (ComputeEmfAndStoreFunctor.cpp:551-560)
    recon_edge<C, D0, D1, LOC_RB>(t, sc - s0, g0 - f00, g1 - f10, qe[CD == 1 ? ELT : ERB]);
    recon_edge<C, D0, D1, LOC_LT>(t, sc - s1, g0 - f01, g1 - f11, qe[CD == 1 ? ERB : ELT]);
    R      val = edge_emf<R, CD>(qe, t.ph) * t.dtdx;
    double out;
    // an edge on a line where four blocks meet is averaged with its sibling copies (self first,
    // then the non-outside siblings); on a conforming mesh the copies are computed from identical
    // data, so the sum is of equal terms
    {
      const int gi[3] = {t.x0 + i, t.y0 + j, t.z0 + k};
      const int bs[3] = {t.bx, t.by, t.bz};
      const int v0 = gi[D0] == 0 ? -1 : (gi[D0] == bs[D0] ? 1 : 0);
      const int v1 = (C::DIM == 2 && D1 == 2) ? 0 : (gi[D1] == 0 ? -1 : (gi[D1] == bs[D1] ? 1 : 0));
      if constexpr (C::AMR)
        out = amr_border_emf<C, CD, D0, D1>(t, gi, v0, v1, val);
      else if (v0 != 0 && v1 != 0)
      {
        const int sl0 = nb_slot(D0 == 0 ? v0 : 0, D0 == 1 ? v0 : 0, 0);
        const int sl1 = nb_slot(D1 == 0 ? v1 : 0, D1 == 1 ? v1 : 0, D1 == 2 ? v1 : 0);
        const int sl2 = nb_slot(D0 == 0 ? v0 : (D1 == 0 ? v1 : 0), D0 == 1 ? v0 : (D1 == 1 ? v1 : 0), D1 == 2 ? v1 : 0);
        const int n0 = t.s_nbr[sl0], n1 = t.s_nbr[sl1], n2 = t.s_nbr[sl2];
        if (n0 >= 0 && n1 >= 0 && n2 >= 0)
        {
          R   acc = R(0);
          int count = 1;
          acc += val;
          if (n0 < t.n_owned)
          {
            acc += val;
            count++;
          }
          if (n1 < t.n_owned)
          {
            acc += val;
            count++;
          }
          if (n2 < t.n_owned)
          {
            acc += val;
            count++;
          }
          val = acc / (R)count;
        }
      }
      if constexpr (!C::AMR)
        out = to_d<R>(val);
    }
    t.emfd[(C::DIM == 3 ? CD : 0) * C::NM + C::mi(i, j, k)] = out;
  }
}

// Fluxes through the tile's faces normal to D (ComputeHydroFluxesAndStoreFunctor.cpp:335-503):
// left state from cell i-1, right state from cell i, normal B = face value + sFaceMag.
template <class C, int D, int START>
__device__ __forceinline__ void
flux_pass(const TileView<C> & t, int tid)
{
  using R = typename C::R;
  constexpr int NX = C::TX + (D == 0), NY = C::TY + (D == 1), NZ = C::TZ + (D == 2 && C::D3);
  constexpr int OFF = D == 0 ? 0 : (D == 1 ? C::NF_X : C::NF_X + C::NF_Y);
  constexpr int ivel = D == 0 ? IU : (D == 1 ? IV : IW);
  constexpr int imag = D == 0 ? IA : (D == 1 ? IB : IC);
  constexpr int NS = C::NS;
  const R *     S = t.sl + D * 8 * NS;
  for (int m = first_item<C>(tid, START); m < NX * NY * NZ; m += C::NT)
  {
    const int i = m % NX, j = (m / NX) % NY, k = m / (NX * NY);
    const int snR = C::si(i, j, k);
    const int snL = snR - s_stride<C>(D);
    R         qL[8], qR[8], flux[8];
#pragma unroll
    for (int v = 0; v < 8; ++v)
    {
      qL[v] = t.q2[v * NS + snL] + R(0.5) * S[v * NS + snL];
      qR[v] = t.q2[v * NS + snR] + R(-0.5) * S[v * NS + snR];
    }
    qL[ID] = rmax<R>(t.ph.smallr, qL[ID]);
    qL[IP] = rmax<R>(t.ph.smallp * qL[ID], qL[IP]);
    qR[ID] = rmax<R>(t.ph.smallr, qR[ID]);
    qR[IP] = rmax<R>(t.ph.smallp * qR[ID], qR[IP]);
    const R bn = t.fb[D][f_index<C, D>(i, j, k)] + t.sf[D * NS + snR];
    qR[imag] = bn;
    qL[imag] = bn;
    if constexpr (D != 0)
    {
      R tmp;
      tmp = qL[IU]; qL[IU] = qL[ivel]; qL[ivel] = tmp;
      tmp = qR[IU]; qR[IU] = qR[ivel]; qR[ivel] = tmp;
      tmp = qL[IA]; qL[IA] = qL[imag]; qL[imag] = tmp;
      tmp = qR[IA]; qR[IA] = qR[imag]; qR[imag] = tmp;
    }
    riemann_mhd<R>(qL, qR, flux, t.ph);
    if constexpr (D != 0)
    {
      R tmp;
      tmp = flux[IU]; flux[IU] = flux[ivel]; flux[ivel] = tmp;
      tmp = flux[IA]; flux[IA] = flux[imag]; flux[imag] = tmp;
    }
#pragma unroll
    for (int v = 0; v < 5; ++v)
      t.fl[v * C::NFT + OFF + m] = flux[v] * t.dtdx;
    if constexpr (C::DIM == 2)
      t.fl[5 * C::NFT + OFF + m] = flux[IC] * t.dtdx;
  }
}

template <class C>
__global__ void __launch_bounds__(C::NT, C::MINB) fused_step_kernel(const StepArgs a)
{
  using R = typename C::R;
  constexpr int DIM = C::DIM, TX = C::TX, TY = C::TY, TZ = C::TZ, NT = C::NT, D3 = C::D3;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  R *   sm = reinterpret_cast<R *>(smem_raw);
  R *   fbx = sm + C::OFF_FBX;
  R *   fby = sm + C::OFF_FBY;
  R *   fbz = sm + C::OFF_FBZ;
  R *   sl = sm + C::OFF_SL;
  R *   q2 = sm + C::OFF_Q2;
  R *   sf = sm + C::OFF_SF;
  R *      ee = sm + C::OFF_E;
  R *      qh = sm + C::OFF_U1;
  double * emfd = reinterpret_cast<double *>(sm + C::OFF_EMFD); // FP64 EMFs for the CT curl
  R *      fl = sm + C::OFF_FL;
  R *      b2s = sm + C::OFF_B2;
  R *      vel = sm + C::OFF_VEL; // viscous variants: t^n velocities of cells [-1, T]
  // neighbour tables ([32] per staged tile), then region kinds of coarse/fine meshes ([32] per staged tile)
  int * s_nbr0 = reinterpret_cast<int *>(sm + C::TOTAL);
  int * s_kind0 = s_nbr0 + (C::PIPE ? 64 : 32);
  __shared__ double       s_red[NT / 32];
  __shared__ unsigned int s_health;
  __shared__ unsigned int s_stage_health[2]; // PIPE: missing / level-jump flags of a staged tile
  __shared__ unsigned int s_stage_jump[2];   // PIPE: neighbour slots at another level

  const int tid = threadIdx.x;
  const int tiles_per_block = a.tiles_x * a.tiles_y * a.tiles_z;
  const int bx = a.bx, by = a.by, bz = a.bz;
  auto cell_off = [](int c, int n) { return c < 0 ? -1 : (c >= n ? 1 : 0); };
  auto face_off = [](int f, int n) { return f < 0 ? -1 : (f > n ? 1 : 0); };

  // ---- PIPE: staging of a tile's gather ----------------------------------------------------------
  double *  stage = reinterpret_cast<double *>(sm + C::OFF_SL);
  // work items: a tile list (the coarse/fine passes, the chunks of the host-buffer step), the tiles of a
  // block list, or all tiles of the owned blocks
  const int n_work =
    C::PIPE ? (a.tile_list ? a.n_list : (a.blk_list ? a.blk_count : a.n_owned) * tiles_per_block) : 0;
  // tile of work item w (a coarse/fine pass's list entry ~tile marks a side-data-only tile)
  auto tile_at = [&](int w) {
    if (a.tile_list)
      return (int)a.tile_list[w];
    if (a.blk_list)
      return a.blk_list[w / tiles_per_block] * tiles_per_block + w % tiles_per_block;
    return w;
  };
  // neighbour table (and region kinds) of work item w into buffer buf (warp 0), with the slots whose
  // block is at another level
  auto load_nbr = [&](int w, int buf) {
    if (tid < 32)
    {
      int tl = tile_at(w);
      if (tl < 0)
        tl = ~tl;
      const int b = tl / tiles_per_block;
      int       nb = -1;
      bool      jump = false;
      if (tid < 27)
      {
        nb = a.neighbor[(int64_t)b * 27 + tid];
        jump = nb >= 0 && nb < a.n_blocks && a.level[nb] != a.level[b];
        s_nbr0[32 * buf + tid] = nb;
        if constexpr (C::AMR)
          s_kind0[32 * buf + tid] = (int)a.kind[(int64_t)b * 27 + tid];
      }
      const unsigned m = __ballot_sync(0xffffffffu, jump);
      if (tid == 0)
      {
        s_stage_jump[buf] = m;
        s_stage_health[buf] = 0u;
      }
    }
  };
  // issue the cp.async copies of tile w's face B and U (Q region) into the staging area; absent
  // neighbours give 0 (faces) and rho = E = 1, momenta 0 (as the direct gather)
  auto stage_tile = [&](int w, int buf) {
    int tl = tile_at(w);
    if (tl < 0)
      tl = ~tl;
    const int   b = tl / tiles_per_block;
    int         t = tl - b * tiles_per_block;
    const int   sx0 = (t % a.tiles_x) * TX;
    t /= a.tiles_x;
    const int   sy0 = (t % a.tiles_y) * TY, sz0 = (t / a.tiles_y) * TZ;
    const int * nbr = s_nbr0 + 32 * buf;
    const int * kinds = s_kind0 + 32 * buf;
    const unsigned jm = s_stage_jump[buf];
    unsigned    fl = 0u;
    // face / conservative arrays of a real or virtual (coarse/fine ghost) block
    auto bsrc_s = [&](int nb) -> const double * {
      if constexpr (C::AMR)
        return nb < a.n_blocks ? a.B + (int64_t)nb * a.nface : a.Bv + (int64_t)(nb - a.n_blocks) * a.nface;
      else
        return a.B + (int64_t)nb * a.nface;
    };
    auto usrc_s = [&](int nb) -> const double * {
      if constexpr (C::AMR)
        return nb < a.n_blocks ? a.U + (int64_t)nb * 5 * a.ncell : a.Uv + (int64_t)(nb - a.n_blocks) * 5 * a.ncell;
      else
        return a.U + (int64_t)nb * 5 * a.ncell;
    };
    // the block's own border face shared with a finer face neighbour: that neighbour's (restricted) value
    auto shared_s = [&](int d, int f, int n, int & nb, int & fq) {
      if constexpr (C::AMR)
      {
        if (nb == b && (f == 0 || f == n))
        {
          const int sl = nb_slot(d == 0 ? (f == 0 ? -1 : 1) : 0, d == 1 ? (f == 0 ? -1 : 1) : 0,
                                 d == 2 ? (f == 0 ? -1 : 1) : 0);
          if (kinds[sl] == RK_FINER)
          {
            nb = nbr[sl];
            fq = f == 0 ? n : 0;
          }
        }
      }
    };
    auto        own = [&](int ox, int oy, int oz) -> int {
      if ((ox | oy | oz) == 0)
        return b;
      const int sl = nb_slot(ox, oy, oz);
      const int nb = nbr[sl];
      if (nb < 0)
        fl |= HEALTH_MISSING_NEIGHBOR;
      else if ((jm >> sl) & 1u)
        fl |= HEALTH_LEVEL_JUMP;
      return nb;
    };
    for (int n = tid; n < C::NFBX; n += NT)
    {
      const int i = n % (TX + 5) - 2;
      const int j = (n / (TX + 5)) % C::QY - 2;
      const int k = D3 ? n / ((TX + 5) * C::QY) - 2 : 0;
      const int fi = sx0 + i, cj = sy0 + j, ck = sz0 + k;
      const int ox = face_off(fi, bx), oy = cell_off(cj, by), oz = D3 ? cell_off(ck, bz) : 0;
      int       nb = own(ox, oy, oz);
      int       fq = fi - ox * bx;
      shared_s(0, fi, bx, nb, fq);
      if (nb >= 0)
        cp_async8(stage + n, bsrc_s(nb) + fq + (int64_t)(bx + 1) * ((cj - oy * by) + (int64_t)by * (ck - oz * bz)));
      else
        stage[n] = 0.0;
    }
    for (int m = tid; m < C::NFBY / 2; m += NT)
    {
      const int n = 2 * m;
      const int i = n % C::QX - 2;
      const int j = (n / C::QX) % (TY + 5) - 2;
      const int k = D3 ? n / (C::QX * (TY + 5)) - 2 : 0;
      const int ci = sx0 + i, fj = sy0 + j, ck = sz0 + k;
      const int ox = cell_off(ci, bx), oy = face_off(fj, by), oz = D3 ? cell_off(ck, bz) : 0;
      int       nb = own(ox, oy, oz);
      int       fq = fj - oy * by;
      shared_s(1, fj, by, nb, fq);
      double *  d = stage + C::NFBX + n;
      if (nb >= 0)
        cp_async16(d, bsrc_s(nb) + a.nfx + (ci - ox * bx) + (int64_t)bx * (fq + (int64_t)(by + 1) * (ck - oz * bz)));
      else
        d[0] = d[1] = 0.0;
    }
    for (int m = tid; m < C::NFBZ / 2; m += NT)
    {
      const int n = 2 * m;
      const int i = n % C::QX - 2;
      const int j = (n / C::QX) % C::QY - 2;
      const int k = D3 ? n / (C::QX * C::QY) - 2 : 0;
      const int ci = sx0 + i, cj = sy0 + j, fk = sz0 + k;
      // 3D z faces; 2D: the cell-centred Bz of the same cells
      const int ox = cell_off(ci, bx), oy = cell_off(cj, by), oz = D3 ? face_off(fk, bz) : 0;
      int       nb = own(ox, oy, oz);
      int       fq = fk - oz * bz;
      if (D3)
        shared_s(2, fk, bz, nb, fq);
      double *  d = stage + C::NFBX + C::NFBY + n;
      if (nb >= 0)
        cp_async16(d, bsrc_s(nb) + a.nfx + a.nfy + (ci - ox * bx) + (int64_t)bx * ((cj - oy * by) + (int64_t)by * fq));
      else
        d[0] = d[1] = 0.0;
    }
    for (int m = tid; m < C::NQ / 2; m += NT)
    {
      const int n = 2 * m;
      const int i = n % C::QX - 2;
      const int j = (n / C::QX) % C::QY - 2;
      const int k = D3 ? n / (C::QX * C::QY) - 2 : 0;
      const int ci = sx0 + i, cj = sy0 + j, ck = sz0 + k;
      const int ox = cell_off(ci, bx), oy = cell_off(cj, by), oz = D3 ? cell_off(ck, bz) : 0;
      const int nb = own(ox, oy, oz);
      double *  d = stage + C::NFB + n;
      if (nb >= 0)
      {
        const double * Ub = usrc_s(nb) + (ci - ox * bx) + (int64_t)bx * ((cj - oy * by) + (int64_t)by * (ck - oz * bz));
#pragma unroll
        for (int v = 0; v < 5; ++v)
          cp_async16(d + v * C::NQ, Ub + (int64_t)v * a.ncell);
      }
      else
      {
#pragma unroll
        for (int v = 0; v < 5; ++v)
          d[v * C::NQ] = d[v * C::NQ + 1] = v < 2 ? 1.0 : 0.0;
      }
    }
    cp_async_commit();
    if (fl)
      atomicOr(&s_stage_health[buf], fl);
  };
  if constexpr (C::PIPE)
  {
    if ((int)blockIdx.x < n_work)
    {
      load_nbr(blockIdx.x, 0);
      __syncthreads();
      stage_tile(blockIdx.x, 0);
    }
  }

  // one tile per CTA, or (PIPE) tiles blockIdx.x, blockIdx.x + gridDim.x, ...
  for (int iter = 0, work = blockIdx.x; C::PIPE ? work < n_work : iter == 0; ++iter, work += gridDim.x)
  {
  const int buf = iter & 1;
  const bool has_next = C::PIPE && work + (int)gridDim.x < n_work;
  int *     s_nbr = s_nbr0 + (C::PIPE ? 32 * buf : 0);
  int       tile = tile_at(C::PIPE ? work : (int)blockIdx.x);
  bool      side_only = false; // pass 1 of a tile that also runs in pass 2: side data only
  if (C::AMR && a.tile_list)
  {
    if (!C::PIPE)
      tile = a.tile_list[blockIdx.x];
    if (tile < 0)
    {
      tile = ~tile;
      side_only = true;
    }
  }
  const int blk = tile / tiles_per_block;
  if (blk >= a.n_owned)
    return;
  int       t = tile - blk * tiles_per_block;
  const int tx = t % a.tiles_x;
  t /= a.tiles_x;
  const int ty = t % a.tiles_y;
  const int tz = t / a.tiles_y;
  const int x0 = tx * TX, y0 = ty * TY, z0 = tz * TZ;

  int * s_kind = s_kind0 + (C::PIPE ? 32 * buf : 0);
  if constexpr (C::PIPE)
    cp_async_wait_all(); // this tile's staged gather (issued during the previous tile)
  else
  {
    if (tid < 32)
    {
      // neighbour table, region kinds, and the slots whose (real) block is at another level
      int  nb = -1;
      bool jump = false;
      if (tid < 27)
      {
        nb = a.neighbor[(int64_t)blk * 27 + tid];
        s_nbr[tid] = nb;
        if constexpr (C::AMR)
          s_kind[tid] = (int)a.kind[(int64_t)blk * 27 + tid];
        jump = nb >= 0 && nb < a.n_blocks && a.level[nb] != a.level[blk];
      }
      const unsigned m = __ballot_sync(0xffffffffu, jump);
      if (tid == 0)
      {
        s_stage_jump[0] = m;
        s_health = 0u;
      }
    }
  }
  __syncthreads();
  const unsigned jump_mask = s_stage_jump[C::PIPE ? buf : 0];
  // the staging flags of this tile, read after the barrier: the threads that issued the staging may have
  // gone straight to this tile (skip and side-data-only paths) without one in between
  if constexpr (C::PIPE)
    if (tid == 0)
      s_health = s_stage_health[buf];

  const int myprob = a.problem ? a.problem[blk] : 0;
  const int mylevel = a.level[blk];
  const double dt = a.dt_dev ? a.dt_dev[myprob] : a.dt;
  if ((__double_as_longlong(dt) << 1) == 0) // dt == +-0 (integer test: no FP64 instruction per warp)
  {
    // a problem that has reached its end time: carry the tile over unchanged (dt = +0), or, once an
    // earlier step has done so and both buffers hold the final state, leave it (dt = -0)
    if (__double_as_longlong(dt) == 0)
    {
      for (int n = tid; n < C::NCELL; n += NT)
      {
        const int     i = n % TX, j = (n / TX) % TY, k = n / (TX * TY);
        const int64_t cell = (x0 + i) + (int64_t)bx * ((y0 + j) + (int64_t)by * (z0 + k));
        for (int v = 0; v < 5; ++v)
          a.U2[((int64_t)blk * 5 + v) * a.ncell + cell] = a.U[((int64_t)blk * 5 + v) * a.ncell + cell];
      }
      // faces: the tile's tiles_per_block share of the block's face array
      for (int64_t f = (int64_t)(tile - blk * tiles_per_block) * NT + tid; f < a.nface;
           f += (int64_t)tiles_per_block * NT)
        a.B2[(int64_t)blk * a.nface + f] = a.B[(int64_t)blk * a.nface + f];
    }
    if constexpr (C::PIPE)
    {
      // staged data of this tile unused; the area takes the next tile's gather
      if (has_next)
        load_nbr(work + gridDim.x, buf ^ 1);
      __syncthreads();
      if (has_next)
        stage_tile(work + gridDim.x, buf ^ 1);
      continue;
    }
    else
      return;
  }
  // tile constants in FP64, computed by one thread (FP64 divisions issued by every warp would cost
  // more than the whole gather on GB300) and read after the phase-1 barrier
  __shared__ double s_tc[1]; // dx
  __shared__ R      s_tr[3]; // (R)dx, (R)(dt/dx), (R)(1/dx)
  if (tid == 0)
  {
    const double dx0 = (1.0 / (double)((int64_t)bx << mylevel)) * a.scaling_factor;
    const double dtdx0 = dt / dx0;
    s_tc[0] = dx0;
    s_tr[0] = (R)dx0;
    s_tr[1] = (R)dtdx0;
    s_tr[2] = (R)(1.0 / dx0);
  }

  Phys<R> ph;
  if constexpr (std::is_same<R, float>::value)
  {
    ph.gamma0 = a.gamma0_f;
    ph.smallr = a.smallr_f;
    ph.smallc = a.smallc_f;
    ph.smallp = a.smallp_f;
    ph.slope_type = a.slope_type_f;
  }
  else
  {
    ph.gamma0 = a.gamma0;
    ph.smallr = a.smallr;
    ph.smallc = a.smallc;
    ph.smallp = a.smallp;
    ph.slope_type = a.slope_type;
  }
  ph.riemann = a.riemann;

  unsigned int health = 0u;

  // ---- resolve a block-local cell / face coordinate to (block, local index) ------------------
  auto owner = [&](int ox, int oy, int oz) -> int {
    if ((ox | oy | oz) == 0)
      return blk;
    const int sl = nb_slot(ox, oy, oz);
    const int nb = s_nbr[sl];
    if (nb < 0)
      health |= HEALTH_MISSING_NEIGHBOR;
    else if ((jump_mask >> sl) & 1u)
      health |= HEALTH_LEVEL_JUMP;
    return nb;
  };
  // face / conservative arrays of a real or virtual (coarse/fine ghost) neighbour block
  auto bsrc = [&](int nb) -> const double * {
    if constexpr (C::AMR)
      return nb < a.n_blocks ? a.B + (int64_t)nb * a.nface : a.Bv + (int64_t)(nb - a.n_blocks) * a.nface;
    else
      return a.B + (int64_t)nb * a.nface;
  };
  auto usrc = [&](int nb) -> const double * {
    if constexpr (C::AMR)
      return nb < a.n_blocks ? a.U + (int64_t)nb * 5 * a.ncell : a.Uv + (int64_t)(nb - a.n_blocks) * 5 * a.ncell;
    else
      return a.U + (int64_t)nb * 5 * a.ncell;
  };
  // coarse/fine meshes: the block's own border face shared with a finer face neighbour is that
  // neighbour's value (restriction), read from its virtual block
  auto shared_face = [&](int d, int f, int n, int & nb, int & fq) {
    if constexpr (C::AMR)
    {
      if (nb == blk && (f == 0 || f == n))
      {
        const int sl = nb_slot(d == 0 ? (f == 0 ? -1 : 1) : 0, d == 1 ? (f == 0 ? -1 : 1) : 0, d == 2 ? (f == 0 ? -1 : 1) : 0);
        if (s_kind[sl] == RK_FINER)
        {
          nb = s_nbr[sl];
          fq = f == 0 ? n : 0;
        }
      }
    }
  };
  // ---- phase 1: gather face B at t^n (FillBlockGhostFaces equivalent) and the conservative state
  // of the Q region. Every global load of the phase is issued before any is consumed, so HBM latency
  // is paid once for the phase rather than once per loop trip.
  // x faces one by one (rows of bx + 1 faces are not 16-byte aligned); y and z faces and the
  // conservative state in 16-byte pairs of x-adjacent items: every tile starts at an even x and block
  // sizes are even, so a pair never straddles two blocks and its address is 16-byte aligned.
  constexpr int ITX = (C::NFBX + NT - 1) / NT;
  constexpr int ITY = (C::NFBY / 2 + NT - 1) / NT;
  constexpr int ITZ = (C::NFBZ / 2 + NT - 1) / NT;
  constexpr int ITQ = (C::NQ / 2 + NT - 1) / NT;
  static_assert(C::QX % 2 == 0, "pair loads need an even Q-region width");
  double        fvx[C::PIPE ? 1 : ITX];
  double2       fvy[C::PIPE ? 1 : ITY], fvz[C::PIPE ? 1 : ITZ];
  double2       uq[C::PIPE ? 1 : ITQ][5];
  if constexpr (C::PIPE)
  {
    // the gather was staged by cp.async during the previous tile: convert the faces
    for (int n = tid; n < C::NFB; n += NT)
      fbx[n] = to_r<R>(stage[n]);
  }
  else
  {
#pragma unroll
  for (int it = 0; it < ITX; ++it)
  {
    const int n = tid + it * NT;
    fvx[it] = 0.0;
    if (n < C::NFBX)
    {
      const int i = n % (TX + 5) - 2;
      const int j = (n / (TX + 5)) % C::QY - 2;
      const int k = D3 ? n / ((TX + 5) * C::QY) - 2 : 0;
      const int fi = x0 + i, cj = y0 + j, ck = z0 + k;
      const int ox = face_off(fi, bx), oy = cell_off(cj, by), oz = D3 ? cell_off(ck, bz) : 0;
      int       nb = owner(ox, oy, oz);
      int       fq = fi - ox * bx;
      shared_face(0, fi, bx, nb, fq);
      if (nb >= 0)
        fvx[it] = bsrc(nb)[fq + (int64_t)(bx + 1) * ((cj - oy * by) + (int64_t)by * (ck - oz * bz))];
    }
  }
#pragma unroll
  for (int it = 0; it < ITY; ++it)
  {
    const int n = 2 * (tid + it * NT);
    fvy[it] = make_double2(0.0, 0.0);
    if (n < C::NFBY)
    {
      const int i = n % C::QX - 2;
      const int j = (n / C::QX) % (TY + 5) - 2;
      const int k = D3 ? n / (C::QX * (TY + 5)) - 2 : 0;
      const int ci = x0 + i, fj = y0 + j, ck = z0 + k;
      const int ox = cell_off(ci, bx), oy = face_off(fj, by), oz = D3 ? cell_off(ck, bz) : 0;
      int       nb = owner(ox, oy, oz);
      int       fq = fj - oy * by;
      shared_face(1, fj, by, nb, fq);
      if (nb >= 0)
        fvy[it] = *reinterpret_cast<const double2 *>(
          bsrc(nb) + a.nfx + (ci - ox * bx) + (int64_t)bx * (fq + (int64_t)(by + 1) * (ck - oz * bz)));
    }
  }
#pragma unroll
  for (int it = 0; it < ITZ; ++it)
  {
    const int n = 2 * (tid + it * NT);
    fvz[it] = make_double2(0.0, 0.0);
    if (n < C::NFBZ)
    {
      const int i = n % C::QX - 2;
      const int j = (n / C::QX) % C::QY - 2;
      const int k = D3 ? n / (C::QX * C::QY) - 2 : 0;
      const int ci = x0 + i, cj = y0 + j, fk = z0 + k;
      const int ox = cell_off(ci, bx), oy = cell_off(cj, by), oz = D3 ? face_off(fk, bz) : 0;
      int       nb = owner(ox, oy, oz);
      int       fq = fk - oz * bz;
      if (D3)
        shared_face(2, fk, bz, nb, fq);
      if (nb >= 0)
        fvz[it] = *reinterpret_cast<const double2 *>(
          bsrc(nb) + a.nfx + a.nfy + (ci - ox * bx) + (int64_t)bx * ((cj - oy * by) + (int64_t)by * fq));
    }
  }
#pragma unroll
  for (int it = 0; it < ITQ; ++it)
  {
    const int n = 2 * (tid + it * NT);
    uq[it][0] = uq[it][1] = make_double2(1.0, 1.0);
    uq[it][2] = uq[it][3] = uq[it][4] = make_double2(0.0, 0.0);
    if (n < C::NQ)
    {
      const int i = n % C::QX - 2;
      const int j = (n / C::QX) % C::QY - 2;
      const int k = D3 ? n / (C::QX * C::QY) - 2 : 0;
      const int ci = x0 + i, cj = y0 + j, ck = z0 + k;
      const int ox = cell_off(ci, bx), oy = cell_off(cj, by), oz = D3 ? cell_off(ck, bz) : 0;
      const int nb = owner(ox, oy, oz);
      if (nb >= 0)
      {
        const double * Ub = usrc(nb) + (ci - ox * bx) + (int64_t)bx * ((cj - oy * by) + (int64_t)by * (ck - oz * bz));
#pragma unroll
        for (int v = 0; v < 5; ++v)
          uq[it][v] = *reinterpret_cast<const double2 *>(Ub + (int64_t)v * a.ncell);
      }
    }
  }
#pragma unroll
  for (int it = 0; it < ITX; ++it)
    if (tid + it * NT < C::NFBX)
      fbx[tid + it * NT] = to_r<R>(fvx[it]);
#pragma unroll
  for (int it = 0; it < ITY; ++it)
  {
    const int n = 2 * (tid + it * NT);
    if (n < C::NFBY)
    {
      fby[n] = to_r<R>(fvy[it].x);
      fby[n + 1] = to_r<R>(fvy[it].y);
    }
  }
#pragma unroll
  for (int it = 0; it < ITZ; ++it)
  {
    const int n = 2 * (tid + it * NT);
    if (n < C::NFBZ)
    {
      fbz[n] = to_r<R>(fvz[it].x);
      fbz[n + 1] = to_r<R>(fvz[it].y);
    }
  }
  }
  __syncthreads();
  const double dx = s_tc[0];
  const R      dtdx = s_tr[1];
  const R      dxr = s_tr[0];
  const R      idxr = s_tr[2];
  if constexpr (C::PIPE)
  {
    // the next tile's neighbour table: its loads have the rest of this tile to land
    if (has_next)
      load_nbr(work + gridDim.x, buf ^ 1);
  }

  // SIMPLE_COPY ghosts of a coarser neighbour take the coarse cell's own cell-centred B
  // (ConvertToPrimitivesVariablesFunctor.cpp:439-446), kept by the ghost prepass in Bccv
  // (one bit per neighbour slot holding such a coarser region; most tiles have none)
  unsigned coarse_mask = 0u;
  if (C::AMR && a.prolongation == 0)
  {
    const int lane = tid & 31;
    coarse_mask = __ballot_sync(0xffffffffu, lane < 27 && s_kind[lane] == RK_COARSER && s_nbr[lane] >= a.n_blocks);
  }
  const bool coarse_copy = coarse_mask != 0u;
  auto       coarse_bcc = [&](int ci, int cj, int ck, double * bc) -> bool {
    const int ox = cell_off(ci, bx), oy = cell_off(cj, by), oz = D3 ? cell_off(ck, bz) : 0;
    if ((ox | oy | oz) == 0)
      return false;
    const int sl = nb_slot(ox, oy, oz);
    if (!((coarse_mask >> sl) & 1u))
      return false;
    const int64_t  loc = (ci - ox * bx) + (int64_t)bx * ((cj - oy * by) + (int64_t)by * (ck - oz * bz));
    const double * Bc = a.Bccv + (int64_t)(s_nbr[sl] - a.n_blocks) * 3 * a.ncell + loc;
    bc[0] = Bc[0];
    bc[1] = Bc[a.ncell];
    bc[2] = Bc[2 * a.ncell];
    return true;
  };

  // A ghost cell inside an outside block takes its cell-centred B from that block's own faces
  // (get_conservative_vars of the outside cell, ConvertToPrimitivesVariablesFunctor.cpp:175-221), whose
  // copy of the shared border face is FillOutside's (a WALL copies the same face index)
  // (the slots of this tile's block whose neighbour is an outside block, one bit each; most tiles have none)
  unsigned out_mask = 0u;
  if (a.n_blocks > a.n_owned)
  {
    const int lane = tid & 31;
    const int nbl = lane < 27 ? s_nbr[lane] : -1;
    out_mask = __ballot_sync(0xffffffffu, nbl >= a.n_owned && nbl < a.n_blocks);
  }
  const bool has_outside = out_mask != 0u;
  auto       outside_bcc = [&](int ci, int cj, int ck, double * bc) -> bool {
    const int ox = cell_off(ci, bx), oy = cell_off(cj, by), oz = D3 ? cell_off(ck, bz) : 0;
    if ((ox | oy | oz) == 0)
      return false;
    const int sl = nb_slot(ox, oy, oz);
    if (!((out_mask >> sl) & 1u))
      return false;
    const int nb = s_nbr[sl];
    const int      li = ci - ox * bx, lj = cj - oy * by, lk = ck - oz * bz;
    const double * Bn = a.B + (int64_t)nb * a.nface;
    const int64_t  xr = li + (int64_t)(bx + 1) * (lj + (int64_t)by * lk);
    const int64_t  yr = a.nfx + li + (int64_t)bx * (lj + (int64_t)(by + 1) * lk);
    bc[0] = 0.5 * (Bn[xr] + Bn[xr + 1]);
    bc[1] = 0.5 * (Bn[yr] + Bn[yr + bx]);
    if (D3)
    {
      const int64_t zr = a.nfx + a.nfy + li + (int64_t)bx * (lj + (int64_t)by * lk);
      bc[2] = 0.5 * (Bn[zr] + Bn[zr + (int64_t)bx * by]);
    }
    else
    {
      const double z = Bn[a.nfx + a.nfy + li + (int64_t)bx * lj];
      bc[2] = 0.5 * (z + z);
    }
    return true;
  };

  // primitive variables on the Q region (ConvertToPrimitivesVariablesFunctor) of cell item n
  auto prim_cell = [&](int n, const double * u) {
    const int i = n % C::QX - 2;
    const int j = (n / C::QX) % C::QY - 2;
    const int k = D3 ? n / (C::QX * C::QY) - 2 : 0;
    const int ci = x0 + i, cj = y0 + j, ck = z0 + k;
    const int qn = C::qi(i, j, k);
    if constexpr (C::EXACT)
    {
      // compute_primitives (models/mhd_utils.h:449-515), cIso == 0
      double Bxc = 0.5 * (fbx[C::fxi(i, j, k)] + fbx[C::fxi(i + 1, j, k)]);
      double Byc = 0.5 * (fby[C::fyi(i, j, k)] + fby[C::fyi(i, j + 1, k)]);
      double Bzc = D3 ? 0.5 * (fbz[C::fzi(i, j, k)] + fbz[C::fzi(i, j, k + 1)])
                      : 0.5 * (fbz[C::fzi(i, j, 0)] + fbz[C::fzi(i, j, 0)]);
      if (coarse_copy || has_outside)
      {
        double bc[3];
        if ((coarse_copy && coarse_bcc(ci, cj, ck, bc)) || (has_outside && outside_bcc(ci, cj, ck, bc)))
        {
          Bxc = bc[0];
          Byc = bc[1];
          Bzc = bc[2];
        }
      }
      const double r = fmax(u[ID], a.smallr);
      const double vx = u[IU] / r, vy = u[IV] / r, vz = u[IW] / r;
      const double eken = 0.5 * (vx * vx + vy * vy + vz * vz);
      const double emag = 0.5 * (Bxc * Bxc + Byc * Byc + Bzc * Bzc);
      const double eint = (u[IP] - emag) / r - eken;
      const double p = fmax((a.gamma0 - 1.0) * r * eint, r * a.smallp);
      qh[0 * C::NQ + qn] = r;
      qh[1 * C::NQ + qn] = p;
      qh[2 * C::NQ + qn] = vx;
      qh[3 * C::NQ + qn] = vy;
      qh[4 * C::NQ + qn] = vz;
    }
    else
    {
      // FP32 recovery; FP64 when magnetic + kinetic energy dominate (low beta / high Mach)
      R      Bxc = R(0.5) * (fbx[C::fxi(i, j, k)] + fbx[C::fxi(i + 1, j, k)]);
      R      Byc = R(0.5) * (fby[C::fyi(i, j, k)] + fby[C::fyi(i, j + 1, k)]);
      R      Bzc = D3 ? R(0.5) * (fbz[C::fzi(i, j, k)] + fbz[C::fzi(i, j, k + 1)]) : fbz[C::fzi(i, j, 0)];
      double bcc[3];
      const bool cc = (coarse_copy && coarse_bcc(ci, cj, ck, bcc)) || (has_outside && outside_bcc(ci, cj, ck, bcc));
      if (cc)
      {
        Bxc = to_r<R>(bcc[0]);
        Byc = to_r<R>(bcc[1]);
        Bzc = to_r<R>(bcc[2]);
      }
      const R r = rmax<R>(to_r<R>(u[ID]), ph.smallr);
      const R ir = R(1) / r;
      const R vx = to_r<R>(u[IU]) * ir, vy = to_r<R>(u[IV]) * ir, vz = to_r<R>(u[IW]) * ir;
      const R ekin = R(0.5) * r * (vx * vx + vy * vy + vz * vz);
      const R emag = R(0.5) * (Bxc * Bxc + Byc * Byc + Bzc * Bzc);
      R       p = (ph.gamma0 - R(1)) * (to_r<R>(u[IP]) - emag - ekin);
      if (ekin + emag > R(4) * p * (R(1) / (ph.gamma0 - R(1))))
      {
        // cancellation-prone cell: recover in FP64 from the FP64 state and face values
        double bxl, bxr, byl, byr, bzl, bzr;
        {
          const int fo = face_off(x0 + i, bx), fo1 = face_off(x0 + i + 1, bx);
          const int co_y = cell_off(cj, by), co_z = D3 ? cell_off(ck, bz) : 0;
          const int nb0 = owner(fo, co_y, co_z), nb1 = owner(fo1, co_y, co_z);
          const int64_t tr = (int64_t)(bx + 1) * ((cj - co_y * by) + (int64_t)by * (ck - co_z * bz));
          bxl = nb0 >= 0 ? bsrc(nb0)[(x0 + i - fo * bx) + tr] : 0.0;
          bxr = nb1 >= 0 ? bsrc(nb1)[(x0 + i + 1 - fo1 * bx) + tr] : 0.0;
        }
        {
          const int fo = face_off(y0 + j, by), fo1 = face_off(y0 + j + 1, by);
          const int co_x = cell_off(ci, bx), co_z = D3 ? cell_off(ck, bz) : 0;
          const int nb0 = owner(co_x, fo, co_z), nb1 = owner(co_x, fo1, co_z);
          const int64_t base = a.nfx + (ci - co_x * bx);
          byl = nb0 >= 0 ? bsrc(nb0)[base + (int64_t)bx * ((y0 + j - fo * by) + (int64_t)(by + 1) * (ck - co_z * bz))] : 0.0;
          byr = nb1 >= 0 ? bsrc(nb1)[base + (int64_t)bx * ((y0 + j + 1 - fo1 * by) + (int64_t)(by + 1) * (ck - co_z * bz))] : 0.0;
        }
        if (D3)
        {
          const int fo = face_off(z0 + k, bz), fo1 = face_off(z0 + k + 1, bz);
          const int co_x = cell_off(ci, bx), co_y = cell_off(cj, by);
          const int nb0 = owner(co_x, co_y, fo), nb1 = owner(co_x, co_y, fo1);
          const int64_t base = a.nfx + a.nfy + (ci - co_x * bx) + (int64_t)bx * (cj - co_y * by);
          bzl = nb0 >= 0 ? bsrc(nb0)[base + (int64_t)bx * by * (z0 + k - fo * bz)] : 0.0;
          bzr = nb1 >= 0 ? bsrc(nb1)[base + (int64_t)bx * by * (z0 + k + 1 - fo1 * bz)] : 0.0;
        }
        else
        {
          bzl = bzr = (double)Bzc;
        }
        const double Bx2 = cc ? bcc[0] : 0.5 * (bxl + bxr), By2 = cc ? bcc[1] : 0.5 * (byl + byr),
                     Bz2 = cc ? bcc[2] : 0.5 * (bzl + bzr);
        const double rd = fmax(u[ID], a.smallr);
        const double emag_d = 0.5 * (Bx2 * Bx2 + By2 * By2 + Bz2 * Bz2);
        const double ekin_d = 0.5 * (u[IU] * u[IU] + u[IV] * u[IV] + u[IW] * u[IW]) / rd;
        p = (R)((a.gamma0 - 1.0) * (u[IP] - emag_d - ekin_d));
        health |= HEALTH_LOW_BETA_FP64;
      }
      p = rmax<R>(p, r * ph.smallp);
      qh[0 * C::NQ + qn] = r;
      qh[1 * C::NQ + qn] = p;
      qh[2 * C::NQ + qn] = vx;
      qh[3 * C::NQ + qn] = vy;
      qh[4 * C::NQ + qn] = vz;
    }
  };
  if constexpr (C::PIPE)
  {
    for (int n = tid; n < C::NQ; n += NT)
    {
      const double u[5] = {stage[C::NFB + n], stage[C::NFB + C::NQ + n], stage[C::NFB + 2 * C::NQ + n],
                           stage[C::NFB + 3 * C::NQ + n], stage[C::NFB + 4 * C::NQ + n]};
      prim_cell(n, u);
    }
  }
  else
  {
    // two x-adjacent cells per thread and iteration
#pragma unroll
    for (int ie = 0; ie < 2 * ITQ; ++ie)
    {
      const int it = ie >> 1, e = ie & 1;
      const int n = 2 * (tid + it * NT) + e;
      if (n >= C::NQ)
        continue;
      const double u[5] = {e ? uq[it][0].y : uq[it][0].x, e ? uq[it][1].y : uq[it][1].x,
                           e ? uq[it][2].y : uq[it][2].x, e ? uq[it][3].y : uq[it][3].x,
                           e ? uq[it][4].y : uq[it][4].x};
      prim_cell(n, u);
    }
  }
  __syncthreads();

  // ---- phase 2: limited slopes + Hancock predictor on the S region ---------------------------
  // (ComputeLimitedSlopesFunctor.cpp:121-314, ComputeUpdatedPrimitiveVariablesFunctor.cpp:284-546)
  if constexpr (C::VISC)
  {
    // keep the t^n velocities the viscous fluxes need past the reuse of the primitive region
    for (int n = tid; n < C::NVEL; n += NT)
    {
      const int i = n % C::VX - 1;
      const int j = (n / C::VX) % C::VY - 1;
      const int k = D3 ? n / (C::VX * C::VY) - 1 : 0;
#pragma unroll
      for (int c = 0; c < DIM; ++c)
        vel[c * C::NVEL + n] = qh[(IU + c) * C::NQ + C::qi(i, j, k)];
    }
  }
  for (int n = tid; n < C::NS; n += NT)
  {
    const int i = n % C::SX - 1;
    const int j = (n / C::SX) % C::SY - 1;
    const int k = D3 ? n / (C::SX * C::SY) - 1 : 0;
    const int q0 = C::qi(i, j, k);
    const int qxp = C::qi(i + 1, j, k), qxm = C::qi(i - 1, j, k);
    const int qyp = C::qi(i, j + 1, k), qym = C::qi(i, j - 1, k);
    const int qzp = D3 ? C::qi(i, j, k + 1) : q0, qzm = D3 ? C::qi(i, j, k - 1) : q0;
    const R   st = ph.slope_type;
    R         dq[3][8];
    constexpr int NH = DIM == 3 ? 5 : 4; // nbvar_hydro_only<dim>() (models/MHDState.h:36-43)
#pragma unroll
    for (int v = 0; v < 5; ++v)
    {
      if (v < NH)
      {
        const R * Q = qh + v * C::NQ;
        dq[0][v] = slope1<R>(Q[q0], Q[qxp], Q[qxm], st);
        dq[1][v] = slope1<R>(Q[q0], Q[qyp], Q[qym], st);
        dq[2][v] = D3 ? slope1<R>(Q[q0], Q[qzp], Q[qzm], st) : R(0);
      }
      else
      {
        dq[0][v] = R(0);
        dq[1][v] = R(0);
        dq[2][v] = R(0);
      }
    }
    // magnetic slopes (slope_unsplit_scalar_mag): normal = B_R - B_L, transverse = limited slope of
    // the face average
    const R AL = fbx[C::fxi(i, j, k)], AR = fbx[C::fxi(i + 1, j, k)];
    const R BL = fby[C::fyi(i, j, k)], BR = fby[C::fyi(i, j + 1, k)];
    const R CL = D3 ? fbz[C::fzi(i, j, k)] : fbz[C::fzi(i, j, 0)];
    const R CR = D3 ? fbz[C::fzi(i, j, k + 1)] : fbz[C::fzi(i, j, 0)];
    auto    avgA = [&](int ii, int jj, int kk) { return (fbx[C::fxi(ii, jj, kk)] + fbx[C::fxi(ii + 1, jj, kk)]) * R(0.5); };
    auto    avgB = [&](int ii, int jj, int kk) { return (fby[C::fyi(ii, jj, kk)] + fby[C::fyi(ii, jj + 1, kk)]) * R(0.5); };
    auto    avgC = [&](int ii, int jj, int kk) {
      return D3 ? (fbz[C::fzi(ii, jj, kk)] + fbz[C::fzi(ii, jj, kk + 1)]) * R(0.5)
                : (fbz[C::fzi(ii, jj, 0)] + fbz[C::fzi(ii, jj, 0)]) * R(0.5);
    };
    dq[0][IA] = AR - AL;
    dq[1][IA] = slope1<R>(avgA(i, j, k), avgA(i, j + 1, k), avgA(i, j - 1, k), st);
    dq[0][IB] = slope1<R>(avgB(i, j, k), avgB(i + 1, j, k), avgB(i - 1, j, k), st);
    dq[1][IB] = BR - BL;
    dq[0][IC] = slope1<R>(avgC(i, j, k), avgC(i + 1, j, k), avgC(i - 1, j, k), st);
    dq[1][IC] = slope1<R>(avgC(i, j, k), avgC(i, j + 1, k), avgC(i, j - 1, k), st);
    if (D3)
    {
      dq[2][IA] = slope1<R>(avgA(i, j, k), avgA(i, j, k + 1), avgA(i, j, k - 1), st);
      dq[2][IB] = slope1<R>(avgB(i, j, k), avgB(i, j, k + 1), avgB(i, j, k - 1), st);
      dq[2][IC] = CR - CL;
    }
    else
    {
      dq[2][IA] = dq[2][IB] = dq[2][IC] = R(0);
    }
#pragma unroll
    for (int d = 0; d < DIM; ++d)
#pragma unroll
      for (int v = 0; v < 8; ++v)
        sl[(d * 8 + v) * C::NS + n] = dq[d][v];

    // Hancock predictor
    const R r = qh[0 * C::NQ + q0], p = qh[1 * C::NQ + q0], u = qh[2 * C::NQ + q0],
            v = qh[3 * C::NQ + q0], w = qh[4 * C::NQ + q0];
    const R A = (AL + AR) * R(0.5), B = (BL + BR) * R(0.5), Cc = (CL + CR) * R(0.5);
    if (a.rk2)
    {
      // RK2_SSP: Q2 = Q (ComputeUpdatedPrimitiveVariablesFunctor.cpp:396-407, 531-542)
      q2[ID * C::NS + n] = r;
      q2[IU * C::NS + n] = u;
      q2[IV * C::NS + n] = v;
      q2[IW * C::NS + n] = w;
      q2[IP * C::NS + n] = p;
      q2[IA * C::NS + n] = A;
      q2[IB * C::NS + n] = B;
      q2[IC * C::NS + n] = Cc;
      continue;
    }
    const R gamma = ph.gamma0;
    const R dtdy = dtdx, dtdz = dtdx;
    const R drx = dq[0][ID], dpx = dq[0][IP], dux = dq[0][IU], dvx = dq[0][IV], dwx = dq[0][IW],
            dAx = dq[0][IA], dBx = dq[0][IB], dCx = dq[0][IC];
    const R dry = dq[1][ID], dpy = dq[1][IP], duy = dq[1][IU], dvy = dq[1][IV], dwy = dq[1][IW],
            dAy = dq[1][IA], dBy = dq[1][IB], dCy = dq[1][IC];
    R sr0, su0, sv0, sw0, sp0, sA0, sB0, sC0;
    if constexpr (DIM == 2)
    {
      sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy;
      su0 = (-u * dux - dpx / r - B * dBx / r - Cc * dCx / r) * dtdx + (-v * duy + B * dAy / r) * dtdy;
      sv0 = (-u * dvx + A * dBx / r) * dtdx + (-v * dvy - dpy / r - A * dAy / r - Cc * dCy / r) * dtdy;
      sw0 = (-u * dwx + A * dCx / r) * dtdx + (-v * dwy + B * dCy / r) * dtdy;
      sp0 = (-u * dpx - dux * gamma * p) * dtdx + (-v * dpy - dvy * gamma * p) * dtdy;
      sA0 = (u * dBy + B * duy - v * dAy - A * dvy) * dtdy;
      sB0 = (-u * dBx - B * dux + v * dAx + A * dvx) * dtdx;
      sC0 = (w * dAx + A * dwx - u * dCx - Cc * dux) * dtdx + (-v * dCy - Cc * dvy + w * dBy + B * dwy) * dtdy;
    }
    else
    {
      const R drz = dq[2][ID], dpz = dq[2][IP], duz = dq[2][IU], dvz = dq[2][IV], dwz = dq[2][IW],
              dAz = dq[2][IA], dBz = dq[2][IB], dCz = dq[2][IC];
      sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy + (-w * drz - dwz * r) * dtdz;
      su0 = (-u * dux - (dpx + B * dBx + Cc * dCx) / r) * dtdx + (-v * duy + B * dAy / r) * dtdy +
            (-w * duz + Cc * dAz / r) * dtdz;
      sv0 = (-u * dvx + A * dBx / r) * dtdx + (-v * dvy - (dpy + A * dAy + Cc * dCy) / r) * dtdy +
            (-w * dvz + Cc * dBz / r) * dtdz;
      sw0 = (-u * dwx + A * dCx / r) * dtdx + (-v * dwy + B * dCy / r) * dtdy +
            (-w * dwz - (dpz + A * dAz + B * dBz) / r) * dtdz;
      sp0 = (-u * dpx - dux * gamma * p) * dtdx + (-v * dpy - dvy * gamma * p) * dtdy +
            (-w * dpz - dwz * gamma * p) * dtdz;
      sA0 = (u * dBy + B * duy - v * dAy - A * dvy) * dtdy + (u * dCz + Cc * duz - w * dAz - A * dwz) * dtdz;
      sB0 = (v * dAx + A * dvx - u * dBx - B * dux) * dtdx + (v * dCz + Cc * dvz - w * dBz - B * dwz) * dtdz;
      sC0 = (w * dAx + A * dwx - u * dCx - Cc * dux) * dtdx + (w * dBy + B * dwy - v * dCy - Cc * dvy) * dtdy;
    }
    // half-step gravity kick and viscous predictor on the velocity, after the sources
    // (ComputeUpdatedPrimitiveVariablesFunctor.cpp:372-383, 505-517)
    R ug = u, vg = v, wg = w;
    if (a.src.gravity)
    {
      const R hdt = (R)dt;
      ug += (R)a.src.g[0] * R(0.5) * hdt;
      vg += (R)a.src.g[1] * R(0.5) * hdt;
      if constexpr (DIM == 3)
        wg += (R)a.src.g[2] * R(0.5) * hdt;
    }
    if constexpr (C::VISC)
    {
      if (a.src.visc_predictor)
      {
        // (ComputeUpdatedPrimitiveVariablesFunctor.cpp:174-280): half a step of nu * Laplacian per axis
        const R nu = (R)a.src.mu / r;
        auto    vp = [&](int var, R val) {
          const R * Q = qh + var * C::NQ;
          const R   q0v = Q[q0];
          const R   d2x = Q[qxp] + Q[qxm] - R(2) * q0v;
          val += R(0.5) * nu * d2x / dxr * dtdx;
          const R d2y = Q[qyp] + Q[qym] - R(2) * q0v;
          val += R(0.5) * nu * d2y / dxr * dtdx;
          if constexpr (DIM == 3)
          {
            const R d2z = Q[qzp] + Q[qzm] - R(2) * q0v;
            val += R(0.5) * nu * d2z / dxr * dtdx;
          }
          return val;
        };
        ug = vp(IU, ug);
        vg = vp(IV, vg);
        if constexpr (DIM == 3)
          wg = vp(IW, wg);
      }
    }
    q2[ID * C::NS + n] = r + R(0.5) * sr0;
    q2[IU * C::NS + n] = ug + R(0.5) * su0;
    q2[IV * C::NS + n] = vg + R(0.5) * sv0;
    q2[IW * C::NS + n] = wg + R(0.5) * sw0;
    q2[IP * C::NS + n] = p + R(0.5) * sp0;
    q2[IA * C::NS + n] = A + R(0.5) * sA0;
    q2[IB * C::NS + n] = B + R(0.5) * sB0;
    q2[IC * C::NS + n] = Cc + R(0.5) * sC0;
  }

  // ---- phase 3: edge electric field at t^n on [-1, T+2) (ComputeElectricFieldFunctor.cpp:97-235)
  for (int n = tid; n < C::NE; n += NT)
  {
    const int i = n % C::EX - 1;
    const int j = (n / C::EX) % C::EY - 1;
    const int k = D3 ? n / (C::EX * C::EY) - 1 : 0;
    const R * QU = qh + 2 * C::NQ;
    const R * QV = qh + 3 * C::NQ;
    const R * QW = qh + 4 * C::NQ;
    if constexpr (DIM == 2)
    {
      const R u = R(0.25) * (QU[C::qi(i - 1, j - 1, 0)] + QU[C::qi(i - 1, j, 0)] + QU[C::qi(i, j - 1, 0)] + QU[C::qi(i, j, 0)]);
      const R v = R(0.25) * (QV[C::qi(i - 1, j - 1, 0)] + QV[C::qi(i - 1, j, 0)] + QV[C::qi(i, j - 1, 0)] + QV[C::qi(i, j, 0)]);
      const R A = R(0.5) * (fbx[C::fxi(i, j - 1, 0)] + fbx[C::fxi(i, j, 0)]);
      const R B = R(0.5) * (fby[C::fyi(i - 1, j, 0)] + fby[C::fyi(i, j, 0)]);
      ee[n] = u * B - v * A;
    }
    else
    {
      {
        const R v = R(0.25) * (QV[C::qi(i, j - 1, k - 1)] + QV[C::qi(i, j - 1, k)] + QV[C::qi(i, j, k - 1)] + QV[C::qi(i, j, k)]);
        const R w = R(0.25) * (QW[C::qi(i, j - 1, k - 1)] + QW[C::qi(i, j - 1, k)] + QW[C::qi(i, j, k - 1)] + QW[C::qi(i, j, k)]);
        const R B = R(0.5) * (fby[C::fyi(i, j, k - 1)] + fby[C::fyi(i, j, k)]);
        const R Cc = R(0.5) * (fbz[C::fzi(i, j - 1, k)] + fbz[C::fzi(i, j, k)]);
        ee[0 * C::NE + n] = v * Cc - w * B;
      }
      {
        const R u = R(0.25) * (QU[C::qi(i - 1, j, k - 1)] + QU[C::qi(i - 1, j, k)] + QU[C::qi(i, j, k - 1)] + QU[C::qi(i, j, k)]);
        const R w = R(0.25) * (QW[C::qi(i - 1, j, k - 1)] + QW[C::qi(i - 1, j, k)] + QW[C::qi(i, j, k - 1)] + QW[C::qi(i, j, k)]);
        const R A = R(0.5) * (fbx[C::fxi(i, j, k - 1)] + fbx[C::fxi(i, j, k)]);
        const R Cc = R(0.5) * (fbz[C::fzi(i - 1, j, k)] + fbz[C::fzi(i, j, k)]);
        ee[1 * C::NE + n] = w * A - u * Cc;
      }
      {
        const R u = R(0.25) * (QU[C::qi(i - 1, j - 1, k)] + QU[C::qi(i - 1, j, k)] + QU[C::qi(i, j - 1, k)] + QU[C::qi(i, j, k)]);
        const R v = R(0.25) * (QV[C::qi(i - 1, j - 1, k)] + QV[C::qi(i - 1, j, k)] + QV[C::qi(i, j - 1, k)] + QV[C::qi(i, j, k)]);
        const R A = R(0.5) * (fbx[C::fxi(i, j - 1, k)] + fbx[C::fxi(i, j, k)]);
        const R B = R(0.5) * (fby[C::fyi(i - 1, j, k)] + fby[C::fyi(i, j, k)]);
        ee[2 * C::NE + n] = u * B - v * A;
      }
    }
  }
  __syncthreads();

  // ---- phase 4: half-step face-B source (ComputeSourceFaceMagFunctor.cpp:114-203) ------------
  for (int n = tid; n < C::NS; n += NT)
  {
    const int i = n % C::SX - 1;
    const int j = (n / C::SX) % C::SY - 1;
    const int k = D3 ? n / (C::SX * C::SY) - 1 : 0;
    const R   dtdy = dtdx, dtdz = dtdx;
    if constexpr (DIM == 2)
    {
      sf[0 * C::NS + n] = (ee[C::ei(i, j + 1, 0)] - ee[C::ei(i, j, 0)]) * R(0.5) * dtdy;
      sf[1 * C::NS + n] = -(ee[C::ei(i + 1, j, 0)] - ee[C::ei(i, j, 0)]) * R(0.5) * dtdx;
    }
    else
    {
      const R * Ex = ee;
      const R * Ey = ee + C::NE;
      const R * Ez = ee + 2 * C::NE;
      sf[0 * C::NS + n] = (Ez[C::ei(i, j + 1, k)] - Ez[C::ei(i, j, k)]) * R(0.5) * dtdy -
                          (Ey[C::ei(i, j, k + 1)] - Ey[C::ei(i, j, k)]) * R(0.5) * dtdz;
      sf[1 * C::NS + n] = -(Ez[C::ei(i + 1, j, k)] - Ez[C::ei(i, j, k)]) * R(0.5) * dtdx +
                          (Ex[C::ei(i, j, k + 1)] - Ex[C::ei(i, j, k)]) * R(0.5) * dtdz;
      sf[2 * C::NS + n] = (Ey[C::ei(i + 1, j, k)] - Ey[C::ei(i, j, k)]) * R(0.5) * dtdx -
                          (Ex[C::ei(i, j + 1, k)] - Ex[C::ei(i, j, k)]) * R(0.5) * dtdy;
    }
  }
  __syncthreads(); // qh (primitives at t^n) and ee are dead from here on

  // ---- phase 5: edge EMFs and face fluxes, one pass per direction; no barrier between passes
  {
    TileView<C> tv;
    tv.fb[0] = fbx;
    tv.fb[1] = fby;
    tv.fb[2] = fbz;
    tv.sl = sl;
    tv.q2 = q2;
    tv.sf = sf;
    tv.emfd = emfd;
    tv.fl = fl;
    tv.s_nbr = s_nbr;
    tv.ph = ph;
    tv.dtdx = dtdx;
    tv.x0 = x0;
    tv.y0 = y0;
    tv.z0 = z0;
    tv.bx = bx;
    tv.by = by;
    tv.bz = bz;
    tv.n_owned = a.n_owned;
    tv.rk2 = a.rk2;
    if constexpr (C::AMR)
    {
      tv.s_kind = s_kind;
      tv.blk = blk;
      tv.pass = a.pass;
      tv.fine = a.fine;
      tv.emf_side = a.emf_side;
      tv.emf_slot = a.emf_slot;
      tv.emf_self = (a.pass == 1 && a.emf_slot[blk] >= 0)
                      ? a.emf_side + (int64_t)a.emf_slot[blk] * C::NECOMP * ((int64_t)(bx + 1) * (by + 1) * (D3 ? bz + 1 : 1))
                      : nullptr;
    }
    constexpr int E2 = edge_count<C, 2>();
    constexpr int E1 = DIM == 3 ? edge_count<C, 1>() : 0;
    constexpr int E0 = DIM == 3 ? edge_count<C, 0>() : 0;
    constexpr int F0 = face_count<C, 0>(), F1 = face_count<C, 1>();
    edge_pass<C, 2, 0>(tv, tid);
    if constexpr (DIM == 3)
    {
      edge_pass<C, 1, E2 % NT>(tv, tid);
      edge_pass<C, 0, (E2 + E1) % NT>(tv, tid);
    }
    flux_pass<C, 0, (E2 + E1 + E0) % NT>(tv, tid);
    flux_pass<C, 1, (E2 + E1 + E0 + F0) % NT>(tv, tid);
    if constexpr (DIM == 3)
      flux_pass<C, 2, (E2 + E1 + E0 + F0 + F1) % NT>(tv, tid);
  }
  __syncthreads();
  if constexpr (C::AMR)
  {
    amr_border_fluxes<C>(a, fl, s_kind, blk, x0, y0, z0, tid, vel, dxr, dtdx);
    __syncthreads();
    if (side_only)
    {
      // this tile's update runs in pass 2; with PIPE the next tile's gather is issued here instead of
      // in phase 6 (the staging area is dead: phase 5 and the border fluxes are done)
      if constexpr (C::PIPE)
      {
        if (has_next)
          stage_tile(work + gridDim.x, buf ^ 1);
        continue;
      }
      else
        return;
    }
  }

  // ---- phase 6: CT update (ReadEmfAndUpdateFunctor.cpp:58-163) on faces [0, T] along each
  // normal; a tile writes faces [0, T) and face T when it ends at the block border, and keeps all
  // of them in shared memory for the CFL of the updated cells. The face loads of this phase and the
  // conservative state of phase 7 are issued together, before either is used.
  double upre[C::CPT][C::NFV];
  {
    const double * Mx = emfd;
    const double * My = emfd + (DIM == 3 ? C::NM : 0);
    const double * Mz = emfd + (DIM == 3 ? 2 * C::NM : 0);
    const bool     ex = (x0 + TX == bx), ey = (y0 + TY == by), ez = (z0 + TZ == bz);
    double *       B2blk = a.B2 + (int64_t)blk * a.nface;
    const double * Bblk = a.B + (int64_t)blk * a.nface;
    // block-local face index of shared-memory face item n
    auto face_g = [&](int n) -> int64_t {
      if (n < C::NB2X)
      {
        const int i = n % (TX + 1), j = (n / (TX + 1)) % TY, k = n / ((TX + 1) * TY);
        return (x0 + i) + (int64_t)(bx + 1) * ((y0 + j) + (int64_t)by * (z0 + k));
      }
      if (n < C::NB2X + C::NB2Y)
      {
        const int nn = n - C::NB2X;
        const int i = nn % TX, j = (nn / TX) % (TY + 1), k = nn / (TX * (TY + 1));
        return a.nfx + (x0 + i) + (int64_t)bx * ((y0 + j) + (int64_t)(by + 1) * (z0 + k));
      }
      const int nn = n - C::NB2X - C::NB2Y;
      const int i = nn % TX, j = (nn / TX) % TY, k = nn / (TX * TY);
      return a.nfx + a.nfy + (x0 + i) + (int64_t)bx * ((y0 + j) + (int64_t)by * (z0 + k));
    };
    constexpr int ITB = (C::NB2 + NT - 1) / NT;
    double        bold[ITB];
#pragma unroll
    for (int it = 0; it < ITB; ++it)
    {
      const int n = tid + it * NT;
      bold[it] = n < C::NB2 ? Bblk[face_g(n)] : 0.0;
    }
#pragma unroll
    for (int c = 0; c < C::CPT; ++c)
    {
      const int n = tid + c * NT;
#pragma unroll
      for (int v = 0; v < C::NFV; ++v)
        upre[c][v] = 0.0;
      if (n < C::NCELL)
      {
        const int     i = n % TX, j = (n / TX) % TY, k = n / (TX * TY);
        const int64_t cell = (x0 + i) + (int64_t)bx * ((y0 + j) + (int64_t)by * (z0 + k));
#pragma unroll
        for (int v = 0; v < 5; ++v)
          upre[c][v] = a.U[((int64_t)blk * 5 + v) * a.ncell + cell];
        if constexpr (DIM == 2)
          upre[c][5] = a.B[(int64_t)blk * a.nface + a.nfx + a.nfy + cell];
      }
    }
    if constexpr (C::PIPE)
    {
      // slopes, predictor and face source are dead: their area receives the next tile's gather while
      // the loads above are in flight and phases 6-7 run
      if (has_next)
        stage_tile(work + gridDim.x, buf ^ 1);
    }
#pragma unroll
    for (int it = 0; it < ITB; ++it)
    {
      const int n = tid + it * NT;
      if (n >= C::NB2)
        continue;
      double bnew;
      bool   owned;
      if (n < C::NB2X)
      {
        const int i = n % (TX + 1), j = (n / (TX + 1)) % TY, k = n / ((TX + 1) * TY);
        double d;
        if constexpr (DIM == 2)
          d = curl2<C::EXACT>(Mz[C::mi(i, j + 1, 0)] - Mz[C::mi(i, j, 0)], 0.0);
        else
          d = curl2<C::EXACT>(Mz[C::mi(i, j + 1, k)] - Mz[C::mi(i, j, k)], My[C::mi(i, j, k + 1)] - My[C::mi(i, j, k)]);
        bnew = bold[it] + d;
        owned = i < TX || ex;
      }
      else if (n < C::NB2X + C::NB2Y)
      {
        const int nn = n - C::NB2X;
        const int i = nn % TX, j = (nn / TX) % (TY + 1), k = nn / (TX * (TY + 1));
        if constexpr (DIM == 2)
          bnew = bold[it] - (Mz[C::mi(i + 1, j, 0)] - Mz[C::mi(i, j, 0)]);
        else
        {
          const double d =
            curl2<C::EXACT>(Mx[C::mi(i, j, k + 1)] - Mx[C::mi(i, j, k)], Mz[C::mi(i + 1, j, k)] - Mz[C::mi(i, j, k)]);
          bnew = bold[it] + d;
        }
        owned = j < TY || ey;
      }
      else
      {
        const int nn = n - C::NB2X - C::NB2Y;
        const int i = nn % TX, j = (nn / TX) % TY, k = nn / (TX * TY);
        const double d =
          curl2<C::EXACT>(My[C::mi(i + 1, j, k)] - My[C::mi(i, j, k)], Mx[C::mi(i, j + 1, k)] - Mx[C::mi(i, j, k)]);
        bnew = bold[it] + d;
        owned = k < TZ || ez;
      }
      if (owned)
        B2blk[face_g(n)] = bnew;
      b2s[n] = to_r<R>(bnew);
    }
  }
  __syncthreads();

  // ---- phase 7: conservative update (ReadFluxesAndConservativeUpdateFunctor.cpp:240-436),
  // write U2 (and 2D Bz), fused CFL of the new state (ComputeDtMHDFunctor.cpp:86-151) ----------
  double my_invdt = 0.0;   // FP64 path
  float  my_invdt_f = 0.0f; // mixed path: FP32 maximum, widened once per CTA
#pragma unroll
  for (int c = 0; c < C::CPT; ++c)
  {
    const int n = tid + c * NT;
    if (n >= C::NCELL)
      continue;
    const int     i = n % TX, j = (n / TX) % TY, k = n / (TX * TY);
    const int64_t cell = (x0 + i) + (int64_t)bx * ((y0 + j) + (int64_t)by * (z0 + k));
    double        u2[C::NFV];
#pragma unroll
    for (int v = 0; v < C::NFV; ++v)
      u2[v] = upre[c][v];
    // mixed path: the 2 DIM face terms of each variable are summed without rounding loss (TwoSum into
    // a sum and an error term, both FP32), then added to the FP64 state as two FP64 adds, so that the
    // flux a face gives one cell and takes from the other cancel in the totals to FP64 round-off
    float dU[C::NFV], eU[C::NFV];
#pragma unroll
    for (int v = 0; v < C::NFV; ++v)
      dU[v] = eU[v] = 0.0f;
#pragma unroll
    for (int dir = 0; dir < DIM; ++dir)
    {
      int fL, fR;
      if (dir == 0)
      {
        fL = i + (TX + 1) * (j + TY * k);
        fR = fL + 1;
      }
      else if (dir == 1)
      {
        fL = C::NF_X + i + TX * (j + (TY + 1) * k);
        fR = fL + TX;
      }
      else
      {
        fL = C::NF_X + C::NF_Y + i + TX * (j + TY * k);
        fR = fL + TX * TY;
      }
#pragma unroll
      for (int v = 0; v < C::NFV; ++v)
      {
        if constexpr (C::EXACT)
        {
          R acc = R(0);
          acc = acc + fl[v * C::NFT + fL];
          acc = acc - fl[v * C::NFT + fR];
          u2[v] += (double)acc;
        }
        else
        {
          if (dir == 0)
            dU[v] = fl[v * C::NFT + fL];
          else
            two_sum_acc(dU[v], eU[v], fl[v * C::NFT + fL]);
          two_sum_acc(dU[v], eU[v], -fl[v * C::NFT + fR]);
        }
      }
    }
    if constexpr (!C::EXACT && C::AMR)
    {
      // A face toward finer neighbours carries the FP64 sum of their fluxes / 2^d, held in the FP32
      // flux array rounded to `hi`; its remainder lo = sum - hi joins the error-free sum here, so the
      // coarse cell gains exactly what the fine cells lose
      if (a.pass == 2)
      {
        const int lc[3] = {i, j, k};
        const int org[3] = {x0, y0, z0};
        const int bsz[3] = {bx, by, bz};
#pragma unroll
        for (int dir = 0; dir < DIM; ++dir)
        {
          const int t1 = dir == 0 ? 1 : 0, t2 = dir == 2 ? 1 : 2;
          const int g1 = org[t1] + lc[t1], g2 = DIM == 3 ? org[t2] + lc[t2] : 0;
          const int gc = org[dir] + lc[dir];
#pragma unroll
          for (int side = -1; side <= 1; side += 2)
          {
            if (side < 0 ? gc != 0 : gc != bsz[dir] - 1)
              continue;
            const int sl = nb_slot(dir == 0 ? side : 0, dir == 1 ? side : 0, dir == 2 ? side : 0);
            if (s_kind[sl] != RK_FINER)
              continue;
#pragma unroll
            for (int v = 0; v < C::NFV; ++v)
            {
              const double sum = fine_face_flux<C>(a, blk, sl, dir, side, g1, g2, v);
              const float  lo = to_r<float>(sum - to_d<float>(to_r<float>(sum)));
              two_sum_acc(dU[v], eU[v], side < 0 ? lo : -lo);
            }
          }
        }
      }
    }
    if constexpr (!C::EXACT)
    {
#pragma unroll
      for (int v = 0; v < C::NFV; ++v)
        u2[v] = (u2[v] + to_d<float>(dU[v])) + to_d<float>(eU[v]);
    }
    if constexpr (C::VISC)
    {
      // viscous fluxes through the same update, after the three hydro directions
      // (GodunovImplemV0.cpp:179-192); a coarse cell next to finer blocks takes their flux sum
      const int lc[3] = {i, j, k};
      const int org[3] = {x0, y0, z0};
      const int bsz[3] = {bx, by, bz};
      R         dV[4] = {R(0), R(0), R(0), R(0)};
#pragma unroll
      for (int dir = 0; dir < DIM; ++dir)
      {
        R fL[4], fR[4];
        viscous_face_flux<C>(vel, dir, i, j, k, (R)a.src.mu, dxr, dtdx, fL);
        viscous_face_flux<C>(vel, dir, i + (dir == 0), j + (dir == 1), k + (dir == 2), (R)a.src.mu, dxr, dtdx, fR);
        if constexpr (C::AMR)
        {
          if (a.pass == 2)
          {
            const int t1 = dir == 0 ? 1 : 0, t2 = dir == 2 ? 1 : 2;
            const int g1 = org[t1] + lc[t1], g2 = DIM == 3 ? org[t2] + lc[t2] : 0;
#pragma unroll
            for (int side = -1; side <= 1; side += 2)
            {
              const int gc = org[dir] + lc[dir];
              if (side < 0 ? gc != 0 : gc != bsz[dir] - 1)
                continue;
              const int sl = nb_slot(dir == 0 ? side : 0, dir == 1 ? side : 0, dir == 2 ? side : 0);
              if (s_kind[sl] != RK_FINER)
                continue;
#pragma unroll
              for (int v = 0; v < 4; ++v)
              {
                const R fv = to_r<R>(fine_face_flux<C>(a, blk, sl, dir, side, g1, g2, C::NFV + v));
                if (side < 0)
                  fL[v] = fv;
                else
                  fR[v] = fv;
              }
            }
          }
        }
#pragma unroll
        for (int v = 0; v < 4; ++v)
        {
          R acc = R(0);
          acc = acc + fL[v];
          acc = acc - fR[v];
          if constexpr (C::EXACT)
            u2[IP + v] += (double)acc;
          else
            dV[v] += acc;
        }
      }
      if constexpr (!C::EXACT)
      {
#pragma unroll
        for (int v = 0; v < 4; ++v)
          u2[IP + v] += to_d<R>(dV[v]);
      }
    }
    if (a.src.gravity)
    {
      // AddGravitySourceTerm (AddGravitySourceTerm.cpp:47-99), FP64
      const double rho_old = upre[c][ID], rho_new = u2[ID];
      double       ru = u2[IU], rv = u2[IV], rw = DIM == 3 ? u2[IW] : 0.0;
      double       ekin_old = 0.5 * (ru * ru + rv * rv) / rho_new;
      if constexpr (DIM == 3)
        ekin_old += 0.5 * (rw * rw) / rho_new;
      ru += dt * a.src.g[0] * (rho_old + rho_new) / 2;
      rv += dt * a.src.g[1] * (rho_old + rho_new) / 2;
      if constexpr (DIM == 3)
        rw += dt * a.src.g[2] * (rho_old + rho_new) / 2;
      u2[IU] = ru;
      u2[IV] = rv;
      if constexpr (DIM == 3)
        u2[IW] = rw;
      double ekin_new = 0.5 * (ru * ru + rv * rv) / rho_new;
      if constexpr (DIM == 3)
        ekin_new += 0.5 * (rw * rw) / rho_new;
      u2[IP] += (ekin_new - ekin_old);
    }
#pragma unroll
    for (int v = 0; v < 5; ++v)
      a.U2[((int64_t)blk * 5 + v) * a.ncell + cell] = u2[v];
    if constexpr (DIM == 2)
      a.B2[(int64_t)blk * a.nface + a.nfx + a.nfy + cell] = u2[5];
    // u2[ID] > 0 and finite E, rho u, as integer tests on the bit patterns
    {
      const long long bd = __double_as_longlong(u2[ID]);
      if (!(bd > 0 && bd <= 0x7ff0000000000000LL))
        health |= HEALTH_BAD_DENSITY;
      const long long ex = 0x7ff0000000000000LL;
      if ((__double_as_longlong(u2[IP]) & ex) == ex || (__double_as_longlong(u2[IU]) & ex) == ex)
        health |= HEALTH_NONFINITE;
    }

    if (a.invdt_out)
    {
      const R Axl = b2s[i + (TX + 1) * (j + TY * k)], Axr = b2s[i + 1 + (TX + 1) * (j + TY * k)];
      const R Ayl = b2s[C::NB2X + i + TX * (j + (TY + 1) * k)], Ayr = b2s[C::NB2X + i + TX * (j + 1 + (TY + 1) * k)];
      [[maybe_unused]] double val = 0.0; // FP64 path
      if constexpr (C::EXACT)
      {
        const double Ax = 0.5 * (Axl + Axr);
        const double Ay = 0.5 * (Ayl + Ayr);
        double       Az;
        if constexpr (DIM == 3)
          Az = 0.5 * (b2s[C::NB2X + C::NB2Y + i + TX * (j + TY * k)] + b2s[C::NB2X + C::NB2Y + i + TX * (j + TY * (k + 1))]);
        else
          Az = 0.5 * (u2[5] + u2[5]);
        const double r = fmax(u2[ID], a.smallr);
        const double vx = u2[IU] / r, vy = u2[IV] / r, vz = u2[IW] / r;
        const double eken = 0.5 * (vx * vx + vy * vy + vz * vz);
        const double emag = 0.5 * (Ax * Ax + Ay * Ay + Az * Az);
        const double eint = (u2[IP] - emag) / r - eken;
        const double p = fmax((a.gamma0 - 1.0) * r * eint, r * a.smallp);
        const double b2 = Ax * Ax + Ay * Ay + Az * Az;
        const double c2 = a.gamma0 * p / r;
        const double d2 = 0.5 * (b2 / r + c2);
        const double cfx = sqrt(d2 + sqrt(d2 * d2 - c2 * Ax * Ax / r)) + fabs(vx);
        const double cfy = sqrt(d2 + sqrt(d2 * d2 - c2 * Ay * Ay / r)) + fabs(vy);
        double cfz = 0.0;
        if constexpr (DIM == 3)
          cfz = sqrt(d2 + sqrt(d2 * d2 - c2 * Az * Az / r)) + fabs(vz);
        val = cfl_inv_dt_fp64(DIM, cfx, cfy, cfz, dx, u2[ID], a.src);
      }
      else
      {
        // FP32 estimate of the fastest signal speed
        const float bxf = 0.5f * (Axl + Axr);
        const float byf = 0.5f * (Ayl + Ayr);
        float       bzf;
        if constexpr (DIM == 3)
          bzf = 0.5f * (b2s[C::NB2X + C::NB2Y + i + TX * (j + TY * k)] + b2s[C::NB2X + C::NB2Y + i + TX * (j + TY * (k + 1))]);
        else
          bzf = to_r<R>(u2[5]);
        const float r = fmaxf(to_r<R>(u2[ID]), ph.smallr);
        const float ir = 1.0f / r;
        const float vx = to_r<R>(u2[IU]) * ir, vy = to_r<R>(u2[IV]) * ir, vz = to_r<R>(u2[IW]) * ir;
        const float ekin = 0.5f * r * (vx * vx + vy * vy + vz * vz);
        const float emag = 0.5f * (bxf * bxf + byf * byf + bzf * bzf);
        const float g = ph.gamma0;
        const float p = fmaxf((g - 1.0f) * (to_r<R>(u2[IP]) - emag - ekin), r * ph.smallp);
        const float b2 = 2.0f * emag;
        const float c2 = g * p * ir;
        const float d2 = 0.5f * (b2 * ir + c2);
        const float cfx = sqrtf(d2 + sqrtf(fmaxf(d2 * d2 - c2 * bxf * bxf * ir, 0.0f))) + fabsf(vx);
        const float cfy = sqrtf(d2 + sqrtf(fmaxf(d2 * d2 - c2 * byf * byf * ir, 0.0f))) + fabsf(vy);
        float       cfz = 0.0f;
        if constexpr (DIM == 3)
          cfz = sqrtf(d2 + sqrtf(fmaxf(d2 * d2 - c2 * bzf * bzf * ir, 0.0f))) + fabsf(vz);
        my_invdt_f = fmaxf(my_invdt_f, cfl_inv_dt_fp32(DIM, cfx, cfy, cfz, dxr, idxr, to_r<R>(u2[ID]), a.src));
      }
      if constexpr (C::EXACT)
        my_invdt = fmax(my_invdt, val);
    }
  }

  if (health)
    atomicOr(&s_health, health);
  if (a.invdt_out)
  {
    if constexpr (C::EXACT)
    {
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
        my_invdt = fmax(my_invdt, __shfl_xor_sync(0xffffffffu, my_invdt, off));
      if ((tid & 31) == 0)
        s_red[tid >> 5] = my_invdt;
    }
    else
    {
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
        my_invdt_f = fmaxf(my_invdt_f, __shfl_xor_sync(0xffffffffu, my_invdt_f, off));
      if ((tid & 31) == 0)
        reinterpret_cast<float *>(s_red)[tid >> 5] = my_invdt_f;
    }
  }
  __syncthreads();
  if (tid == 0)
  {
    if (a.invdt_out)
    {
      double m;
      if constexpr (C::EXACT)
      {
        m = s_red[0];
        for (int w = 1; w < NT / 32; ++w)
          m = fmax(m, s_red[w]);
      }
      else
      {
        float mf = reinterpret_cast<const float *>(s_red)[0];
        for (int w = 1; w < NT / 32; ++w)
          mf = fmaxf(mf, reinterpret_cast<const float *>(s_red)[w]);
        m = f2d_bits(mf);
      }
      atomic_max_pos_double(&a.invdt_out[myprob], m);
    }
    if (s_health)
      atomicOr(a.health, s_health);
  }
  } // tile loop
}

} // namespace gmhd

// Column step: the mixed-precision MUSCL-Hancock + CT stage of one leaf block computed by z-marching
// columns (3D, conforming meshes).
//
// A CTA owns a column: a TX x TY footprint of one leaf block through the block's whole z extent. It
// walks the column plane by plane, keeping only the planes still needed in shared memory, so the
// two-cell halo is recomputed along x and y only (the 8^3 tiles of fused_step_kernel also recompute
// it along z, above and below every tile). Same arithmetic, in the same order, as fused_step_kernel
// (mixed path): primitives, limited slopes + Hancock predictor, edge E, sFaceMag, HLLD face fluxes,
// 2D-HLLD edge EMFs with the border averaging, FP64 CT update, conservative update (TwoSum face terms,
// FP64 adds) and the fused CFL of the new state. References: scheme/GodunovImplemV0.cpp:101-207 and
// the functors cited in fused_step.cuh.
//
// Pipeline. Step s (s = -4 .. bz+1) runs three intervals separated by CTA barriers:
//   I1: edge E of plane s+1 (z edges) and level s+1 (x, y edges); slopes + predictor of S-plane s;
//       CT update of the faces of output plane s-2 (and its top z faces)
//   I2: half-step face source of S-plane s; primitives of Q-plane s+2 from global memory; conservative
//       update, health checks and CFL of output plane s-2
//   I3: face fluxes and edge EMFs: z edges and x/y fluxes of plane s-1, x/y edges and z fluxes of
//       level s (the face / edge layer between planes s-1 and s)
// Every plane-wide array is a ring of the few planes alive at once (Q: 3 planes; t^n faces: 5 planes
// of Bx, By, 4 levels of Bz; slopes, predictor, face source: 2 S-planes; E: 2; fluxes, EMFs: 1-2).
// About 103 KB of shared memory for 16 x 8 columns, so two 256-thread CTAs share an SM and one's
// barrier waits overlap the other's work.
#pragma once

#include "fused_step.cuh"

namespace gmhd
{

template <int TX_, int TY_, int NT_>
struct ColCfg
{
  using R = float;
  static constexpr int TX = TX_, TY = TY_, NT = NT_;
  // Q plane: cells [-2, T+2)
  static constexpr int QX = TX + 4, QY = TY + 4, NQP = QX * QY;
  // t^n faces: Bx faces [-2, TX+2] x cells [-2, TY+2); By cells x faces [-2, TY+2]; Bz cells, per level
  static constexpr int BXX = TX + 5, NBXP = BXX * QY;
  static constexpr int NBYP = QX * (TY + 5);
  static constexpr int NBZP = QX * QY;
  // S plane (slopes, predictor, face source): cells [-1, T+1)
  static constexpr int SX = TX + 2, SY = TY + 2, NSP = SX * SY;
  // edge E plane / level: edges [-1, T+2)
  static constexpr int EX = TX + 3, EY = TY + 3, NEP = EX * EY;
  // face fluxes of a plane (x, y) and of a level (z)
  static constexpr int NFX = (TX + 1) * TY, NFY = TX * (TY + 1), NFZ = TX * TY;
  // EMFs: z edges of a plane, x and y edges of a level
  static constexpr int NMZ = (TX + 1) * (TY + 1), NMX = TX * (TY + 1), NMY = (TX + 1) * TY;

  // shared memory, in floats
  static constexpr int OFF_Q = 0;                       // [3 planes][5][NQP]
  static constexpr int OFF_BX = OFF_Q + 15 * NQP;       // [5 planes][NBXP]
  static constexpr int OFF_BY = OFF_BX + 5 * NBXP;      // [5 planes][NBYP]
  static constexpr int OFF_BZ = OFF_BY + 5 * NBYP;      // [4 levels][NBZP]
  static constexpr int OFF_SL = OFF_BZ + 4 * NBZP;      // [2 S-planes][3 dirs][8][NSP]
  static constexpr int OFF_Q2 = OFF_SL + 48 * NSP;      // [2][8][NSP]
  static constexpr int OFF_SF = OFF_Q2 + 16 * NSP;      // [2][3][NSP]
  static constexpr int OFF_EZ = OFF_SF + 6 * NSP;       // [2 planes][NEP]
  static constexpr int OFF_EX = OFF_EZ + 2 * NEP;       // [2 levels][NEP]
  static constexpr int OFF_EY = OFF_EX + 2 * NEP;       // [2 levels][NEP]
  static constexpr int OFF_FX = OFF_EY + 2 * NEP;       // [5][NFX]
  static constexpr int OFF_FY = OFF_FX + 5 * NFX;       // [5][NFY]
  static constexpr int OFF_FZ = OFF_FY + 5 * NFY;       // [2 levels][5][NFZ]
  static constexpr int OFF_NX = OFF_FZ + 10 * NFZ;      // updated Bx of a plane (FP32, CFL)
  static constexpr int OFF_NY = OFF_NX + NFX;           // updated By
  static constexpr int OFF_NZ = OFF_NY + NFY;           // [2 levels] updated Bz
  static constexpr int OFF_M = ((OFF_NZ + 2 * NFZ + 1) / 2) * 2; // FP64 EMFs from here (8-byte aligned)
  static constexpr int M_DOUBLES = NMZ + 2 * NMX + 2 * NMY;
  static constexpr int TOTAL = OFF_M + 2 * M_DOUBLES;
  static constexpr size_t SMEM_BYTES = sizeof(float) * (size_t)TOTAL;

  __device__ static int qp(int i, int j) { return (i + 2) + QX * (j + 2); }
  __device__ static int bxp(int i, int j) { return (i + 2) + BXX * (j + 2); }
  __device__ static int byp(int i, int j) { return (i + 2) + QX * (j + 2); }
  __device__ static int bzp(int i, int j) { return (i + 2) + QX * (j + 2); }
  __device__ static int sp(int i, int j) { return (i + 1) + SX * (j + 1); }
  __device__ static int ep(int i, int j) { return (i + 1) + EX * (j + 1); }
};

// ring slots (planes and levels start at -2)
__device__ __forceinline__ int
ring3(int p)
{
  return (p + 6) % 3;
}
__device__ __forceinline__ int
ring5(int p)
{
  return (p + 10) % 5;
}
__device__ __forceinline__ int
ring4(int l)
{
  return (l + 8) & 3;
}
__device__ __forceinline__ int
ring2(int p)
{
  return (p + 4) & 1;
}

// Shared-memory views of a column CTA.
template <class K>
struct ColView
{
  float * sm;
  __device__ float * Q(int plane, int v) const { return sm + K::OFF_Q + (ring3(plane) * 5 + v) * K::NQP; }
  __device__ float * Bx(int plane) const { return sm + K::OFF_BX + ring5(plane) * K::NBXP; }
  __device__ float * By(int plane) const { return sm + K::OFF_BY + ring5(plane) * K::NBYP; }
  __device__ float * Bz(int level) const { return sm + K::OFF_BZ + ring4(level) * K::NBZP; }
  __device__ float * Sl(int splane, int d, int v) const
  {
    return sm + K::OFF_SL + ((ring2(splane) * 3 + d) * 8 + v) * K::NSP;
  }
  __device__ float * Q2(int splane, int v) const { return sm + K::OFF_Q2 + (ring2(splane) * 8 + v) * K::NSP; }
  __device__ float * Sf(int splane, int c) const { return sm + K::OFF_SF + (ring2(splane) * 3 + c) * K::NSP; }
  __device__ float * Ez(int plane) const { return sm + K::OFF_EZ + ring2(plane) * K::NEP; }
  __device__ float * Ex(int level) const { return sm + K::OFF_EX + ring2(level) * K::NEP; }
  __device__ float * Ey(int level) const { return sm + K::OFF_EY + ring2(level) * K::NEP; }
  __device__ float * Fx(int v) const { return sm + K::OFF_FX + v * K::NFX; }
  __device__ float * Fy(int v) const { return sm + K::OFF_FY + v * K::NFY; }
  __device__ float * Fz(int level, int v) const { return sm + K::OFF_FZ + ((level & 1) * 5 + v) * K::NFZ; }
  __device__ float * Nx() const { return sm + K::OFF_NX; }
  __device__ float * Ny() const { return sm + K::OFF_NY; }
  __device__ float * Nz(int level) const { return sm + K::OFF_NZ + (level & 1) * K::NFZ; }
  __device__ double * Mz() const { return reinterpret_cast<double *>(sm + K::OFF_M); }
  __device__ double * Mx(int level) const { return Mz() + K::NMZ + (level & 1) * K::NMX; }
  __device__ double * My(int level) const { return Mz() + K::NMZ + 2 * K::NMX + (level & 1) * K::NMY; }
  // t^n face component c (0 Bx, 1 By, 2 Bz) of the cell at (i, j) in plane p, shifted by sh along c
  // (sh 1: the cell's right / top face); along z the face level is p + sh
  template <int c>
  __device__ float face(int i, int j, int p, int sh) const
  {
    if constexpr (c == 0)
      return Bx(p)[K::bxp(i + sh, j)];
    else if constexpr (c == 1)
      return By(p)[K::byp(i, j + sh)];
    else
      return Bz(p + sh)[K::bzp(i, j)];
  }
};

// reconstruct_state_3d_at_edge (ComputeEmfAndStoreFunctor.cpp:103-367) of the cell at (i, j) of
// S-plane p for the edge corner LOC, on the column layout; the same operations in the same order as
// recon_edge of fused_step.cuh.
template <class K, int D0, int D1, int LOC>
__device__ __forceinline__ void
col_recon_edge(const ColView<K> & t, int i, int j, int p, const Phys<float> & ph, int rk2, float * q)
{
  constexpr bool sh0 = LOC == LOC_RT || LOC == LOC_RB;
  constexpr bool sh1 = LOC == LOC_RT || LOC == LOC_LT;
  constexpr int  sd0 = (LOC == LOC_RT || LOC == LOC_RB) ? 1 : -1;
  constexpr int  sd1 = (LOC == LOC_RT || LOC == LOC_LT) ? 1 : -1;
  constexpr int  sb0 = (LOC == LOC_RT || LOC == LOC_LT) ? 1 : -1;
  constexpr int  sb1 = (LOC == LOC_RT || LOC == LOC_RB) ? 1 : -1;
  const int      sc = K::sp(i, j);
#pragma unroll
  for (int v = 0; v < 8; ++v)
    q[v] = t.Q2(p, v)[sc];
  // the cell's D0 face (right one when shifted) and its neighbours along D1, and the same for D1
  auto f0 = [&](int o) {
    const int io = D1 == 0 ? o : 0, jo = D1 == 1 ? o : 0, po = D1 == 2 ? o : 0;
    return t.template face<D0>(i + io, j + jo, p + po, sh0 ? 1 : 0);
  };
  auto f1 = [&](int o) {
    const int io = D0 == 0 ? o : 0, jo = D0 == 1 ? o : 0, po = D0 == 2 ? o : 0;
    return t.template face<D1>(i + io, j + jo, p + po, sh1 ? 1 : 0);
  };
  const float F0c = f0(0), F1c = f1(0);
  float       B0 = F0c, B1 = F1c;
  if (!rk2)
  {
    // sf of the cell itself or, shifted, of its neighbour across that face (its left / bottom face)
    const int i0 = (D0 == 0 && sh0) ? 1 : 0, j0 = (D0 == 1 && sh0) ? 1 : 0, p0 = (D0 == 2 && sh0) ? 1 : 0;
    const int i1 = (D1 == 0 && sh1) ? 1 : 0, j1 = (D1 == 1 && sh1) ? 1 : 0, p1 = (D1 == 2 && sh1) ? 1 : 0;
    B0 += t.Sf(p + p0, D0)[K::sp(i + i0, j + j0)];
    B1 += t.Sf(p + p1, D1)[K::sp(i + i1, j + j1)];
  }
  const float dB0d1 = slope1<float>(F0c, f0(1), f0(-1), ph.slope_type);
  const float dB1d0 = slope1<float>(F1c, f1(1), f1(-1), ph.slope_type);
  const float * S0 = t.Sl(p, D0, 0) + sc;
  const float * S1 = t.Sl(p, D1, 0) + sc;
  const float   g0 = (float)sd0, g1 = (float)sd1;
  auto          h = [&](int v) { return 0.5f * (g0 * S0[v * K::NSP] + g1 * S1[v * K::NSP]); };
#pragma unroll
  for (int v = 0; v < 5; ++v)
    q[v] += h(v);
  if constexpr (D0 == 0)
    q[IA] = B0 + 0.5f * ((float)sb0 * dB0d1);
  else
    q[IA] += h(IA);
  if constexpr (D0 == 1)
    q[IB] = B0 + 0.5f * ((float)sb0 * dB0d1);
  else
    q[IB] += h(IB);
  if constexpr (D1 == 1)
    q[IB] = B1 + 0.5f * ((float)sb1 * dB1d0);
  else
    q[IB] += h(IB);
  if constexpr (D1 == 2)
    q[IC] = B1 + 0.5f * ((float)sb1 * dB1d0);
  else
    q[IC] += h(IC);
  q[ID] = rmax<float>(ph.smallr, q[ID]);
  q[IP] = rmax<float>(ph.smallp * q[ID], q[IP]);
}

// Per-column constants and neighbour data shared by the item functions.
struct ColCtx
{
  Phys<float> ph;
  float       dtdx, dxr, idxr;
  double      dx, dt;
  int         blk, x0, y0, bx, by, bz, n_owned, rk2;
  const int * nbr; // [27] neighbour table of the block (shared memory)
};

// EMF along CD of the edge at (i, j) on plane / level p (corner cells in S-planes p and p-1 for x and
// y edges), with the border averaging on a conforming mesh (CorrectEmfAtBlockBorderFunctor.cpp:298-356).
template <class K, int CD>
__device__ __forceinline__ double
col_edge(const ColView<K> & t, const ColCtx & c, int i, int j, int p)
{
  constexpr int D0 = CD == 0 ? 1 : 0;
  constexpr int D1 = CD == 2 ? 1 : 2;
  // corner cells: LB (0, 0), RT (-1, -1), RB (-1 along D0), LT (-1 along D1)
  auto ci = [&](int o0, int o1) { return i + (D0 == 0 ? o0 : 0) + (D1 == 0 ? o1 : 0); };
  auto cj = [&](int o0, int o1) { return j + (D0 == 1 ? o0 : 0) + (D1 == 1 ? o1 : 0); };
  auto cp = [&](int o1) { return p + (D1 == 2 ? o1 : 0); };
  float qe[4][8];
  col_recon_edge<K, D0, D1, LOC_LB>(t, ci(0, 0), cj(0, 0), cp(0), c.ph, c.rk2, qe[ELB]);
  col_recon_edge<K, D0, D1, LOC_RT>(t, ci(-1, -1), cj(-1, -1), cp(-1), c.ph, c.rk2, qe[ERT]);
  // y edges: the reference swaps the RB and LT states (ComputeEmfAndStoreFunctor.cpp:551-560)
  col_recon_edge<K, D0, D1, LOC_RB>(t, ci(-1, 0), cj(-1, 0), cp(0), c.ph, c.rk2, qe[CD == 1 ? ELT : ERB]);
  col_recon_edge<K, D0, D1, LOC_LT>(t, ci(0, -1), cj(0, -1), cp(-1), c.ph, c.rk2, qe[CD == 1 ? ERB : ELT]);
  float val = edge_emf<float, CD>(qe, c.ph) * c.dtdx;
  const int gi[3] = {c.x0 + i, c.y0 + j, p};
  const int bs[3] = {c.bx, c.by, c.bz};
  const int v0 = gi[D0] == 0 ? -1 : (gi[D0] == bs[D0] ? 1 : 0);
  const int v1 = gi[D1] == 0 ? -1 : (gi[D1] == bs[D1] ? 1 : 0);
  if (v0 != 0 && v1 != 0)
  {
    const int sl0 = nb_slot(D0 == 0 ? v0 : 0, D0 == 1 ? v0 : 0, 0);
    const int sl1 = nb_slot(D1 == 0 ? v1 : 0, D1 == 1 ? v1 : 0, D1 == 2 ? v1 : 0);
    const int sl2 = nb_slot(D0 == 0 ? v0 : (D1 == 0 ? v1 : 0), D0 == 1 ? v0 : (D1 == 1 ? v1 : 0), D1 == 2 ? v1 : 0);
    const int n0 = c.nbr[sl0], n1 = c.nbr[sl1], n2 = c.nbr[sl2];
    if (n0 >= 0 && n1 >= 0 && n2 >= 0)
    {
      float acc = 0.0f;
      int   count = 1;
      acc += val;
      if (n0 < c.n_owned)
      {
        acc += val;
        count++;
      }
      if (n1 < c.n_owned)
      {
        acc += val;
        count++;
      }
      if (n2 < c.n_owned)
      {
        acc += val;
        count++;
      }
      val = acc / (float)count;
    }
  }
  return to_d<float>(val);
}

// Face flux along D (ComputeHydroFluxesAndStoreFunctor.cpp:335-503) between the cells (i, j) of
// S-planes pL and pR (D = z) or the cells (i - 1, j) / (i, j - 1) and (i, j) of plane pR; normal B =
// t^n face value (bn) + the half-step source of the right cell. Writes the NFV fluxes * dt/dx.
template <class K, int D>
__device__ __forceinline__ void
col_flux(const ColView<K> & t, const ColCtx & c, int i, int j, int pR, float * out)
{
  constexpr int ivel = D == 0 ? IU : (D == 1 ? IV : IW);
  constexpr int imag = D == 0 ? IA : (D == 1 ? IB : IC);
  const int     iL = D == 0 ? i - 1 : i, jL = D == 1 ? j - 1 : j, pL = D == 2 ? pR - 1 : pR;
  const int     sR = K::sp(i, j), sL = K::sp(iL, jL);
  float         qL[8], qR[8], flux[8];
#pragma unroll
  for (int v = 0; v < 8; ++v)
  {
    qL[v] = t.Q2(pL, v)[sL] + 0.5f * t.Sl(pL, D, v)[sL];
    qR[v] = t.Q2(pR, v)[sR] + (-0.5f) * t.Sl(pR, D, v)[sR];
  }
  qL[ID] = rmax<float>(c.ph.smallr, qL[ID]);
  qL[IP] = rmax<float>(c.ph.smallp * qL[ID], qL[IP]);
  qR[ID] = rmax<float>(c.ph.smallr, qR[ID]);
  qR[IP] = rmax<float>(c.ph.smallp * qR[ID], qR[IP]);
  const float bn = t.template face<D>(i, j, pR, 0) + t.Sf(pR, D)[sR];
  qR[imag] = bn;
  qL[imag] = bn;
  if constexpr (D != 0)
  {
    float tmp;
    tmp = qL[IU]; qL[IU] = qL[ivel]; qL[ivel] = tmp;
    tmp = qR[IU]; qR[IU] = qR[ivel]; qR[ivel] = tmp;
    tmp = qL[IA]; qL[IA] = qL[imag]; qL[imag] = tmp;
    tmp = qR[IA]; qR[IA] = qR[imag]; qR[imag] = tmp;
  }
  riemann_mhd<float>(qL, qR, flux, c.ph);
  if constexpr (D != 0)
  {
    float tmp;
    tmp = flux[IU]; flux[IU] = flux[ivel]; flux[ivel] = tmp;
    tmp = flux[IA]; flux[IA] = flux[imag]; flux[imag] = tmp;
  }
#pragma unroll
  for (int v = 0; v < 5; ++v)
    out[v] = flux[v] * c.dtdx;
}

template <class K>
__global__ void __launch_bounds__(K::NT, 2) column_step_kernel(const StepArgs a)
{
  constexpr int TX = K::TX, TY = K::TY, NT = K::NT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ColView<K> t;
  t.sm = reinterpret_cast<float *>(smem_raw);
  __shared__ int          s_nbr[32];
  __shared__ unsigned int s_jump;
  __shared__ unsigned int s_health;
  __shared__ double       s_dx;
  __shared__ float        s_tr[3]; // dx, dt/dx, 1/dx (FP32)
  __shared__ float        s_red[NT / 32];

  const int tid = threadIdx.x;
  const int bx = a.bx, by = a.by, bz = a.bz;
  const int cols_x = bx / TX, cols_per_block = cols_x * (by / TY);
  const int n_work = (a.blk_list ? a.blk_count : a.n_owned) * cols_per_block;
  auto      cell_off = [](int c, int n) { return c < 0 ? -1 : (c >= n ? 1 : 0); };
  auto      face_off = [](int f, int n) { return f < 0 ? -1 : (f > n ? 1 : 0); };

  Phys<float> ph;
  ph.gamma0 = a.gamma0_f;
  ph.smallr = a.smallr_f;
  ph.smallc = a.smallc_f;
  ph.smallp = a.smallp_f;
  ph.slope_type = a.slope_type_f;
  ph.riemann = a.riemann;

  for (int work = blockIdx.x; work < n_work; work += gridDim.x)
  {
    const int blk = a.blk_list ? a.blk_list[work / cols_per_block] : work / cols_per_block;
    const int cidx = work % cols_per_block;
    const int x0 = (cidx % cols_x) * TX, y0 = (cidx / cols_x) * TY;
    if (tid < 32)
    {
      int  nb = -1;
      bool jump = false;
      if (tid < 27)
      {
        nb = a.neighbor[(int64_t)blk * 27 + tid];
        s_nbr[tid] = nb;
        jump = nb >= 0 && nb < a.n_blocks && a.level[nb] != a.level[blk];
      }
      const unsigned m = __ballot_sync(0xffffffffu, jump);
      if (tid == 0)
      {
        s_jump = m;
        s_health = 0u;
      }
    }
    const int    myprob = a.problem ? a.problem[blk] : 0;
    const double dt = a.dt_dev ? a.dt_dev[myprob] : a.dt;
    if (tid == 0)
    {
      const double dx0 = (1.0 / (double)((int64_t)bx << a.level[blk])) * a.scaling_factor;
      s_dx = dx0;
      s_tr[0] = (float)dx0;
      s_tr[1] = (float)(dt / dx0);
      s_tr[2] = (float)(1.0 / dx0);
    }
    __syncthreads();
    if (__double_as_longlong(dt) == (long long)0x8000000000000000ull)
    {
      // dt = -0: an earlier step has carried this finished problem over; both buffers hold its state
      __syncthreads();
      continue;
    }
    if (__double_as_longlong(dt) == 0)
    {
      // a problem that has reached its end time: carry the column over unchanged
      for (int n = tid; n < TX * TY * bz; n += NT)
      {
        const int     i = n % TX, j = (n / TX) % TY, k = n / (TX * TY);
        const int64_t cell = (x0 + i) + (int64_t)bx * ((y0 + j) + (int64_t)by * k);
        for (int v = 0; v < 5; ++v)
          a.U2[((int64_t)blk * 5 + v) * a.ncell + cell] = a.U[((int64_t)blk * 5 + v) * a.ncell + cell];
      }
      const int nxf = TX + (x0 + TX == bx ? 1 : 0), nyf = TY + (y0 + TY == by ? 1 : 0);
      const int64_t base = (int64_t)blk * a.nface;
      for (int n = tid; n < (nxf * TY + TX * nyf) * bz + TX * TY * (bz + 1); n += NT)
      {
        int64_t f;
        if (n < nxf * TY * bz)
        {
          const int i = n % nxf, j = (n / nxf) % TY, k = n / (nxf * TY);
          f = (x0 + i) + (int64_t)(bx + 1) * ((y0 + j) + (int64_t)by * k);
        }
        else if (n < (nxf * TY + TX * nyf) * bz)
        {
          const int m = n - nxf * TY * bz;
          const int i = m % TX, j = (m / TX) % nyf, k = m / (TX * nyf);
          f = a.nfx + (x0 + i) + (int64_t)bx * ((y0 + j) + (int64_t)(by + 1) * k);
        }
        else
        {
          const int m = n - (nxf * TY + TX * nyf) * bz;
          const int i = m % TX, j = (m / TX) % TY, k = m / (TX * TY);
          f = a.nfx + a.nfy + (x0 + i) + (int64_t)bx * ((y0 + j) + (int64_t)by * k);
        }
        a.B2[base + f] = a.B[base + f];
      }
      __syncthreads();
      continue;
    }

    ColCtx c;
    c.ph = ph;
    c.dx = s_dx;
    c.dxr = s_tr[0];
    c.dtdx = s_tr[1];
    c.idxr = s_tr[2];
    c.dt = dt;
    c.blk = blk;
    c.x0 = x0;
    c.y0 = y0;
    c.bx = bx;
    c.by = by;
    c.bz = bz;
    c.n_owned = a.n_owned;
    c.rk2 = a.rk2;
    c.nbr = s_nbr;
    const unsigned jump_mask = s_jump;
    unsigned int   health = 0u;
    float          my_invdt = 0.0f;

    // block of a block-local cell or face position, recording missing neighbours / level jumps
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
    const double * Bblk = a.B + (int64_t)blk * a.nface;
    double *       B2blk = a.B2 + (int64_t)blk * a.nface;
    const bool     ex = (x0 + TX == bx), ey = (y0 + TY == by);

    for (int s = -4; s <= bz + 1; ++s)
    {
      // ================= I1: edge E (plane s+1, level s+1), slopes + predictor (S-plane s),
      //                       CT update of output plane s-2 ==================================
      {
        // ---- edge electric field at t^n (ComputeElectricFieldFunctor.cpp:97-235)
        if (s >= -2 && s <= bz)
        {
          const bool do_ez = s + 1 <= bz;
          constexpr int NEZI = (TX + 3) * (TY + 3), NEXI = (TX + 2) * (TY + 3), NEYI = (TX + 3) * (TY + 2);
          const int     L = s + 1; // level of the x / y edges, plane of the z edges
          const float * QU1 = t.Q(L, IU), *QV1 = t.Q(L, IV), *QW1 = t.Q(L, IW);
          const float * QU0 = t.Q(L - 1, IU), *QV0 = t.Q(L - 1, IV), *QW0 = t.Q(L - 1, IW);
          const float * bxL = t.Bx(L), *byL = t.By(L), *bx0 = t.Bx(L - 1), *by0 = t.By(L - 1), *bzL = t.Bz(L);
          for (int m = tid; m < NEZI + NEXI + NEYI; m += NT)
          {
            if (m < NEZI)
            {
              if (!do_ez)
                continue;
              const int i = m % (TX + 3) - 1, j = m / (TX + 3) - 1;
              const float u = 0.25f * (QU1[K::qp(i - 1, j - 1)] + QU1[K::qp(i - 1, j)] + QU1[K::qp(i, j - 1)] + QU1[K::qp(i, j)]);
              const float v = 0.25f * (QV1[K::qp(i - 1, j - 1)] + QV1[K::qp(i - 1, j)] + QV1[K::qp(i, j - 1)] + QV1[K::qp(i, j)]);
              const float A = 0.5f * (bxL[K::bxp(i, j - 1)] + bxL[K::bxp(i, j)]);
              const float B = 0.5f * (byL[K::byp(i - 1, j)] + byL[K::byp(i, j)]);
              t.Ez(L)[K::ep(i, j)] = u * B - v * A;
            }
            else if (m < NEZI + NEXI)
            {
              const int n = m - NEZI;
              const int i = n % (TX + 2) - 1, j = n / (TX + 2) - 1;
              const float v = 0.25f * (QV0[K::qp(i, j - 1)] + QV1[K::qp(i, j - 1)] + QV0[K::qp(i, j)] + QV1[K::qp(i, j)]);
              const float w = 0.25f * (QW0[K::qp(i, j - 1)] + QW1[K::qp(i, j - 1)] + QW0[K::qp(i, j)] + QW1[K::qp(i, j)]);
              const float B = 0.5f * (by0[K::byp(i, j)] + byL[K::byp(i, j)]);
              const float Cc = 0.5f * (bzL[K::bzp(i, j - 1)] + bzL[K::bzp(i, j)]);
              t.Ex(L)[K::ep(i, j)] = v * Cc - w * B;
            }
            else
            {
              const int n = m - NEZI - NEXI;
              const int i = n % (TX + 3) - 1, j = n / (TX + 3) - 1;
              const float u = 0.25f * (QU0[K::qp(i - 1, j)] + QU1[K::qp(i - 1, j)] + QU0[K::qp(i, j)] + QU1[K::qp(i, j)]);
              const float w = 0.25f * (QW0[K::qp(i - 1, j)] + QW1[K::qp(i - 1, j)] + QW0[K::qp(i, j)] + QW1[K::qp(i, j)]);
              const float A = 0.5f * (bx0[K::bxp(i, j)] + bxL[K::bxp(i, j)]);
              const float Cc = 0.5f * (bzL[K::bzp(i - 1, j)] + bzL[K::bzp(i, j)]);
              t.Ey(L)[K::ep(i, j)] = w * A - u * Cc;
            }
          }
        }
        // ---- limited slopes + Hancock predictor of S-plane s (ComputeLimitedSlopesFunctor.cpp:121-314,
        //      ComputeUpdatedPrimitiveVariablesFunctor.cpp:284-546)
        if (s >= -1 && s <= bz)
        {
          const int p = s;
          const float st = ph.slope_type;
          for (int n = tid; n < K::NSP; n += NT)
          {
            const int i = n % K::SX - 1, j = n / K::SX - 1;
            const int q0 = K::qp(i, j), qxp = K::qp(i + 1, j), qxm = K::qp(i - 1, j), qyp = K::qp(i, j + 1),
                      qym = K::qp(i, j - 1);
            float dq[3][8];
#pragma unroll
            for (int v = 0; v < 5; ++v)
            {
              const float * Qc = t.Q(p, v);
              dq[0][v] = slope1<float>(Qc[q0], Qc[qxp], Qc[qxm], st);
              dq[1][v] = slope1<float>(Qc[q0], Qc[qyp], Qc[qym], st);
              dq[2][v] = slope1<float>(Qc[q0], t.Q(p + 1, v)[q0], t.Q(p - 1, v)[q0], st);
            }
            const float * BXc = t.Bx(p), *BYc = t.By(p);
            const float   AL = BXc[K::bxp(i, j)], AR = BXc[K::bxp(i + 1, j)];
            const float   BL = BYc[K::byp(i, j)], BR = BYc[K::byp(i, j + 1)];
            const float   CL = t.Bz(p)[K::bzp(i, j)], CR = t.Bz(p + 1)[K::bzp(i, j)];
            auto avgA = [&](int ii, int jj, int pp) {
              return (t.Bx(pp)[K::bxp(ii, jj)] + t.Bx(pp)[K::bxp(ii + 1, jj)]) * 0.5f;
            };
            auto avgB = [&](int ii, int jj, int pp) {
              return (t.By(pp)[K::byp(ii, jj)] + t.By(pp)[K::byp(ii, jj + 1)]) * 0.5f;
            };
            auto avgC = [&](int ii, int jj, int pp) {
              return (t.Bz(pp)[K::bzp(ii, jj)] + t.Bz(pp + 1)[K::bzp(ii, jj)]) * 0.5f;
            };
            dq[0][IA] = AR - AL;
            dq[1][IA] = slope1<float>(avgA(i, j, p), avgA(i, j + 1, p), avgA(i, j - 1, p), st);
            dq[0][IB] = slope1<float>(avgB(i, j, p), avgB(i + 1, j, p), avgB(i - 1, j, p), st);
            dq[1][IB] = BR - BL;
            dq[0][IC] = slope1<float>(avgC(i, j, p), avgC(i + 1, j, p), avgC(i - 1, j, p), st);
            dq[1][IC] = slope1<float>(avgC(i, j, p), avgC(i, j + 1, p), avgC(i, j - 1, p), st);
            dq[2][IA] = slope1<float>(avgA(i, j, p), avgA(i, j, p + 1), avgA(i, j, p - 1), st);
            dq[2][IB] = slope1<float>(avgB(i, j, p), avgB(i, j, p + 1), avgB(i, j, p - 1), st);
            dq[2][IC] = CR - CL;
#pragma unroll
            for (int d = 0; d < 3; ++d)
#pragma unroll
              for (int v = 0; v < 8; ++v)
                t.Sl(p, d, v)[n] = dq[d][v];

            const float r = t.Q(p, ID)[q0], pr = t.Q(p, IP)[q0], u = t.Q(p, IU)[q0], v = t.Q(p, IV)[q0],
                        w = t.Q(p, IW)[q0];
            const float A = (AL + AR) * 0.5f, B = (BL + BR) * 0.5f, Cc = (CL + CR) * 0.5f;
            float *     Q2 = t.Q2(p, 0);
            if (a.rk2)
            {
              Q2[ID * K::NSP + n] = r;
              Q2[IU * K::NSP + n] = u;
              Q2[IV * K::NSP + n] = v;
              Q2[IW * K::NSP + n] = w;
              Q2[IP * K::NSP + n] = pr;
              Q2[IA * K::NSP + n] = A;
              Q2[IB * K::NSP + n] = B;
              Q2[IC * K::NSP + n] = Cc;
              continue;
            }
            const float gamma = ph.gamma0;
            const float dtdx = c.dtdx, dtdy = dtdx, dtdz = dtdx;
            const float drx = dq[0][ID], dpx = dq[0][IP], dux = dq[0][IU], dvx = dq[0][IV], dwx = dq[0][IW],
                        dAx = dq[0][IA], dBx = dq[0][IB], dCx = dq[0][IC];
            const float dry = dq[1][ID], dpy = dq[1][IP], duy = dq[1][IU], dvy = dq[1][IV], dwy = dq[1][IW],
                        dAy = dq[1][IA], dBy = dq[1][IB], dCy = dq[1][IC];
            const float drz = dq[2][ID], dpz = dq[2][IP], duz = dq[2][IU], dvz = dq[2][IV], dwz = dq[2][IW],
                        dAz = dq[2][IA], dBz = dq[2][IB], dCz = dq[2][IC];
            const float sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy + (-w * drz - dwz * r) * dtdz;
            const float su0 = (-u * dux - (dpx + B * dBx + Cc * dCx) / r) * dtdx + (-v * duy + B * dAy / r) * dtdy +
                              (-w * duz + Cc * dAz / r) * dtdz;
            const float sv0 = (-u * dvx + A * dBx / r) * dtdx + (-v * dvy - (dpy + A * dAy + Cc * dCy) / r) * dtdy +
                              (-w * dvz + Cc * dBz / r) * dtdz;
            const float sw0 = (-u * dwx + A * dCx / r) * dtdx + (-v * dwy + B * dCy / r) * dtdy +
                              (-w * dwz - (dpz + A * dAz + B * dBz) / r) * dtdz;
            const float sp0 = (-u * dpx - dux * gamma * pr) * dtdx + (-v * dpy - dvy * gamma * pr) * dtdy +
                              (-w * dpz - dwz * gamma * pr) * dtdz;
            const float sA0 = (u * dBy + B * duy - v * dAy - A * dvy) * dtdy + (u * dCz + Cc * duz - w * dAz - A * dwz) * dtdz;
            const float sB0 = (v * dAx + A * dvx - u * dBx - B * dux) * dtdx + (v * dCz + Cc * dvz - w * dBz - B * dwz) * dtdz;
            const float sC0 = (w * dAx + A * dwx - u * dCx - Cc * dux) * dtdx + (w * dBy + B * dwy - v * dCy - Cc * dvy) * dtdy;
            float ug = u, vg = v, wg = w;
            if (a.src.gravity)
            {
              const float hdt = (float)dt;
              ug += (float)a.src.g[0] * 0.5f * hdt;
              vg += (float)a.src.g[1] * 0.5f * hdt;
              wg += (float)a.src.g[2] * 0.5f * hdt;
            }
            Q2[ID * K::NSP + n] = r + 0.5f * sr0;
            Q2[IU * K::NSP + n] = ug + 0.5f * su0;
            Q2[IV * K::NSP + n] = vg + 0.5f * sv0;
            Q2[IW * K::NSP + n] = wg + 0.5f * sw0;
            Q2[IP * K::NSP + n] = pr + 0.5f * sp0;
            Q2[IA * K::NSP + n] = A + 0.5f * sA0;
            Q2[IB * K::NSP + n] = B + 0.5f * sB0;
            Q2[IC * K::NSP + n] = Cc + 0.5f * sC0;
          }
        }
        // ---- CT update of output plane s-2 (ReadEmfAndUpdateFunctor.cpp:58-163): Bx, By of the plane
        //      and Bz of its top level (plane 0 also its bottom level)
        if (s >= 2)
        {
          const int p = s - 2;
          const double * Mz = t.Mz();
          const double * My0 = t.My(p), *My1 = t.My(p + 1), *Mx0 = t.Mx(p), *Mx1 = t.Mx(p + 1);
          constexpr int  NBX = (TX + 1) * TY, NBY = TX * (TY + 1), NBZ = TX * TY;
          const int      nz = p == 0 ? 2 * NBZ : NBZ;
          for (int m = tid; m < NBX + NBY + nz; m += NT)
          {
            double  bnew;
            int64_t fg;
            bool    owned;
            if (m < NBX)
            {
              const int i = m % (TX + 1), j = m / (TX + 1);
              fg = (x0 + i) + (int64_t)(bx + 1) * ((y0 + j) + (int64_t)by * p);
              const double d = curl2<false>(Mz[i + (TX + 1) * (j + 1)] - Mz[i + (TX + 1) * j],
                                            My1[i + (TX + 1) * j] - My0[i + (TX + 1) * j]);
              bnew = Bblk[fg] + d;
              owned = i < TX || ex;
              t.Nx()[m] = to_r<float>(bnew);
            }
            else if (m < NBX + NBY)
            {
              const int n = m - NBX;
              const int i = n % TX, j = n / TX;
              fg = a.nfx + (x0 + i) + (int64_t)bx * ((y0 + j) + (int64_t)(by + 1) * p);
              const double d =
                curl2<false>(Mx1[i + TX * j] - Mx0[i + TX * j], Mz[(i + 1) + (TX + 1) * j] - Mz[i + (TX + 1) * j]);
              bnew = Bblk[fg] + d;
              owned = j < TY || ey;
              t.Ny()[n] = to_r<float>(bnew);
            }
            else
            {
              int       n = m - NBX - NBY;
              const int L = n < NBZ ? p + 1 : 0; // top level of the plane; plane 0 also level 0
              n = n < NBZ ? n : n - NBZ;
              const int i = n % TX, j = n / TX;
              const double * MxL = t.Mx(L), *MyL = t.My(L);
              fg = a.nfx + a.nfy + (x0 + i) + (int64_t)bx * ((y0 + j) + (int64_t)by * L);
              const double d = curl2<false>(MyL[(i + 1) + (TX + 1) * j] - MyL[i + (TX + 1) * j],
                                            MxL[i + TX * (j + 1)] - MxL[i + TX * j]);
              bnew = Bblk[fg] + d;
              owned = true;
              t.Nz(L)[n] = to_r<float>(bnew);
            }
            if (owned)
              B2blk[fg] = bnew;
          }
        }
      }
      __syncthreads();

      // ================= I2: face source (S-plane s), primitives of Q-plane s+2, conservative update
      //                       + CFL of output plane s-2 =================================================
      {
        // ---- half-step face-B source (ComputeSourceFaceMagFunctor.cpp:114-203)
        if (s >= -1 && s <= bz)
        {
          const int     p = s;
          const float   h = 0.5f * c.dtdx;
          const float * Ez = t.Ez(p), *Ex0 = t.Ex(p), *Ex1 = t.Ex(p + 1), *Ey0 = t.Ey(p), *Ey1 = t.Ey(p + 1);
          for (int n = tid; n < K::NSP; n += NT)
          {
            const int i = n % K::SX - 1, j = n / K::SX - 1;
            t.Sf(p, 0)[n] = (Ez[K::ep(i, j + 1)] - Ez[K::ep(i, j)]) * 0.5f * c.dtdx -
                            (Ey1[K::ep(i, j)] - Ey0[K::ep(i, j)]) * 0.5f * c.dtdx;
            t.Sf(p, 1)[n] = -(Ez[K::ep(i + 1, j)] - Ez[K::ep(i, j)]) * 0.5f * c.dtdx +
                            (Ex1[K::ep(i, j)] - Ex0[K::ep(i, j)]) * 0.5f * c.dtdx;
            t.Sf(p, 2)[n] = (Ey0[K::ep(i + 1, j)] - Ey0[K::ep(i, j)]) * 0.5f * c.dtdx -
                            (Ex0[K::ep(i, j + 1)] - Ex0[K::ep(i, j)]) * 0.5f * c.dtdx;
          }
          (void)h;
        }
        // ---- primitives of Q-plane s+2 from U, B in global memory; its t^n faces to FP32
        //      (ConvertToPrimitivesVariablesFunctor.cpp:173-719, models/mhd_utils.h:449-515)
        if (s <= bz - 1)
        {
          const int q = s + 2;
          float *   fx = t.Bx(q), *fy = t.By(q), *fzt = t.Bz(q + 1);
          constexpr int NPRIM = K::NQP, NXE = K::QY, NYE = K::QX;
          for (int m = tid; m < NPRIM + NXE + NYE; m += NT)
          {
            if (m >= NPRIM)
            {
              // the last x-face column and y-face row of the plane
              int i, j, comp;
              if (m < NPRIM + NXE)
              {
                i = TX + 2;
                j = m - NPRIM - 2;
                comp = 0;
              }
              else
              {
                i = m - NPRIM - NXE - 2;
                j = TY + 2;
                comp = 1;
              }
              const int gi = x0 + i, gj = y0 + j;
              const int ox = comp == 0 ? face_off(gi, bx) : cell_off(gi, bx);
              const int oy = comp == 0 ? cell_off(gj, by) : face_off(gj, by);
              const int oz = cell_off(q, bz);
              const int nb = owner(ox, oy, oz);
              double    val = 0.0;
              if (nb >= 0)
              {
                const double * Bn = a.B + (int64_t)nb * a.nface;
                const int      li = gi - ox * bx, lj = gj - oy * by, lk = q - oz * bz;
                val = comp == 0 ? Bn[li + (int64_t)(bx + 1) * (lj + (int64_t)by * lk)]
                                : Bn[a.nfx + li + (int64_t)bx * (lj + (int64_t)(by + 1) * lk)];
              }
              if (comp == 0)
                fx[K::bxp(i, j)] = to_r<float>(val);
              else
                fy[K::byp(i, j)] = to_r<float>(val);
              continue;
            }
            const int i = m % K::QX - 2, j = m / K::QX - 2;
            const int gi = x0 + i, gj = y0 + j;
            const int cox = cell_off(gi, bx), coy = cell_off(gj, by), coz = cell_off(q, bz);
            // the cell's six faces, each read from the block that owns that face index
            double bxl = 0.0, bxr = 0.0, byl = 0.0, byr = 0.0, bzl = 0.0, bzr = 0.0;
            {
              const int o0 = face_off(gi, bx), o1 = face_off(gi + 1, bx);
              const int n0 = owner(o0, coy, coz), n1 = owner(o1, coy, coz);
              const int64_t tr = (int64_t)(bx + 1) * ((gj - coy * by) + (int64_t)by * (q - coz * bz));
              if (n0 >= 0)
                bxl = a.B[(int64_t)n0 * a.nface + (gi - o0 * bx) + tr];
              if (n1 >= 0)
                bxr = a.B[(int64_t)n1 * a.nface + (gi + 1 - o1 * bx) + tr];
            }
            {
              const int o0 = face_off(gj, by), o1 = face_off(gj + 1, by);
              const int n0 = owner(cox, o0, coz), n1 = owner(cox, o1, coz);
              const int64_t base = a.nfx + (gi - cox * bx);
              const int64_t zk = (int64_t)(by + 1) * (q - coz * bz);
              if (n0 >= 0)
                byl = a.B[(int64_t)n0 * a.nface + base + (int64_t)bx * ((gj - o0 * by) + zk)];
              if (n1 >= 0)
                byr = a.B[(int64_t)n1 * a.nface + base + (int64_t)bx * ((gj + 1 - o1 * by) + zk)];
            }
            {
              const int o0 = face_off(q, bz), o1 = face_off(q + 1, bz);
              const int n0 = owner(cox, coy, o0), n1 = owner(cox, coy, o1);
              const int64_t base = a.nfx + a.nfy + (gi - cox * bx) + (int64_t)bx * (gj - coy * by);
              if (n0 >= 0)
                bzl = a.B[(int64_t)n0 * a.nface + base + (int64_t)bx * by * (q - o0 * bz)];
              if (n1 >= 0)
                bzr = a.B[(int64_t)n1 * a.nface + base + (int64_t)bx * by * (q + 1 - o1 * bz)];
            }
            double u[5] = {1.0, 1.0, 0.0, 0.0, 0.0};
            const int nb = owner(cox, coy, coz);
            if (nb >= 0)
            {
              const double * Ub = a.U + (int64_t)nb * 5 * a.ncell + (gi - cox * bx) +
                                  (int64_t)bx * ((gj - coy * by) + (int64_t)by * (q - coz * bz));
#pragma unroll
              for (int v = 0; v < 5; ++v)
                u[v] = Ub[(int64_t)v * a.ncell];
            }
            const float fxl = to_r<float>(bxl), fxr = to_r<float>(bxr), fyl = to_r<float>(byl),
                        fyr = to_r<float>(byr), fzl = to_r<float>(bzl), fzr = to_r<float>(bzr);
            fx[K::bxp(i, j)] = fxl;
            fy[K::byp(i, j)] = fyl;
            fzt[K::bzp(i, j)] = fzr;
            if (s == -4)
              t.Bz(q)[K::bzp(i, j)] = fzl; // the first plane's bottom faces
            // a cell inside an outside block takes its cell-centred B from that block's own faces
            // (get_conservative_vars of the outside cell; FillOutside's copy of the shared border face)
            if (nb >= a.n_owned && nb < a.n_blocks)
            {
              const int      li = gi - cox * bx, lj = gj - coy * by, lk = q - coz * bz;
              const double * Bn = a.B + (int64_t)nb * a.nface;
              const int64_t  xr = li + (int64_t)(bx + 1) * (lj + (int64_t)by * lk);
              const int64_t  yr = a.nfx + li + (int64_t)bx * (lj + (int64_t)(by + 1) * lk);
              const int64_t  zr = a.nfx + a.nfy + li + (int64_t)bx * (lj + (int64_t)by * lk);
              bxl = Bn[xr];
              bxr = Bn[xr + 1];
              byl = Bn[yr];
              byr = Bn[yr + bx];
              bzl = Bn[zr];
              bzr = Bn[zr + (int64_t)bx * by];
            }
            // FP32 recovery; FP64 when magnetic + kinetic energy dominate (low beta / high Mach)
            const float Bxc = 0.5f * (to_r<float>(bxl) + to_r<float>(bxr)),
                        Byc = 0.5f * (to_r<float>(byl) + to_r<float>(byr)),
                        Bzc = 0.5f * (to_r<float>(bzl) + to_r<float>(bzr));
            const float r = rmax<float>(to_r<float>(u[ID]), ph.smallr);
            const float ir = 1.0f / r;
            const float vx = to_r<float>(u[IU]) * ir, vy = to_r<float>(u[IV]) * ir, vz = to_r<float>(u[IW]) * ir;
            const float ekin = 0.5f * r * (vx * vx + vy * vy + vz * vz);
            const float emag = 0.5f * (Bxc * Bxc + Byc * Byc + Bzc * Bzc);
            float       pr = (ph.gamma0 - 1.0f) * (to_r<float>(u[IP]) - emag - ekin);
            if (ekin + emag > 4.0f * pr * (1.0f / (ph.gamma0 - 1.0f)))
            {
              const double Bx2 = 0.5 * (bxl + bxr), By2 = 0.5 * (byl + byr), Bz2 = 0.5 * (bzl + bzr);
              const double rd = fmax(u[ID], a.smallr);
              const double emag_d = 0.5 * (Bx2 * Bx2 + By2 * By2 + Bz2 * Bz2);
              const double ekin_d = 0.5 * (u[IU] * u[IU] + u[IV] * u[IV] + u[IW] * u[IW]) / rd;
              pr = (float)((a.gamma0 - 1.0) * (u[IP] - emag_d - ekin_d));
              health |= HEALTH_LOW_BETA_FP64;
            }
            pr = rmax<float>(pr, r * ph.smallp);
            const int qn = K::qp(i, j);
            t.Q(q, ID)[qn] = r;
            t.Q(q, IP)[qn] = pr;
            t.Q(q, IU)[qn] = vx;
            t.Q(q, IV)[qn] = vy;
            t.Q(q, IW)[qn] = vz;
          }
        }
        // ---- conservative update + CFL of output plane s-2 (ReadFluxesAndConservativeUpdateFunctor.cpp:
        //      240-436, AddGravitySourceTerm.cpp:47-99, ComputeDtMHDFunctor.cpp:86-151)
        if (s >= 2)
        {
          const int p = s - 2;
          for (int n = tid; n < TX * TY; n += NT)
          {
            const int     i = n % TX, j = n / TX;
            const int64_t cell = (x0 + i) + (int64_t)bx * ((y0 + j) + (int64_t)by * p);
            double        u2[5];
#pragma unroll
            for (int v = 0; v < 5; ++v)
              u2[v] = a.U[((int64_t)blk * 5 + v) * a.ncell + cell];
            const double rho_old = u2[ID];
            const int    fxL = i + (TX + 1) * j, fyL = i + TX * j, fz = i + TX * j;
#pragma unroll
            for (int v = 0; v < 5; ++v)
            {
              float ds = t.Fx(v)[fxL], de = 0.0f;
              two_sum_acc(ds, de, -t.Fx(v)[fxL + 1]);
              two_sum_acc(ds, de, t.Fy(v)[fyL]);
              two_sum_acc(ds, de, -t.Fy(v)[fyL + TX]);
              two_sum_acc(ds, de, t.Fz(p, v)[fz]);
              two_sum_acc(ds, de, -t.Fz(p + 1, v)[fz]);
              u2[v] = (u2[v] + to_d<float>(ds)) + to_d<float>(de);
            }
            if (a.src.gravity)
            {
              const double rho_new = u2[ID];
              double       ru = u2[IU], rv = u2[IV], rw = u2[IW];
              double       ekin_old = 0.5 * (ru * ru + rv * rv) / rho_new;
              ekin_old += 0.5 * (rw * rw) / rho_new;
              ru += dt * a.src.g[0] * (rho_old + rho_new) / 2;
              rv += dt * a.src.g[1] * (rho_old + rho_new) / 2;
              rw += dt * a.src.g[2] * (rho_old + rho_new) / 2;
              u2[IU] = ru;
              u2[IV] = rv;
              u2[IW] = rw;
              double ekin_new = 0.5 * (ru * ru + rv * rv) / rho_new;
              ekin_new += 0.5 * (rw * rw) / rho_new;
              u2[IP] += (ekin_new - ekin_old);
            }
#pragma unroll
            for (int v = 0; v < 5; ++v)
              a.U2[((int64_t)blk * 5 + v) * a.ncell + cell] = u2[v];
            {
              const long long bd = __double_as_longlong(u2[ID]);
              if (!(bd > 0 && bd <= 0x7ff0000000000000LL))
                health |= HEALTH_BAD_DENSITY;
              const long long exm = 0x7ff0000000000000LL;
              if ((__double_as_longlong(u2[IP]) & exm) == exm || (__double_as_longlong(u2[IU]) & exm) == exm)
                health |= HEALTH_NONFINITE;
            }
            if (a.invdt_out)
            {
              const float Axl = t.Nx()[i + (TX + 1) * j], Axr = t.Nx()[i + 1 + (TX + 1) * j];
              const float Ayl = t.Ny()[i + TX * j], Ayr = t.Ny()[i + TX * (j + 1)];
              const float bxf = 0.5f * (Axl + Axr);
              const float byf = 0.5f * (Ayl + Ayr);
              const float bzf = 0.5f * (t.Nz(p)[fz] + t.Nz(p + 1)[fz]);
              const float r = fmaxf(to_r<float>(u2[ID]), ph.smallr);
              const float ir = 1.0f / r;
              const float vx = to_r<float>(u2[IU]) * ir, vy = to_r<float>(u2[IV]) * ir, vz = to_r<float>(u2[IW]) * ir;
              const float ekin = 0.5f * r * (vx * vx + vy * vy + vz * vz);
              const float emag = 0.5f * (bxf * bxf + byf * byf + bzf * bzf);
              const float g = ph.gamma0;
              const float pr = fmaxf((g - 1.0f) * (to_r<float>(u2[IP]) - emag - ekin), r * ph.smallp);
              const float b2 = 2.0f * emag;
              const float c2 = g * pr * ir;
              const float d2 = 0.5f * (b2 * ir + c2);
              const float cfx = sqrtf(d2 + sqrtf(fmaxf(d2 * d2 - c2 * bxf * bxf * ir, 0.0f))) + fabsf(vx);
              const float cfy = sqrtf(d2 + sqrtf(fmaxf(d2 * d2 - c2 * byf * byf * ir, 0.0f))) + fabsf(vy);
              const float cfz = sqrtf(d2 + sqrtf(fmaxf(d2 * d2 - c2 * bzf * bzf * ir, 0.0f))) + fabsf(vz);
              my_invdt = fmaxf(my_invdt, cfl_inv_dt_fp32(3, cfx, cfy, cfz, c.dxr, c.idxr, to_r<float>(u2[ID]), a.src));
            }
          }
        }
      }
      __syncthreads();

      // ================= I3: EMFs and face fluxes (ComputeEmfAndStoreFunctor.cpp:371-590,
      //                       ComputeHydroFluxesAndStoreFunctor.cpp:335-503) ===========================
      if (s >= 0 && s <= bz)
      {
        const int     L = s, p = s - 1;
        const bool    plane = s >= 1; // plane s-1 exists (z edges, x / y fluxes)
        constexpr int NMZI = K::NMZ, NMXI = K::NMX, NMYI = K::NMY, NFZI = K::NFZ, NFXI = K::NFX, NFYI = K::NFY;
        // one list: z edges, x edges, y edges, z fluxes, x fluxes, y fluxes
        constexpr int E0 = NMZI, E1 = E0 + NMXI, E2 = E1 + NMYI, E3 = E2 + NFZI, E4 = E3 + NFXI, E5 = E4 + NFYI;
        for (int m = tid; m < E5; m += NT)
        {
          if (m < E0)
          {
            if (!plane)
              continue;
            const int i = m % (TX + 1), j = m / (TX + 1);
            t.Mz()[m] = col_edge<K, 2>(t, c, i, j, p);
          }
          else if (m < E1)
          {
            const int n = m - E0;
            const int i = n % TX, j = n / TX;
            t.Mx(L)[n] = col_edge<K, 0>(t, c, i, j, L);
          }
          else if (m < E2)
          {
            const int n = m - E1;
            const int i = n % (TX + 1), j = n / (TX + 1);
            t.My(L)[n] = col_edge<K, 1>(t, c, i, j, L);
          }
          else if (m < E3)
          {
            const int n = m - E2;
            const int i = n % TX, j = n / TX;
            float     f[5];
            col_flux<K, 2>(t, c, i, j, L, f);
#pragma unroll
            for (int v = 0; v < 5; ++v)
              t.Fz(L, v)[n] = f[v];
          }
          else if (m < E4)
          {
            if (!plane)
              continue;
            const int n = m - E3;
            const int i = n % (TX + 1), j = n / (TX + 1);
            float     f[5];
            col_flux<K, 0>(t, c, i, j, p, f);
#pragma unroll
            for (int v = 0; v < 5; ++v)
              t.Fx(v)[n] = f[v];
          }
          else
          {
            if (!plane)
              continue;
            const int n = m - E4;
            const int i = n % TX, j = n / TX;
            float     f[5];
            col_flux<K, 1>(t, c, i, j, p, f);
#pragma unroll
            for (int v = 0; v < 5; ++v)
              t.Fy(v)[n] = f[v];
          }
        }
      }
      __syncthreads();
    } // plane steps

    // column epilogue: CFL maximum and health flags
    if (health)
      atomicOr(&s_health, health);
    if (a.invdt_out)
    {
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
        my_invdt = fmaxf(my_invdt, __shfl_xor_sync(0xffffffffu, my_invdt, off));
      if ((tid & 31) == 0)
        s_red[tid >> 5] = my_invdt;
    }
    __syncthreads();
    if (tid == 0)
    {
      if (a.invdt_out)
      {
        float mf = s_red[0];
        for (int w = 1; w < NT / 32; ++w)
          mf = fmaxf(mf, s_red[w]);
        atomic_max_pos_double(&a.invdt_out[myprob], f2d_bits(mf));
      }
      if (s_health)
        atomicOr(a.health, s_health);
    }
    __syncthreads();
  } // columns
}

} // namespace gmhd

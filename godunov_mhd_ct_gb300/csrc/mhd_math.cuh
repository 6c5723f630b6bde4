// Per-cell MHD math on the device, templated on the compute type R (double or float).
//
// Same operand order as godunov_mhd_ct's models/mhd_utils.h and models/RiemannSolvers_MHD.h, so
// that the double instantiation, compiled with --fmad=false, gives the same bits as an FP64 host
// build of the reference formulas. Citations are to those files.
#pragma once

#include <cstdint>
#include <type_traits>

namespace gmhd
{

// Variable slots (models/MHD.h:35-62): ID, IP, IU, IV, IW, IA, IB, IC.
enum : int
{
  ID = 0,
  IP = 1,
  IU = 2,
  IV = 3,
  IW = 4,
  IA = 5,
  IB = 6,
  IC = 7
};

// Riemann solver ids (models/riemann_solver_types.h:26-37).
enum : int
{
  RS_LLF = 2,
  RS_HLL = 3,
  RS_HLLC = 4,
  RS_HLLD = 5
};

// Source terms of the step (all off by default): uniform gravity and viscosity.
struct Sources
{
  int    gravity;        // [gravity] enabled
  double g[3];           // [gravity] uniform_gx, uniform_gy, uniform_gz
  int    viscosity;      // [viscosity] enabled
  double mu;             // [viscosity] mu
  int    visc_predictor; // viscous term of the Hancock predictor
};

// One cell's 1/dt from its fast speeds v_d = c_f,d + |u_d| (ComputeDtMHDFunctor.cpp:86-151): sum of
// v_d / dx; with gravity each term is scaled by k / (sqrt(1 + 2k) - 1), k = sum|g| dx / sum v_d^2
// floored at 1e-4 (:155-249); with viscosity at least 4 nu / dx^2, nu = mu / rho of the conservative
// density (:144-148). FP64 with the reference's operand order.
__device__ __forceinline__ double
cfl_inv_dt_fp64(int dim, double vx, double vy, double vz, double dx, double rho, const Sources & s)
{
  double val;
  if (s.gravity)
  {
    double v2 = vx * vx + vy * vy;
    if (dim == 3)
      v2 += vz * vz;
    double k = fabs(s.g[0]) + fabs(s.g[1]);
    if (dim == 3)
      k += fabs(s.g[2]);
    k *= dx / v2;
    k = fmax(k, 1e-4);
    const double factor = k / (sqrt(1.0 + 2.0 * k) - 1.0);
    val = 0.0;
    val += (vx * factor) / dx;
    val += (vy * factor) / dx;
    if (dim == 3)
      val += (vz * factor) / dx;
  }
  else
    val = dim == 3 ? vx / dx + vy / dx + vz / dx : vx / dx + vy / dx;
  if (s.viscosity)
  {
    const double nu = s.mu / rho;
    val = fmax(val, 4 * nu / (dx * dx));
  }
  return val;
}

// compute_cfl (scheme/ComputeDtMHDFunctor.cpp:86-151) of cell (i, j, k) of one block in the C-ABI
// layout, FP64 with the reference operand order: face B averaged to the cell centre, primitive
// recovery (models/mhd_utils.h:449-515), fast speeds (find_speed_info, :340-394), then
// cfl_inv_dt_fp64. Ub / Bb point at the block's U and face arrays; c is the cell's index in the block.
// Units that call it are compiled with --fmad=false, so every caller gets the same bits.
__device__ __forceinline__ double
cell_inv_dt_fp64(const double * __restrict__ Ub, const double * __restrict__ Bb, int dim, int bx, int by, int i,
                 int j, int k, int64_t c, int64_t ncell, int64_t nfx, int64_t nfy, double dx, double gamma0,
                 double smallr, double smallp, const Sources & src)
{
  const double Ax = 0.5 * (Bb[i + (int64_t)(bx + 1) * (j + (int64_t)by * k)] +
                           Bb[i + 1 + (int64_t)(bx + 1) * (j + (int64_t)by * k)]);
  const double Ay = 0.5 * (Bb[nfx + i + (int64_t)bx * (j + (int64_t)(by + 1) * k)] +
                           Bb[nfx + i + (int64_t)bx * (j + 1 + (int64_t)(by + 1) * k)]);
  double Az;
  if (dim == 3)
    Az = 0.5 * (Bb[nfx + nfy + i + (int64_t)bx * (j + (int64_t)by * k)] +
                Bb[nfx + nfy + i + (int64_t)bx * (j + (int64_t)by * (k + 1))]);
  else
    Az = 0.5 * (Bb[nfx + nfy + c] + Bb[nfx + nfy + c]);
  const double r = fmax(Ub[c], smallr);
  const double vx = Ub[2 * ncell + c] / r, vy = Ub[3 * ncell + c] / r, vz = Ub[4 * ncell + c] / r;
  const double eken = 0.5 * (vx * vx + vy * vy + vz * vz);
  const double emag = 0.5 * (Ax * Ax + Ay * Ay + Az * Az);
  const double eint = (Ub[ncell + c] - emag) / r - eken;
  const double p = fmax((gamma0 - 1.0) * r * eint, r * smallp);
  const double b2 = Ax * Ax + Ay * Ay + Az * Az;
  const double c2 = gamma0 * p / r;
  const double d2 = 0.5 * (b2 / r + c2);
  const double cfx = sqrt(d2 + sqrt(d2 * d2 - c2 * Ax * Ax / r)) + fabs(vx);
  const double cfy = sqrt(d2 + sqrt(d2 * d2 - c2 * Ay * Ay / r)) + fabs(vy);
  const double cfz = dim == 3 ? sqrt(d2 + sqrt(d2 * d2 - c2 * Az * Az / r)) + fabs(vz) : 0.0;
  return cfl_inv_dt_fp64(dim, cfx, cfy, cfz, dx, Ub[c], src);
}

// FP32 estimate of cfl_inv_dt_fp64 for the mixed path. The gravity factor is evaluated as
// (sqrt(1 + 2k) + 1) / 2, equal to k / (sqrt(1 + 2k) - 1) but without its cancellation at small k.
__device__ __forceinline__ float
cfl_inv_dt_fp32(int dim, float vx, float vy, float vz, float dx, float idx, float rho, const Sources & s)
{
  float sum = vx + vy;
  if (dim == 3)
    sum += vz;
  if (s.gravity)
  {
    float v2 = vx * vx + vy * vy;
    if (dim == 3)
      v2 += vz * vz;
    float gs = fabsf((float)s.g[0]) + fabsf((float)s.g[1]);
    if (dim == 3)
      gs += fabsf((float)s.g[2]);
    const float k = fmaxf(gs * dx / v2, 1e-4f);
    sum *= 0.5f * (sqrtf(1.0f + 2.0f * k) + 1.0f);
  }
  float val = sum * idx;
  if (s.viscosity)
    val = fmaxf(val, 4.0f * ((float)s.mu / rho) * idx * idx);
  return val;
}

template <typename R>
struct Phys
{
  R   gamma0;
  R   smallr;
  R   smallc;
  R   smallp;
  R   slope_type;
  int riemann;
};

template <typename R>
__device__ __forceinline__ R
dsqrt(R x)
{
  return sqrt(x);
}
template <>
__device__ __forceinline__ float
dsqrt<float>(float x)
{
  return sqrtf(x);
}

template <typename R>
__device__ __forceinline__ R
rmax(R a, R b)
{
  return fmax(a, b);
}
template <>
__device__ __forceinline__ float
rmax<float>(float a, float b)
{
  return fmaxf(a, b);
}
template <typename R>
__device__ __forceinline__ R
rmin(R a, R b)
{
  return fmin(a, b);
}
template <>
__device__ __forceinline__ float
rmin<float>(float a, float b)
{
  return fminf(a, b);
}
template <typename R>
__device__ __forceinline__ R
rabs(R a)
{
  return fabs(a);
}
template <>
__device__ __forceinline__ float
rabs<float>(float a)
{
  return fabsf(a);
}
template <typename R>
__device__ __forceinline__ R
rcopysign(R a, R b)
{
  return copysign(a, b);
}
template <>
__device__ __forceinline__ float
rcopysign<float>(float a, float b)
{
  return copysignf(a, b);
}

// Divisions that share a divisor. FP64 keeps the reference's x / y (bit-exact parity); the FP32
// path multiplies by one reciprocal inv = recip(y) computed for all of them (unused, and removed,
// on the FP64 path).
template <typename R>
__device__ __forceinline__ R
recip(R y)
{
  return R(1) / y;
}
template <typename R>
__device__ __forceinline__ R
qdiv(R x, R y, R inv)
{
  (void)inv;
  return x / y;
}
template <>
__device__ __forceinline__ float
qdiv<float>(float x, float y, float inv)
{
  (void)y;
  return x * inv;
}
// x / sqrt(r): FP64 as written, FP32 as x * rsqrt(r)
template <typename R>
__device__ __forceinline__ R
div_sqrt(R x, R r)
{
  return x / dsqrt<R>(r);
}
template <>
__device__ __forceinline__ float
div_sqrt<float>(float x, float r)
{
  return x * rsqrtf(r);
}

// find_speed_fast<dir> (models/mhd_utils.h:93-122)
template <typename R>
__device__ __forceinline__ R
speed_fast(const R * q, int dir, const Phys<R> & s)
{
  const R d = q[ID], p = q[IP], a = q[IA], b = q[IB], c = q[IC];
  const R id = recip<R>(d);
  const R b2 = a * a + b * b + c * c;
  const R c2 = qdiv<R>(s.gamma0 * p, d, id);
  const R d2 = R(0.5) * (qdiv<R>(b2, d, id) + c2);
  const R bn = dir == 0 ? a : (dir == 1 ? b : c);
  return dsqrt<R>(d2 + dsqrt<R>(d2 * d2 - qdiv<R>(c2 * bn * bn, d, id)));
}

// find_mhd_flux (models/mhd_utils.h:182-245), cIso == 0
template <typename R>
__device__ __forceinline__ void
mhd_flux(const R * q, R * cv, R * ff, const Phys<R> & s)
{
  const R p = q[IP];
  const R entho = R(1) / (s.gamma0 - R(1));
  const R d = q[ID], u = q[IU], v = q[IV], w = q[IW], a = q[IA], b = q[IB], c = q[IC];
  const R ecin = R(0.5) * (u * u + v * v + w * w) * d;
  const R emag = R(0.5) * (a * a + b * b + c * c);
  const R etot = p * entho + ecin + emag;
  const R ptot = p + emag;
  cv[ID] = d;
  cv[IP] = etot;
  cv[IU] = d * u;
  cv[IV] = d * v;
  cv[IW] = d * w;
  cv[IA] = a;
  cv[IB] = b;
  cv[IC] = c;
  ff[ID] = d * u;
  ff[IP] = (etot + ptot) * u - a * (a * u + b * v + c * w);
  ff[IU] = d * u * u - a * a + ptot;
  ff[IV] = d * u * v - a * b;
  ff[IW] = d * u * w - a * c;
  ff[IA] = R(0);
  ff[IB] = b * u - a * v;
  ff[IC] = c * u - a * w;
}

// riemann_hll (models/RiemannSolvers_MHD.h:43-102)
template <typename R>
__device__ void
riemann_hll(R * qL, R * qR, R * flux, const Phys<R> & s)
{
  const R bx_mean = R(0.5) * (qL[IA] + qR[IA]);
  qL[IA] = bx_mean;
  qR[IA] = bx_mean;
  R uL[8], fL[8], uR[8], fR[8];
  mhd_flux(qL, uL, fL, s);
  mhd_flux(qR, uR, fR, s);
  const R cfL = speed_fast(qL, 0, s);
  const R cfR = speed_fast(qR, 0, s);
  const R vL = qL[IU], vR = qR[IU];
  const R sl = rmin<R>(rmin<R>(vL, vR) - rmax<R>(cfL, cfR), R(0));
  const R sr = rmax<R>(rmax<R>(vL, vR) + rmax<R>(cfL, cfR), R(0));
#pragma unroll
  for (int n = 0; n < 8; ++n)
    flux[n] = (sr * fL[n] - sl * fR[n] + sr * sl * (uR[n] - uL[n])) / (sr - sl);
}

// riemann_llf (models/RiemannSolvers_MHD.h:118-153)
template <typename R>
__device__ void
riemann_llf(R * qL, R * qR, R * flux, const Phys<R> & s)
{
  const R bx_mean = R(0.5) * (qL[IA] + qR[IA]);
  qL[IA] = bx_mean;
  qR[IA] = bx_mean;
  R uL[8], fL[8], uR[8], fR[8];
  mhd_flux(qL, uL, fL, s);
  mhd_flux(qR, uR, fR, s);
#pragma unroll
  for (int n = 0; n < 8; ++n)
    flux[n] = (fL[n] + fR[n]) / R(2);
  // x-direction info speed (models/mhd_utils.h:405-433)
  R cinfo[2];
  for (int side = 0; side < 2; ++side)
  {
    const R * q = side == 0 ? qL : qR;
    const R   d = q[ID], p = q[IP], a = q[IA], b = q[IB], c = q[IC];
    const R   b2 = a * a + b * b + c * c;
    const R   c2 = s.gamma0 * p / d;
    const R   d2 = R(0.5) * (b2 / d + c2);
    const R   cf = dsqrt<R>(d2 + dsqrt<R>(d2 * d2 - c2 * a * a / d));
    cinfo[side] = cf + rabs<R>(q[IU]);
  }
  const R vel_info = rmax<R>(cinfo[0], cinfo[1]);
#pragma unroll
  for (int n = 0; n < 8; ++n)
    flux[n] -= vel_info * (uR[n] - uL[n]) / R(2);
}

// riemann_hllc (models/RiemannSolvers_MHD.h:165-286); components IA..IC are left at 0
template <typename R>
__device__ void
riemann_hllc(const R * qL, const R * qR, R * flux, const Phys<R> & s)
{
  const R entho = R(1) / (s.gamma0 - R(1));
  const R rl = rmax<R>(qL[ID], s.smallr);
  const R pl = rmax<R>(qL[IP], rl * s.smallp);
  const R ul = qL[IU];
  R       ecinl = R(0.5) * rl * ul * ul;
  ecinl += R(0.5) * rl * qL[IV] * qL[IV];
  ecinl += R(0.5) * rl * qL[IW] * qL[IW];
  const R etotl = pl * entho + ecinl;
  const R ptotl = pl;
  const R rr = rmax<R>(qR[ID], s.smallr);
  const R pr = rmax<R>(qR[IP], rr * s.smallp);
  const R ur = qR[IU];
  R       ecinr = R(0.5) * rr * ur * ur;
  ecinr += R(0.5) * rr * qR[IV] * qR[IV];
  ecinr += R(0.5) * rr * qR[IW] * qR[IW];
  const R etotr = pr * entho + ecinr;
  const R ptotr = pr;
  const R cfastl = dsqrt<R>(rmax<R>(s.gamma0 * pl / rl, s.smallc * s.smallc));
  const R cfastr = dsqrt<R>(rmax<R>(s.gamma0 * pr / rr, s.smallc * s.smallc));
  const R SL = rmin<R>(ul, ur) - rmax<R>(cfastl, cfastr);
  const R SR = rmax<R>(ul, ur) + rmax<R>(cfastl, cfastr);
  const R rcl = rl * (ul - SL);
  const R rcr = rr * (SR - ur);
  const R ustar = (rcr * ur + rcl * ul + (ptotl - ptotr)) / (rcr + rcl);
  const R ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) / (rcr + rcl);
  const R rstarl = rl * (SL - ul) / (SL - ustar);
  const R etotstarl = ((SL - ul) * etotl - ptotl * ul + ptotstar * ustar) / (SL - ustar);
  const R rstarr = rr * (SR - ur) / (SR - ustar);
  const R etotstarr = ((SR - ur) * etotr - ptotr * ur + ptotstar * ustar) / (SR - ustar);
  R       ro, uo, ptoto, etoto;
  if (SL > R(0))
  {
    ro = rl; uo = ul; ptoto = ptotl; etoto = etotl;
  }
  else if (ustar > R(0))
  {
    ro = rstarl; uo = ustar; ptoto = ptotstar; etoto = etotstarl;
  }
  else if (SR > R(0))
  {
    ro = rstarr; uo = ustar; ptoto = ptotstar; etoto = etotstarr;
  }
  else
  {
    ro = rr; uo = ur; ptoto = ptotr; etoto = etotr;
  }
  flux[ID] = ro * uo;
  flux[IU] = ro * uo * uo + ptoto;
  flux[IP] = (etoto + ptoto) * uo;
  flux[IV] = flux[ID] > R(0) ? flux[ID] * qL[IV] : flux[ID] * qR[IV];
  flux[IW] = flux[ID] > R(0) ? flux[ID] * qL[IW] : flux[ID] * qR[IW];
}

// riemann_hlld (models/RiemannSolvers_MHD.h:311-551), Miyoshi & Kusano 2005
template <typename R>
__device__ void
riemann_hlld(R * qL, R * qR, R * flux, const Phys<R> & s)
{
  const R entho = R(1) / (s.gamma0 - R(1));
  const R a = R(0.5) * (qL[IA] + qR[IA]);
  const R sgnm = (a >= 0) ? R(1) : R(-1);
  qL[IA] = a;
  qR[IA] = a;
  const R rl = qL[ID], pl = qL[IP], ul = qL[IU], vl = qL[IV], wl = qL[IW], bl = qL[IB], cl = qL[IC];
  const R ecinl = R(0.5) * (ul * ul + vl * vl + wl * wl) * rl;
  const R emagl = R(0.5) * (a * a + bl * bl + cl * cl);
  const R etotl = pl * entho + ecinl + emagl;
  const R ptotl = pl + emagl;
  const R vdotbl = ul * a + vl * bl + wl * cl;
  const R rr = qR[ID], pr = qR[IP], ur = qR[IU], vr = qR[IV], wr = qR[IW], br = qR[IB], cr = qR[IC];
  const R ecinr = R(0.5) * (ur * ur + vr * vr + wr * wr) * rr;
  const R emagr = R(0.5) * (a * a + br * br + cr * cr);
  const R etotr = pr * entho + ecinr + emagr;
  const R ptotr = pr + emagr;
  const R vdotbr = ur * a + vr * br + wr * cr;

  const R cfastl = speed_fast(qL, 0, s);
  const R cfastr = speed_fast(qR, 0, s);
  const R sl = rmin<R>(ul, ur) - rmax<R>(cfastl, cfastr);
  const R sr = rmax<R>(ul, ur) + rmax<R>(cfastl, cfastr);
  const R rcl = rl * (ul - sl);
  const R rcr = rr * (sr - ur);
  const R irc = recip<R>(rcr + rcl);
  const R ustar = qdiv<R>(rcr * ur + rcl * ul + (ptotl - ptotr), rcr + rcl, irc);
  const R ptotstar = qdiv<R>(rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur), rcr + rcl, irc);

  const R isl = recip<R>(sl - ustar);
  const R rstarl = qdiv<R>(rl * (sl - ul), sl - ustar, isl);
  R       estar = rl * (sl - ul) * (sl - ustar) - a * a;
  const R el = rl * (sl - ul) * (sl - ul) - a * a;
  R       vstarl, wstarl, bstarl, cstarl;
  if (rabs<R>(estar) < R(1e-4) * (a * a))
  {
    vstarl = vl; bstarl = bl; wstarl = wl; cstarl = cl;
  }
  else
  {
    const R ie = recip<R>(estar);
    vstarl = vl - qdiv<R>(a * bl * (ustar - ul), estar, ie);
    bstarl = qdiv<R>(bl * el, estar, ie);
    wstarl = wl - qdiv<R>(a * cl * (ustar - ul), estar, ie);
    cstarl = qdiv<R>(cl * el, estar, ie);
  }
  const R vdotbstarl = ustar * a + vstarl * bstarl + wstarl * cstarl;
  const R etotstarl =
    qdiv<R>((sl - ul) * etotl - ptotl * ul + ptotstar * ustar + a * (vdotbl - vdotbstarl), sl - ustar, isl);
  R sqrrstarl, calfvenl;
  if constexpr (std::is_same<R, float>::value)
  {
    const float rs = rsqrtf(rstarl);
    sqrrstarl = rstarl * rs;
    calfvenl = rabs<R>(a) * rs;
  }
  else
  {
    sqrrstarl = dsqrt<R>(rstarl);
    calfvenl = rabs<R>(a) / sqrrstarl;
  }
  const R sal = ustar - calfvenl;

  const R isr = recip<R>(sr - ustar);
  const R rstarr = qdiv<R>(rr * (sr - ur), sr - ustar, isr);
  estar = rr * (sr - ur) * (sr - ustar) - a * a;
  const R er = rr * (sr - ur) * (sr - ur) - a * a;
  R       vstarr, wstarr, bstarr, cstarr;
  if (rabs<R>(estar) < R(1e-4) * (a * a))
  {
    vstarr = vr; bstarr = br; wstarr = wr; cstarr = cr;
  }
  else
  {
    const R ie = recip<R>(estar);
    vstarr = vr - qdiv<R>(a * br * (ustar - ur), estar, ie);
    bstarr = qdiv<R>(br * er, estar, ie);
    wstarr = wr - qdiv<R>(a * cr * (ustar - ur), estar, ie);
    cstarr = qdiv<R>(cr * er, estar, ie);
  }
  const R vdotbstarr = ustar * a + vstarr * bstarr + wstarr * cstarr;
  const R etotstarr =
    qdiv<R>((sr - ur) * etotr - ptotr * ur + ptotstar * ustar + a * (vdotbr - vdotbstarr), sr - ustar, isr);
  R sqrrstarr, calfvenr;
  if constexpr (std::is_same<R, float>::value)
  {
    const float rs = rsqrtf(rstarr);
    sqrrstarr = rstarr * rs;
    calfvenr = rabs<R>(a) * rs;
  }
  else
  {
    sqrrstarr = dsqrt<R>(rstarr);
    calfvenr = rabs<R>(a) / sqrrstarr;
  }
  const R sar = ustar + calfvenr;

  const R isq = recip<R>(sqrrstarl + sqrrstarr);
  const R vstarstar =
    qdiv<R>(sqrrstarl * vstarl + sqrrstarr * vstarr + sgnm * (bstarr - bstarl), sqrrstarl + sqrrstarr, isq);
  const R wstarstar =
    qdiv<R>(sqrrstarl * wstarl + sqrrstarr * wstarr + sgnm * (cstarr - cstarl), sqrrstarl + sqrrstarr, isq);
  const R bstarstar =
    qdiv<R>(sqrrstarl * bstarr + sqrrstarr * bstarl + sgnm * sqrrstarl * sqrrstarr * (vstarr - vstarl),
            sqrrstarl + sqrrstarr, isq);
  const R cstarstar =
    qdiv<R>(sqrrstarl * cstarr + sqrrstarr * cstarl + sgnm * sqrrstarl * sqrrstarr * (wstarr - wstarl),
            sqrrstarl + sqrrstarr, isq);
  const R vdotbstarstar = ustar * a + vstarstar * bstarstar + wstarstar * cstarstar;
  const R etotstarstarl = etotstarl - sgnm * sqrrstarl * (vdotbstarl - vdotbstarstar);
  const R etotstarstarr = etotstarr + sgnm * sqrrstarr * (vdotbstarr - vdotbstarstar);

  R ro, uo, vo, wo, bo, co, ptoto, etoto, vdotbo;
  if (sl > 0)
  {
    ro = rl; uo = ul; vo = vl; wo = wl; bo = bl; co = cl;
    ptoto = ptotl; etoto = etotl; vdotbo = vdotbl;
  }
  else if (sal > 0)
  {
    ro = rstarl; uo = ustar; vo = vstarl; wo = wstarl; bo = bstarl; co = cstarl;
    ptoto = ptotstar; etoto = etotstarl; vdotbo = vdotbstarl;
  }
  else if (ustar > 0)
  {
    ro = rstarl; uo = ustar; vo = vstarstar; wo = wstarstar; bo = bstarstar; co = cstarstar;
    ptoto = ptotstar; etoto = etotstarstarl; vdotbo = vdotbstarstar;
  }
  else if (sar > 0)
  {
    ro = rstarr; uo = ustar; vo = vstarstar; wo = wstarstar; bo = bstarstar; co = cstarstar;
    ptoto = ptotstar; etoto = etotstarstarr; vdotbo = vdotbstarstar;
  }
  else if (sr > 0)
  {
    ro = rstarr; uo = ustar; vo = vstarr; wo = wstarr; bo = bstarr; co = cstarr;
    ptoto = ptotstar; etoto = etotstarr; vdotbo = vdotbstarr;
  }
  else
  {
    ro = rr; uo = ur; vo = vr; wo = wr; bo = br; co = cr;
    ptoto = ptotr; etoto = etotr; vdotbo = vdotbr;
  }
  flux[ID] = ro * uo;
  flux[IP] = (etoto + ptoto) * uo - a * vdotbo;
  flux[IU] = ro * uo * uo - a * a + ptoto;
  flux[IV] = ro * uo * vo - a * bo;
  flux[IW] = ro * uo * wo - a * co;
  flux[IA] = R(0);
  flux[IB] = bo * uo - a * vo;
  flux[IC] = co * uo - a * wo;
}

// riemann_mhd dispatch (models/RiemannSolvers_MHD.h:559-590)
template <typename R>
__device__ __forceinline__ void
riemann_mhd(R * qL, R * qR, R * flux, const Phys<R> & s)
{
  if (s.riemann == RS_HLLD)
    riemann_hlld(qL, qR, flux, s);
  else if (s.riemann == RS_HLL)
    riemann_hll(qL, qR, flux, s);
  else if (s.riemann == RS_LLF)
    riemann_llf(qL, qR, flux, s);
  else
  {
#pragma unroll
    for (int n = 0; n < 8; ++n)
      flux[n] = R(0);
    riemann_hllc(qL, qR, flux, s);
  }
}

template <typename R>
__device__ __forceinline__ R
max4(R a0, R a1, R a2, R a3)
{
  R r = a0;
  r = (a1 > r) ? a1 : r;
  r = (a2 > r) ? a2 : r;
  r = (a3 > r) ? a3 : r;
  return r;
}
template <typename R>
__device__ __forceinline__ R
min4(R a0, R a1, R a2, R a3)
{
  R r = a0;
  r = (a1 < r) ? a1 : r;
  r = (a2 < r) ? a2 : r;
  r = (a3 < r) ? a3 : r;
  return r;
}
template <typename R>
__device__ __forceinline__ R
max5(R a0, R a1, R a2, R a3, R a4)
{
  R r = a0;
  r = (a1 > r) ? a1 : r;
  r = (a2 > r) ? a2 : r;
  r = (a3 > r) ? a3 : r;
  r = (a4 > r) ? a4 : r;
  return r;
}

// Edge-state slots: reconstructed states around an edge and the 2D Riemann problem states.
enum : int
{
  ERT = 0,
  ELT = 1,
  ERB = 2,
  ELB = 3
};
enum : int
{
  SLL = 0,
  SRL = 1,
  SLR = 2,
  SRR = 3
};

// compute_emf<dir> + mag_riemann2d_hlld (models/RiemannSolvers_MHD.h:629-869, 890-1097).
// qe[ERT..ELB] are the reconstructed edge states; emf_dir 0 (EMFX), 1 (EMFY), 2 (EMFZ).
template <typename R, int EMF_DIR>
__device__ R
edge_emf(const R (*qe)[8], const Phys<R> & s)
{
  // (first, second parallel velocity; orthogonal velocity) and the same for B
  constexpr int iu = EMF_DIR == 2 ? IU : (EMF_DIR == 1 ? IW : IV);
  constexpr int iv = EMF_DIR == 2 ? IV : (EMF_DIR == 1 ? IU : IW);
  constexpr int iw = EMF_DIR == 2 ? IW : (EMF_DIR == 1 ? IV : IU);
  constexpr int ia = EMF_DIR == 2 ? IA : (EMF_DIR == 1 ? IC : IB);
  constexpr int ib = EMF_DIR == 2 ? IB : (EMF_DIR == 1 ? IA : IC);
  constexpr int ic = EMF_DIR == 2 ? IC : (EMF_DIR == 1 ? IB : IA);
  const R *qRT = qe[ERT], *qLT = qe[ELT], *qRB = qe[ERB], *qLB = qe[ELB];
  // 4 states (LL, RL, LR, RR) in the rotated frame
  const R rLL = qRT[ID], rRL = qLT[ID], rLR = qRB[ID], rRR = qLB[ID];
  const R pLL = qRT[IP], pRL = qLT[IP], pLR = qRB[IP], pRR = qLB[IP];
  const R uLL = qRT[iu], uRL = qLT[iu], uLR = qRB[iu], uRR = qLB[iu];
  const R vLL = qRT[iv], vRL = qLT[iv], vLR = qRB[iv], vRR = qLB[iv];
  const R aLL = R(0.5) * (qRT[ia] + qLT[ia]);
  const R aRL = R(0.5) * (qRT[ia] + qLT[ia]);
  const R aLR = R(0.5) * (qRB[ia] + qLB[ia]);
  const R aRR = R(0.5) * (qRB[ia] + qLB[ia]);
  const R bLL = R(0.5) * (qRT[ib] + qRB[ib]);
  const R bRL = R(0.5) * (qLT[ib] + qLB[ib]);
  const R bLR = R(0.5) * (qRT[ib] + qRB[ib]);
  const R bRR = R(0.5) * (qLT[ib] + qLB[ib]);
  const R cLL = qRT[ic], cRL = qLT[ic], cLR = qRB[ic], cRR = qLB[ic];
  (void)iw;

  const R ELL = uLL * bLL - vLL * aLL;
  const R ERL = uRL * bRL - vRL * aRL;
  const R ELR = uLR * bLR - vLR * aLR;
  const R ERR = uRR * bRR - vRR * aRR;

  // find_speed_fast<IX>/<IY> for the 4 states (models/mhd_utils.h:93-122)
  auto fast = [&](R d, R p, R a, R b, R c, R bn) {
    const R id = recip<R>(d);
    const R b2 = a * a + b * b + c * c;
    const R c2 = qdiv<R>(s.gamma0 * p, d, id);
    const R d2 = R(0.5) * (qdiv<R>(b2, d, id) + c2);
    return dsqrt<R>(d2 + dsqrt<R>(d2 * d2 - qdiv<R>(c2 * bn * bn, d, id)));
  };
  const R cFastLLx = fast(rLL, pLL, aLL, bLL, cLL, aLL);
  const R cFastLRx = fast(rLR, pLR, aLR, bLR, cLR, aLR);
  const R cFastRLx = fast(rRL, pRL, aRL, bRL, cRL, aRL);
  const R cFastRRx = fast(rRR, pRR, aRR, bRR, cRR, aRR);
  const R cFastLLy = fast(rLL, pLL, aLL, bLL, cLL, bLL);
  const R cFastLRy = fast(rLR, pLR, aLR, bLR, cLR, bLR);
  const R cFastRLy = fast(rRL, pRL, aRL, bRL, cRL, bRL);
  const R cFastRRy = fast(rRR, pRR, aRR, bRR, cRR, bRR);

  const R SL = min4(uLL, uLR, uRL, uRR) - max4(cFastLLx, cFastLRx, cFastRLx, cFastRRx);
  const R SR = max4(uLL, uLR, uRL, uRR) + max4(cFastLLx, cFastLRx, cFastRLx, cFastRRx);
  const R SB = min4(vLL, vLR, vRL, vRR) - max4(cFastLLy, cFastLRy, cFastRLy, cFastRRy);
  const R ST = max4(vLL, vLR, vRL, vRR) + max4(cFastLLy, cFastLRy, cFastRLy, cFastRRy);

  const R PtotLL = pLL + R(0.5) * (aLL * aLL + bLL * bLL + cLL * cLL);
  const R PtotLR = pLR + R(0.5) * (aLR * aLR + bLR * bLR + cLR * cLR);
  const R PtotRL = pRL + R(0.5) * (aRL * aRL + bRL * bRL + cRL * cRL);
  const R PtotRR = pRR + R(0.5) * (aRR * aRR + bRR * bRR + cRR * cRR);

  const R rcLLx = rLL * (uLL - SL);
  const R rcRLx = rRL * (SR - uRL);
  const R rcLRx = rLR * (uLR - SL);
  const R rcRRx = rRR * (SR - uRR);
  const R rcLLy = rLL * (vLL - SB);
  const R rcLRy = rLR * (ST - vLR);
  const R rcRLy = rRL * (vRL - SB);
  const R rcRRy = rRR * (ST - vRR);

  const R ustar =
    (rcLLx * uLL + rcLRx * uLR + rcRLx * uRL + rcRRx * uRR + (PtotLL - PtotRL + PtotLR - PtotRR)) /
    (rcLLx + rcLRx + rcRLx + rcRRx);
  const R vstar =
    (rcLLy * vLL + rcLRy * vLR + rcRLy * vRL + rcRRy * vRR + (PtotLL - PtotLR + PtotRL - PtotRR)) /
    (rcLLy + rcLRy + rcRLy + rcRRy);

  // shared divisors of the star states
  const R dLu = SL - ustar, dRu = SR - ustar, dBv = SB - vstar, dTv = ST - vstar;
  const R iLu = recip<R>(dLu), iRu = recip<R>(dRu), iBv = recip<R>(dBv), iTv = recip<R>(dTv);

  const R rstarLLx = qdiv<R>(rLL * (SL - uLL), dLu, iLu);
  const R BstarLL = qdiv<R>(bLL * (SL - uLL), dLu, iLu);
  const R rstarLLy = qdiv<R>(rLL * (SB - vLL), dBv, iBv);
  const R AstarLL = qdiv<R>(aLL * (SB - vLL), dBv, iBv);
  const R rstarLL = qdiv<R>(qdiv<R>(rLL * (SL - uLL), dLu, iLu) * (SB - vLL), dBv, iBv);
  const R EstarLLx = ustar * BstarLL - vLL * aLL;
  const R EstarLLy = uLL * bLL - vstar * AstarLL;
  const R EstarLL = ustar * BstarLL - vstar * AstarLL;

  const R rstarLRx = qdiv<R>(rLR * (SL - uLR), dLu, iLu);
  const R BstarLR = qdiv<R>(bLR * (SL - uLR), dLu, iLu);
  const R rstarLRy = qdiv<R>(rLR * (ST - vLR), dTv, iTv);
  const R AstarLR = qdiv<R>(aLR * (ST - vLR), dTv, iTv);
  const R rstarLR = qdiv<R>(qdiv<R>(rLR * (SL - uLR), dLu, iLu) * (ST - vLR), dTv, iTv);
  const R EstarLRx = ustar * BstarLR - vLR * aLR;
  const R EstarLRy = uLR * bLR - vstar * AstarLR;
  const R EstarLR = ustar * BstarLR - vstar * AstarLR;

  const R rstarRLx = qdiv<R>(rRL * (SR - uRL), dRu, iRu);
  const R BstarRL = qdiv<R>(bRL * (SR - uRL), dRu, iRu);
  const R rstarRLy = qdiv<R>(rRL * (SB - vRL), dBv, iBv);
  const R AstarRL = qdiv<R>(aRL * (SB - vRL), dBv, iBv);
  const R rstarRL = qdiv<R>(qdiv<R>(rRL * (SR - uRL), dRu, iRu) * (SB - vRL), dBv, iBv);
  const R EstarRLx = ustar * BstarRL - vRL * aRL;
  const R EstarRLy = uRL * bRL - vstar * AstarRL;
  const R EstarRL = ustar * BstarRL - vstar * AstarRL;

  const R rstarRRx = qdiv<R>(rRR * (SR - uRR), dRu, iRu);
  const R BstarRR = qdiv<R>(bRR * (SR - uRR), dRu, iRu);
  const R rstarRRy = qdiv<R>(rRR * (ST - vRR), dTv, iTv);
  const R AstarRR = qdiv<R>(aRR * (ST - vRR), dTv, iTv);
  const R rstarRR = qdiv<R>(qdiv<R>(rRR * (SR - uRR), dRu, iRu) * (ST - vRR), dTv, iTv);
  const R EstarRRx = ustar * BstarRR - vRR * aRR;
  const R EstarRRy = uRR * bRR - vstar * AstarRR;
  const R EstarRR = ustar * BstarRR - vstar * AstarRR;

  const R calfvenL = max5<R>(div_sqrt<R>(rabs<R>(aLR), rstarLRx), div_sqrt<R>(rabs<R>(AstarLR), rstarLR),
                             div_sqrt<R>(rabs<R>(aLL), rstarLLx), div_sqrt<R>(rabs<R>(AstarLL), rstarLL), s.smallc);
  const R calfvenR = max5<R>(div_sqrt<R>(rabs<R>(aRR), rstarRRx), div_sqrt<R>(rabs<R>(AstarRR), rstarRR),
                             div_sqrt<R>(rabs<R>(aRL), rstarRLx), div_sqrt<R>(rabs<R>(AstarRL), rstarRL), s.smallc);
  const R calfvenB = max5<R>(div_sqrt<R>(rabs<R>(bLL), rstarLLy), div_sqrt<R>(rabs<R>(BstarLL), rstarLL),
                             div_sqrt<R>(rabs<R>(bRL), rstarRLy), div_sqrt<R>(rabs<R>(BstarRL), rstarRL), s.smallc);
  const R calfvenT = max5<R>(div_sqrt<R>(rabs<R>(bLR), rstarLRy), div_sqrt<R>(rabs<R>(BstarLR), rstarLR),
                             div_sqrt<R>(rabs<R>(bRR), rstarRRy), div_sqrt<R>(rabs<R>(BstarRR), rstarRR), s.smallc);

  const R SAL = rmin<R>(ustar - calfvenL, R(0));
  const R SAR = rmax<R>(ustar + calfvenR, R(0));
  const R SAB = rmin<R>(vstar - calfvenB, R(0));
  const R SAT = rmax<R>(vstar + calfvenT, R(0));

  const R dRL = SAR - SAL, dTB = SAT - SAB;
  const R iRL = recip<R>(dRL), iTB = recip<R>(dTB);
  const R AstarT = qdiv<R>(SAR * AstarRR - SAL * AstarLR, dRL, iRL);
  const R AstarB = qdiv<R>(SAR * AstarRL - SAL * AstarLL, dRL, iRL);
  const R BstarR = qdiv<R>(SAT * BstarRR - SAB * BstarRL, dTB, iTB);
  const R BstarL = qdiv<R>(SAT * BstarLR - SAB * BstarLL, dTB, iTB);

  R       E = 0, tmpE = 0;
  const R SB_pos = (1 + rcopysign<R>(R(1), SB)) / 2, SB_neg = 1 - SB_pos;
  const R ST_pos = (1 + rcopysign<R>(R(1), ST)) / 2, ST_neg = 1 - ST_pos;
  const R SL_pos = (1 + rcopysign<R>(R(1), SL)) / 2, SL_neg = 1 - SL_pos;
  const R SR_pos = (1 + rcopysign<R>(R(1), SR)) / 2, SR_neg = 1 - SR_pos;

  tmpE = qdiv<R>(qdiv<R>(SAL * SAB * EstarRR - SAL * SAT * EstarRL - SAR * SAB * EstarLR + SAR * SAT * EstarLL, dRL,
                         iRL),
                 dTB, iTB) -
         qdiv<R>(SAT * SAB, dTB, iTB) * (AstarT - AstarB) + qdiv<R>(SAR * SAL, dRL, iRL) * (BstarR - BstarL);
  E += (SB_neg * ST_pos * SL_neg * SR_pos) * tmpE;

  tmpE = qdiv<R>(SAR * EstarLLx - SAL * EstarRLx + SAR * SAL * (bRL - bLL), dRL, iRL);
  tmpE = SL_pos * ELL + SL_neg * SR_neg * ERL + SL_neg * SR_pos * tmpE;
  E += SB_pos * tmpE;

  tmpE = qdiv<R>(SAR * EstarLRx - SAL * EstarRRx + SAR * SAL * (bRR - bLR), dRL, iRL);
  tmpE = SL_pos * ELR + SL_neg * SR_neg * ERR + SL_neg * SR_pos * tmpE;
  E += (SB_neg * ST_neg) * tmpE;

  tmpE = qdiv<R>(SAT * EstarLLy - SAB * EstarLRy - SAT * SAB * (aLR - aLL), dTB, iTB);
  E += (SB_neg * ST_pos * SL_pos) * tmpE;

  tmpE = qdiv<R>(SAT * EstarRLy - SAB * EstarRRy - SAT * SAB * (aRR - aRL), dTB, iTB);
  E += (SB_neg * ST_pos * SL_neg * SR_neg) * tmpE;

  return E;
}

// slope_unsplit_scalar (scheme/ComputeLimitedSlopesFunctor.cpp:121-144)
template <typename R>
__device__ __forceinline__ R
slope1(R q, R qp, R qm, R slope_type)
{
  R dq = 0;
  if (slope_type == R(1) || slope_type == R(2))
  {
    const R dlft = slope_type * (q - qm);
    const R drgt = slope_type * (qp - q);
    const R dcen = R(0.5) * (qp - qm);
    const R dsgn = (dcen >= R(0)) ? R(1) : R(-1);
    const R slop = rmin<R>(rabs<R>(dlft), rabs<R>(drgt));
    const R dlim = (dlft * drgt) <= R(0) ? R(0) : slop;
    dq = dsgn * rmin<R>(dlim, rabs<R>(dcen));
  }
  return dq;
}

} // namespace gmhd

namespace gmhd
{
// FP64 <-> FP32 conversions on the integer pipe. On GB300 the FP64 pipe (which also executes
// F2F conversions) has a small fraction of the FP32 rate, so the mixed path converts by
// rebuilding the IEEE-754 bit patterns instead.

// double -> float, rounding the 29 dropped mantissa bits half away from zero; results below the
// float normal range flush to signed zero, above it saturate to infinity; NaN stays NaN.
__device__ __forceinline__ float
d2f_bits(double x)
{
  const unsigned hi = (unsigned)__double2hiint(x);
  const unsigned lo = (unsigned)__double2loint(x);
  const unsigned sign = hi & 0x80000000u;
  const unsigned mag = hi & 0x7fffffffu;
  // the low 8 exponent bits and the top 23 mantissa bits in place (one funnel shift); for exponents
  // 897..1150 (the float normal range) e - 896 == (e & 0xff) ^ 0x80, so the rebias 1023 -> 127 is a
  // flip of the field's top bit; then the first dropped bit rounds, a carry out of the mantissa
  // moving into the exponent as it should
  const unsigned bits = ((__funnelshift_l(lo, hi, 3) & 0x7fffffffu) ^ 0x40000000u) + ((lo >> 28) & 1u);
  // |x| below the float normal range (exponent <= 896) -> signed zero; at or above 2^128
  // (exponent >= 1151), infinity or NaN -> infinity / quiet NaN
  if (mag < 0x38100000u)
    return __uint_as_float(sign);
  if (mag >= 0x47f00000u)
  {
    const bool nan = mag > 0x7ff00000u || (mag == 0x7ff00000u && lo != 0u);
    return __uint_as_float(sign | 0x7f800000u | (nan ? 0x400000u : 0u));
  }
  return __uint_as_float(sign | bits);
}

// float -> double, exact for normal numbers, zero, infinity and NaN (subnormals flush to zero).
__device__ __forceinline__ double
f2d_bits(float x)
{
  const unsigned b = __float_as_uint(x);
  const unsigned sign = b & 0x80000000u;
  const unsigned e = (b >> 23) & 0xffu;
  const unsigned m = b & 0x7fffffu;
  const unsigned eb = e == 0xffu ? 0x7ffu : e + 896u;
  unsigned       hi = sign | (eb << 20) | (m >> 3);
  unsigned       lo = m << 29;
  hi = e == 0u ? sign : hi;
  lo = e == 0u ? 0u : lo;
  return __hiloint2double((int)hi, (int)lo);
}

// Adds t to the running sum s and the rounding error of that addition to e (Knuth's TwoSum: six
// FP32 operations, no branch, valid for any magnitudes; no multiply, so FMA contraction cannot
// change it). After the last term, s + e holds the exact sum of the terms up to the rounding of e
// itself, which is of order eps^2 relative to the terms.
__device__ __forceinline__ void
two_sum_acc(float & s, float & e, float t)
{
  const float u = s + t;
  const float tb = u - s;
  const float err = (s - (u - tb)) + (t - tb);
  s = u;
  e += err;
}

template <typename R>
__device__ __forceinline__ R
to_r(double x)
{
  return x;
}
template <>
__device__ __forceinline__ float
to_r<float>(double x)
{
  return d2f_bits(x);
}

template <typename R>
__device__ __forceinline__ double
to_d(R x)
{
  return x;
}
template <>
__device__ __forceinline__ double
to_d<float>(float x)
{
  return f2d_bits(x);
}
} // namespace gmhd

// Oracle — test infrastructure only. Nothing in the product links, includes or calls this file;
// tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it as the checker.
//
// Plain-C++ FP64 restatement of the per-cell MHD math of godunov_mhd_ct (models/mhd_utils.h and
// models/RiemannSolvers_MHD.h). Every floating-point expression keeps the reference's operand
// order, so that a GPU kernel compiled without FMA contraction can match it bit for bit.
// Compile with -ffp-contract=off: the expressions below must not be fused.
#pragma once

#include <cmath>
#include <cstdint>

namespace oracle
{

// Variable ids (models/MHD.h:35-62).
enum : int
{
  ID = 0,
  IP = 1,
  IU = 2,
  IV = 3,
  IW = 4,
  IA = 5,
  IB = 6,
  IC = 7,
  IAR = 8,
  IBR = 9,
  ICR = 10
};

// Riemann solver ids (models/riemann_solver_types.h:26-37; same numeric order as the enum).
enum : int
{
  RIEMANN_LLF = 2,
  RIEMANN_HLL = 3,
  RIEMANN_HLLC = 4,
  RIEMANN_HLLD = 5
};

// Hydro/MHD settings actually read on the hot path (models/HydroSettings.cpp:18-31).
struct Settings
{
  double gamma0;
  double cfl;
  double slope_type;
  double smallr;
  double smallc;
  double smallp;  // smallc^2 / gamma0
  double smallpp; // smallr * smallp
  double cIso;    // always 0 in the reference (HydroSettings.cpp:27)
  int    riemann;
  int    rk2 = 0; // [amr] time_integrator: 0 HANCOCK, 1 RK2_SSP
  // uniform gravity ([gravity] enabled, uniform_gx/gy/gz; kalypsso-core get_uniform_gravity_vector)
  int    gravity = 0;
  double grav[3] = {0.0, 0.0, 0.0};
  // viscosity ([viscosity] enabled, mu; kalypsso-core ViscosityParams) and its Hancock predictor term
  int    viscosity = 0;
  double mu = 0.0;
  int    visc_predictor = 0;
};

inline Settings
make_settings(double gamma0, double cfl, double slope_type, double smallr, double smallc, int riemann)
{
  Settings s;
  s.gamma0 = gamma0;
  s.cfl = cfl;
  s.slope_type = slope_type;
  s.smallr = smallr;
  s.smallc = smallc;
  s.smallp = smallc * smallc / gamma0;
  s.smallpp = smallr * s.smallp;
  s.cIso = 0.0;
  s.riemann = riemann;
  return s;
}

// find_speed_fast<dir> (models/mhd_utils.h:93-122); dir selects the B component that is normal.
inline double
find_speed_fast(const double * q, int dir, const Settings & s)
{
  const double d = q[ID];
  const double p = q[IP];
  const double a = q[IA];
  const double b = q[IB];
  const double c = q[IC];
  const double b2 = a * a + b * b + c * c;
  const double c2 = s.gamma0 * p / d;
  const double d2 = 0.5 * (b2 / d + c2);
  const double bn = dir == 0 ? a : (dir == 1 ? b : c);
  return std::sqrt(d2 + std::sqrt(d2 * d2 - c2 * bn * bn / d));
}

// find_speed_info<dim> (models/mhd_utils.h:340-394): fast speed + |v| per direction.
inline void
find_speed_info(const double * q, int dim, double * out, const Settings & s)
{
  const double d = q[ID], p = q[IP], u = q[IU], v = q[IV], w = q[IW];
  const double a = q[IA], b = q[IB], c = q[IC];
  const double b2 = a * a + b * b + c * c;
  const double c2 = s.gamma0 * p / d;
  const double d2 = 0.5 * (b2 / d + c2);
  double       cf = std::sqrt(d2 + std::sqrt(d2 * d2 - c2 * a * a / d));
  out[0] = cf + std::fabs(u);
  cf = std::sqrt(d2 + std::sqrt(d2 * d2 - c2 * b * b / d));
  out[1] = cf + std::fabs(v);
  if (dim == 3)
  {
    cf = std::sqrt(d2 + std::sqrt(d2 * d2 - c2 * c * c / d));
    out[2] = cf + std::fabs(w);
  }
}

// compute_primitives (models/mhd_utils.h:449-515). u holds (rho, E, rho u, rho v, rho w, Bx, By, Bz)
// with cell-centred B; q receives (rho, p, u, v, w, Bx, By, Bz). Returns the sound speed in *c.
inline void
compute_primitives(const double * u, double * q, double * c_out, const Settings & s)
{
  q[ID] = std::fmax(u[ID], s.smallr);
  q[IU] = u[IU] / q[ID];
  q[IV] = u[IV] / q[ID];
  q[IW] = u[IW] / q[ID];
  q[IA] = u[IA];
  q[IB] = u[IB];
  q[IC] = u[IC];
  const double eken = 0.5 * (q[IU] * q[IU] + q[IV] * q[IV] + q[IW] * q[IW]);
  const double emag = 0.5 * (q[IA] * q[IA] + q[IB] * q[IB] + q[IC] * q[IC]);
  const double eint = (u[IP] - emag) / q[ID] - eken;
  if (s.cIso > 0)
  {
    q[IP] = q[ID] * s.cIso * s.cIso;
    if (c_out)
      *c_out = s.cIso;
  }
  else
  {
    q[IP] = std::fmax((s.gamma0 - 1.0) * q[ID] * eint, q[ID] * s.smallp);
    if (c_out)
      *c_out = std::sqrt(s.gamma0 * q[IP] / q[ID]);
  }
}

// find_mhd_flux (models/mhd_utils.h:182-245), used by HLL and LLF.
inline void
find_mhd_flux(const double * q, double * cv, double * ff, const Settings & s)
{
  const double p = s.cIso > 0 ? q[ID] * s.cIso * s.cIso : q[IP];
  const double entho = 1.0 / (s.gamma0 - 1.0);
  const double d = q[ID], u = q[IU], v = q[IV], w = q[IW], a = q[IA], b = q[IB], c = q[IC];
  const double ecin = 0.5 * (u * u + v * v + w * w) * d;
  const double emag = 0.5 * (a * a + b * b + c * c);
  const double etot = p * entho + ecin + emag;
  const double ptot = p + emag;
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
  ff[IA] = 0.0;
  ff[IB] = b * u - a * v;
  ff[IC] = c * u - a * w;
}

// riemann_hll (models/RiemannSolvers_MHD.h:43-102). qL/qR are modified (normal B averaged).
inline void
riemann_hll(double * qL, double * qR, double * flux, const Settings & s)
{
  const double bx_mean = 0.5 * (qL[IA] + qR[IA]);
  qL[IA] = bx_mean;
  qR[IA] = bx_mean;
  double uL[8], fL[8], uR[8], fR[8];
  find_mhd_flux(qL, uL, fL, s);
  find_mhd_flux(qR, uR, fR, s);
  const double cfL = find_speed_fast(qL, 0, s);
  const double cfR = find_speed_fast(qR, 0, s);
  const double vL = qL[IU], vR = qR[IU];
  const double sl = std::fmin(std::fmin(vL, vR) - std::fmax(cfL, cfR), 0.0);
  const double sr = std::fmax(std::fmax(vL, vR) + std::fmax(cfL, cfR), 0.0);
  for (int n = 0; n < 8; ++n)
    flux[n] = (sr * fL[n] - sl * fR[n] + sr * sl * (uR[n] - uL[n])) / (sr - sl);
}

// riemann_llf (models/RiemannSolvers_MHD.h:118-153).
inline void
riemann_llf(double * qL, double * qR, double * flux, const Settings & s)
{
  const double bx_mean = 0.5 * (qL[IA] + qR[IA]);
  qL[IA] = bx_mean;
  qR[IA] = bx_mean;
  double uL[8], fL[8], uR[8], fR[8];
  find_mhd_flux(qL, uL, fL, s);
  find_mhd_flux(qR, uR, fR, s);
  for (int n = 0; n < 8; ++n)
    flux[n] = (fL[n] + fR[n]) / 2;
  // find_speed_info (scalar overload, models/mhd_utils.h:405-433): x-direction only.
  double sL[3], sR[3];
  find_speed_info(qL, 2, sL, s);
  find_speed_info(qR, 2, sR, s);
  const double vel_info = std::fmax(sL[0], sR[0]);
  for (int n = 0; n < 8; ++n)
    flux[n] -= vel_info * (uR[n] - uL[n]) / 2;
}

// riemann_hllc (models/RiemannSolvers_MHD.h:165-286). Writes ID, IP, IU, IV, IW only.
inline void
riemann_hllc(const double * qL, const double * qR, double * flux, const Settings & s)
{
  const double entho = 1.0 / (s.gamma0 - 1.0);
  const double rl = std::fmax(qL[ID], s.smallr);
  const double pl = std::fmax(qL[IP], rl * s.smallp);
  const double ul = qL[IU];
  double       ecinl = 0.5 * rl * ul * ul;
  ecinl += 0.5 * rl * qL[IV] * qL[IV];
  ecinl += 0.5 * rl * qL[IW] * qL[IW];
  const double etotl = pl * entho + ecinl;
  const double ptotl = pl;
  const double rr = std::fmax(qR[ID], s.smallr);
  const double pr = std::fmax(qR[IP], rr * s.smallp);
  const double ur = qR[IU];
  double       ecinr = 0.5 * rr * ur * ur;
  ecinr += 0.5 * rr * qR[IV] * qR[IV];
  ecinr += 0.5 * rr * qR[IW] * qR[IW];
  const double etotr = pr * entho + ecinr;
  const double ptotr = pr;
  const double cfastl = std::sqrt(std::fmax(s.gamma0 * pl / rl, s.smallc * s.smallc));
  const double cfastr = std::sqrt(std::fmax(s.gamma0 * pr / rr, s.smallc * s.smallc));
  const double SL = std::fmin(ul, ur) - std::fmax(cfastl, cfastr);
  const double SR = std::fmax(ul, ur) + std::fmax(cfastl, cfastr);
  const double rcl = rl * (ul - SL);
  const double rcr = rr * (SR - ur);
  const double ustar = (rcr * ur + rcl * ul + (ptotl - ptotr)) / (rcr + rcl);
  const double ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) / (rcr + rcl);
  const double rstarl = rl * (SL - ul) / (SL - ustar);
  const double etotstarl = ((SL - ul) * etotl - ptotl * ul + ptotstar * ustar) / (SL - ustar);
  const double rstarr = rr * (SR - ur) / (SR - ustar);
  const double etotstarr = ((SR - ur) * etotr - ptotr * ur + ptotstar * ustar) / (SR - ustar);
  double       ro, uo, ptoto, etoto;
  if (SL > 0.0)
  {
    ro = rl;
    uo = ul;
    ptoto = ptotl;
    etoto = etotl;
  }
  else if (ustar > 0.0)
  {
    ro = rstarl;
    uo = ustar;
    ptoto = ptotstar;
    etoto = etotstarl;
  }
  else if (SR > 0.0)
  {
    ro = rstarr;
    uo = ustar;
    ptoto = ptotstar;
    etoto = etotstarr;
  }
  else
  {
    ro = rr;
    uo = ur;
    ptoto = ptotr;
    etoto = etotr;
  }
  flux[ID] = ro * uo;
  flux[IU] = ro * uo * uo + ptoto;
  flux[IP] = (etoto + ptoto) * uo;
  flux[IV] = flux[ID] > 0.0 ? flux[ID] * qL[IV] : flux[ID] * qR[IV];
  flux[IW] = flux[ID] > 0.0 ? flux[ID] * qL[IW] : flux[ID] * qR[IW];
}

// riemann_hlld (models/RiemannSolvers_MHD.h:311-551), Miyoshi & Kusano 2005.
inline void
riemann_hlld(double * qL, double * qR, double * flux, const Settings & s)
{
  const double gamma0 = s.gamma0;
  const double entho = 1.0 / (gamma0 - 1.0);
  const double a = 0.5 * (qL[IA] + qR[IA]);
  const double sgnm = (a >= 0) ? 1.0 : -1.0;
  qL[IA] = a;
  qR[IA] = a;
  if (s.cIso > 0)
  {
    qL[IP] = qL[ID] * s.cIso * s.cIso;
    qR[IP] = qR[ID] * s.cIso * s.cIso;
  }
  const double rl = qL[ID], pl = qL[IP], ul = qL[IU], vl = qL[IV], wl = qL[IW], bl = qL[IB],
               cl = qL[IC];
  const double ecinl = 0.5 * (ul * ul + vl * vl + wl * wl) * rl;
  const double emagl = 0.5 * (a * a + bl * bl + cl * cl);
  const double etotl = pl * entho + ecinl + emagl;
  const double ptotl = pl + emagl;
  const double vdotbl = ul * a + vl * bl + wl * cl;

  const double rr = qR[ID], pr = qR[IP], ur = qR[IU], vr = qR[IV], wr = qR[IW], br = qR[IB],
               cr = qR[IC];
  const double ecinr = 0.5 * (ur * ur + vr * vr + wr * wr) * rr;
  const double emagr = 0.5 * (a * a + br * br + cr * cr);
  const double etotr = pr * entho + ecinr + emagr;
  const double ptotr = pr + emagr;
  const double vdotbr = ur * a + vr * br + wr * cr;

  const double cfastl = find_speed_fast(qL, 0, s);
  const double cfastr = find_speed_fast(qR, 0, s);

  const double sl = std::fmin(ul, ur) - std::fmax(cfastl, cfastr);
  const double sr = std::fmax(ul, ur) + std::fmax(cfastl, cfastr);

  const double rcl = rl * (ul - sl);
  const double rcr = rr * (sr - ur);

  const double ustar = (rcr * ur + rcl * ul + (ptotl - ptotr)) / (rcr + rcl);
  const double ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) / (rcr + rcl);

  // left star state
  const double rstarl = rl * (sl - ul) / (sl - ustar);
  double       estar = rl * (sl - ul) * (sl - ustar) - a * a;
  const double el = rl * (sl - ul) * (sl - ul) - a * a;
  double       vstarl, wstarl, bstarl, cstarl;
  if (std::fabs(estar) < 1e-4 * (a * a))
  {
    vstarl = vl;
    bstarl = bl;
    wstarl = wl;
    cstarl = cl;
  }
  else
  {
    vstarl = vl - a * bl * (ustar - ul) / estar;
    bstarl = bl * el / estar;
    wstarl = wl - a * cl * (ustar - ul) / estar;
    cstarl = cl * el / estar;
  }
  const double vdotbstarl = ustar * a + vstarl * bstarl + wstarl * cstarl;
  const double etotstarl =
    ((sl - ul) * etotl - ptotl * ul + ptotstar * ustar + a * (vdotbl - vdotbstarl)) / (sl - ustar);
  const double sqrrstarl = std::sqrt(rstarl);
  const double calfvenl = std::fabs(a) / sqrrstarl;
  const double sal = ustar - calfvenl;

  // right star state
  const double rstarr = rr * (sr - ur) / (sr - ustar);
  estar = rr * (sr - ur) * (sr - ustar) - a * a;
  const double er = rr * (sr - ur) * (sr - ur) - a * a;
  double       vstarr, wstarr, bstarr, cstarr;
  if (std::fabs(estar) < 1e-4 * (a * a))
  {
    vstarr = vr;
    bstarr = br;
    wstarr = wr;
    cstarr = cr;
  }
  else
  {
    vstarr = vr - a * br * (ustar - ur) / estar;
    bstarr = br * er / estar;
    wstarr = wr - a * cr * (ustar - ur) / estar;
    cstarr = cr * er / estar;
  }
  const double vdotbstarr = ustar * a + vstarr * bstarr + wstarr * cstarr;
  const double etotstarr =
    ((sr - ur) * etotr - ptotr * ur + ptotstar * ustar + a * (vdotbr - vdotbstarr)) / (sr - ustar);
  const double sqrrstarr = std::sqrt(rstarr);
  const double calfvenr = std::fabs(a) / sqrrstarr;
  const double sar = ustar + calfvenr;

  // double star state
  const double vstarstar =
    (sqrrstarl * vstarl + sqrrstarr * vstarr + sgnm * (bstarr - bstarl)) / (sqrrstarl + sqrrstarr);
  const double wstarstar =
    (sqrrstarl * wstarl + sqrrstarr * wstarr + sgnm * (cstarr - cstarl)) / (sqrrstarl + sqrrstarr);
  const double bstarstar =
    (sqrrstarl * bstarr + sqrrstarr * bstarl + sgnm * sqrrstarl * sqrrstarr * (vstarr - vstarl)) /
    (sqrrstarl + sqrrstarr);
  const double cstarstar =
    (sqrrstarl * cstarr + sqrrstarr * cstarl + sgnm * sqrrstarl * sqrrstarr * (wstarr - wstarl)) /
    (sqrrstarl + sqrrstarr);
  const double vdotbstarstar = ustar * a + vstarstar * bstarstar + wstarstar * cstarstar;
  const double etotstarstarl = etotstarl - sgnm * sqrrstarl * (vdotbstarl - vdotbstarstar);
  const double etotstarstarr = etotstarr + sgnm * sqrrstarr * (vdotbstarr - vdotbstarstar);

  double ro, uo, vo, wo, bo, co, ptoto, etoto, vdotbo;
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
  flux[IA] = 0.0;
  flux[IB] = bo * uo - a * vo;
  flux[IC] = co * uo - a * wo;
}

// riemann_mhd dispatch (models/RiemannSolvers_MHD.h:559-623). Returns 0, or -1 for an unknown id
// (the reference aborts there).
inline int
riemann_mhd(double * qL, double * qR, double * flux, const Settings & s)
{
  switch (s.riemann)
  {
    case RIEMANN_HLLD: riemann_hlld(qL, qR, flux, s); return 0;
    case RIEMANN_HLL: riemann_hll(qL, qR, flux, s); return 0;
    case RIEMANN_LLF: riemann_llf(qL, qR, flux, s); return 0;
    case RIEMANN_HLLC: riemann_hllc(qL, qR, flux, s); return 0;
    default: return -1;
  }
}

inline double
fmax4(double a0, double a1, double a2, double a3)
{
  double r = a0;
  r = (a1 > r) ? a1 : r;
  r = (a2 > r) ? a2 : r;
  r = (a3 > r) ? a3 : r;
  return r;
}
inline double
fmin4(double a0, double a1, double a2, double a3)
{
  double r = a0;
  r = (a1 < r) ? a1 : r;
  r = (a2 < r) ? a2 : r;
  r = (a3 < r) ? a3 : r;
  return r;
}
inline double
fmax5(double a0, double a1, double a2, double a3, double a4)
{
  double r = a0;
  r = (a1 > r) ? a1 : r;
  r = (a2 > r) ? a2 : r;
  r = (a3 > r) ? a3 : r;
  r = (a4 > r) ? a4 : r;
  return r;
}

// Slots of the 4 states entering the 2D magnetic Riemann problem (LL, RL, LR, RR) and of the 4
// reconstructed edge states (RT, LT, RB, LB). The numeric values only index local arrays.
enum : int
{
  SLL = 0,
  SRL = 1,
  SLR = 2,
  SRR = 3
};
enum : int
{
  ERT = 0,
  ELT = 1,
  ERB = 2,
  ELB = 3
};

// mag_riemann2d_hlld (models/RiemannSolvers_MHD.h:629-869), branchless region select.
inline double
mag_riemann2d_hlld(const double (*q)[8], const double * e, const Settings & s)
{
  const double *qLL = q[SLL], *qRL = q[SRL], *qLR = q[SLR], *qRR = q[SRR];
  const double  ELL = e[SLL], ERL = e[SRL], ELR = e[SLR], ERR = e[SRR];

  const double rLL = qLL[ID], pLL = qLL[IP], uLL = qLL[IU], vLL = qLL[IV], aLL = qLL[IA],
               bLL = qLL[IB], cLL = qLL[IC];
  const double rLR = qLR[ID], pLR = qLR[IP], uLR = qLR[IU], vLR = qLR[IV], aLR = qLR[IA],
               bLR = qLR[IB], cLR = qLR[IC];
  const double rRL = qRL[ID], pRL = qRL[IP], uRL = qRL[IU], vRL = qRL[IV], aRL = qRL[IA],
               bRL = qRL[IB], cRL = qRL[IC];
  const double rRR = qRR[ID], pRR = qRR[IP], uRR = qRR[IU], vRR = qRR[IV], aRR = qRR[IA],
               bRR = qRR[IB], cRR = qRR[IC];

  const double cFastLLx = find_speed_fast(qLL, 0, s);
  const double cFastLRx = find_speed_fast(qLR, 0, s);
  const double cFastRLx = find_speed_fast(qRL, 0, s);
  const double cFastRRx = find_speed_fast(qRR, 0, s);
  const double cFastLLy = find_speed_fast(qLL, 1, s);
  const double cFastLRy = find_speed_fast(qLR, 1, s);
  const double cFastRLy = find_speed_fast(qRL, 1, s);
  const double cFastRRy = find_speed_fast(qRR, 1, s);

  const double SL = fmin4(uLL, uLR, uRL, uRR) - fmax4(cFastLLx, cFastLRx, cFastRLx, cFastRRx);
  const double SR = fmax4(uLL, uLR, uRL, uRR) + fmax4(cFastLLx, cFastLRx, cFastRLx, cFastRRx);
  const double SB = fmin4(vLL, vLR, vRL, vRR) - fmax4(cFastLLy, cFastLRy, cFastRLy, cFastRRy);
  const double ST = fmax4(vLL, vLR, vRL, vRR) + fmax4(cFastLLy, cFastLRy, cFastRLy, cFastRRy);

  const double PtotLL = pLL + 0.5 * (aLL * aLL + bLL * bLL + cLL * cLL);
  const double PtotLR = pLR + 0.5 * (aLR * aLR + bLR * bLR + cLR * cLR);
  const double PtotRL = pRL + 0.5 * (aRL * aRL + bRL * bRL + cRL * cRL);
  const double PtotRR = pRR + 0.5 * (aRR * aRR + bRR * bRR + cRR * cRR);

  const double rcLLx = rLL * (uLL - SL);
  const double rcRLx = rRL * (SR - uRL);
  const double rcLRx = rLR * (uLR - SL);
  const double rcRRx = rRR * (SR - uRR);
  const double rcLLy = rLL * (vLL - SB);
  const double rcLRy = rLR * (ST - vLR);
  const double rcRLy = rRL * (vRL - SB);
  const double rcRRy = rRR * (ST - vRR);

  const double ustar =
    (rcLLx * uLL + rcLRx * uLR + rcRLx * uRL + rcRRx * uRR + (PtotLL - PtotRL + PtotLR - PtotRR)) /
    (rcLLx + rcLRx + rcRLx + rcRRx);
  const double vstar =
    (rcLLy * vLL + rcLRy * vLR + rcRLy * vRL + rcRRy * vRR + (PtotLL - PtotLR + PtotRL - PtotRR)) /
    (rcLLy + rcLRy + rcRLy + rcRRy);

  const double rstarLLx = rLL * (SL - uLL) / (SL - ustar);
  const double BstarLL = bLL * (SL - uLL) / (SL - ustar);
  const double rstarLLy = rLL * (SB - vLL) / (SB - vstar);
  const double AstarLL = aLL * (SB - vLL) / (SB - vstar);
  const double rstarLL = rLL * (SL - uLL) / (SL - ustar) * (SB - vLL) / (SB - vstar);
  const double EstarLLx = ustar * BstarLL - vLL * aLL;
  const double EstarLLy = uLL * bLL - vstar * AstarLL;
  const double EstarLL = ustar * BstarLL - vstar * AstarLL;

  const double rstarLRx = rLR * (SL - uLR) / (SL - ustar);
  const double BstarLR = bLR * (SL - uLR) / (SL - ustar);
  const double rstarLRy = rLR * (ST - vLR) / (ST - vstar);
  const double AstarLR = aLR * (ST - vLR) / (ST - vstar);
  const double rstarLR = rLR * (SL - uLR) / (SL - ustar) * (ST - vLR) / (ST - vstar);
  const double EstarLRx = ustar * BstarLR - vLR * aLR;
  const double EstarLRy = uLR * bLR - vstar * AstarLR;
  const double EstarLR = ustar * BstarLR - vstar * AstarLR;

  const double rstarRLx = rRL * (SR - uRL) / (SR - ustar);
  const double BstarRL = bRL * (SR - uRL) / (SR - ustar);
  const double rstarRLy = rRL * (SB - vRL) / (SB - vstar);
  const double AstarRL = aRL * (SB - vRL) / (SB - vstar);
  const double rstarRL = rRL * (SR - uRL) / (SR - ustar) * (SB - vRL) / (SB - vstar);
  const double EstarRLx = ustar * BstarRL - vRL * aRL;
  const double EstarRLy = uRL * bRL - vstar * AstarRL;
  const double EstarRL = ustar * BstarRL - vstar * AstarRL;

  const double rstarRRx = rRR * (SR - uRR) / (SR - ustar);
  const double BstarRR = bRR * (SR - uRR) / (SR - ustar);
  const double rstarRRy = rRR * (ST - vRR) / (ST - vstar);
  const double AstarRR = aRR * (ST - vRR) / (ST - vstar);
  const double rstarRR = rRR * (SR - uRR) / (SR - ustar) * (ST - vRR) / (ST - vstar);
  const double EstarRRx = ustar * BstarRR - vRR * aRR;
  const double EstarRRy = uRR * bRR - vstar * AstarRR;
  const double EstarRR = ustar * BstarRR - vstar * AstarRR;

  const double calfvenL = fmax5(std::fabs(aLR) / std::sqrt(rstarLRx),
                                std::fabs(AstarLR) / std::sqrt(rstarLR),
                                std::fabs(aLL) / std::sqrt(rstarLLx),
                                std::fabs(AstarLL) / std::sqrt(rstarLL),
                                s.smallc);
  const double calfvenR = fmax5(std::fabs(aRR) / std::sqrt(rstarRRx),
                                std::fabs(AstarRR) / std::sqrt(rstarRR),
                                std::fabs(aRL) / std::sqrt(rstarRLx),
                                std::fabs(AstarRL) / std::sqrt(rstarRL),
                                s.smallc);
  const double calfvenB = fmax5(std::fabs(bLL) / std::sqrt(rstarLLy),
                                std::fabs(BstarLL) / std::sqrt(rstarLL),
                                std::fabs(bRL) / std::sqrt(rstarRLy),
                                std::fabs(BstarRL) / std::sqrt(rstarRL),
                                s.smallc);
  const double calfvenT = fmax5(std::fabs(bLR) / std::sqrt(rstarLRy),
                                std::fabs(BstarLR) / std::sqrt(rstarLR),
                                std::fabs(bRR) / std::sqrt(rstarRRy),
                                std::fabs(BstarRR) / std::sqrt(rstarRR),
                                s.smallc);

  const double SAL = std::fmin(ustar - calfvenL, 0.0);
  const double SAR = std::fmax(ustar + calfvenR, 0.0);
  const double SAB = std::fmin(vstar - calfvenB, 0.0);
  const double SAT = std::fmax(vstar + calfvenT, 0.0);

  const double AstarT = (SAR * AstarRR - SAL * AstarLR) / (SAR - SAL);
  const double AstarB = (SAR * AstarRL - SAL * AstarLL) / (SAR - SAL);
  const double BstarR = (SAT * BstarRR - SAB * BstarRL) / (SAT - SAB);
  const double BstarL = (SAT * BstarLR - SAB * BstarLL) / (SAT - SAB);

  double E = 0, tmpE = 0;
  const double SB_pos = (1 + std::copysign(1.0, SB)) / 2, SB_neg = 1 - SB_pos;
  const double ST_pos = (1 + std::copysign(1.0, ST)) / 2, ST_neg = 1 - ST_pos;
  const double SL_pos = (1 + std::copysign(1.0, SL)) / 2, SL_neg = 1 - SL_pos;
  const double SR_pos = (1 + std::copysign(1.0, SR)) / 2, SR_neg = 1 - SR_pos;

  tmpE = (SAL * SAB * EstarRR - SAL * SAT * EstarRL - SAR * SAB * EstarLR + SAR * SAT * EstarLL) /
           (SAR - SAL) / (SAT - SAB) -
         SAT * SAB / (SAT - SAB) * (AstarT - AstarB) + SAR * SAL / (SAR - SAL) * (BstarR - BstarL);
  E += (SB_neg * ST_pos * SL_neg * SR_pos) * tmpE;

  tmpE = (SAR * EstarLLx - SAL * EstarRLx + SAR * SAL * (bRL - bLL)) / (SAR - SAL);
  tmpE = SL_pos * ELL + SL_neg * SR_neg * ERL + SL_neg * SR_pos * tmpE;
  E += SB_pos * tmpE;

  tmpE = (SAR * EstarLRx - SAL * EstarRRx + SAR * SAL * (bRR - bLR)) / (SAR - SAL);
  tmpE = SL_pos * ELR + SL_neg * SR_neg * ERR + SL_neg * SR_pos * tmpE;
  E += (SB_neg * ST_neg) * tmpE;

  tmpE = (SAT * EstarLLy - SAB * EstarLRy - SAT * SAB * (aLR - aLL)) / (SAT - SAB);
  E += (SB_neg * ST_pos * SL_pos) * tmpE;

  tmpE = (SAT * EstarRLy - SAB * EstarRRy - SAT * SAB * (aRR - aRL)) / (SAT - SAB);
  E += (SB_neg * ST_pos * SL_neg * SR_neg) * tmpE;

  return E;
}

// compute_emf<emfDir> (models/RiemannSolvers_MHD.h:890-1097). qEdge holds the reconstructed states
// indexed by ERT/ELT/ERB/ELB; emf_dir is 0 (EMFX), 1 (EMFY) or 2 (EMFZ).
inline double
compute_emf(const double (*qe)[8], int emf_dir, const Settings & s)
{
  const double *qRT = qe[ERT], *qLT = qe[ELT], *qRB = qe[ERB], *qLB = qe[ELB];
  double        qq[4][8];
  double *      qLL = qq[SLL], *qRL = qq[SRL], *qLR = qq[SLR], *qRR = qq[SRR];

  qLL[ID] = qRT[ID];
  qRL[ID] = qLT[ID];
  qLR[ID] = qRB[ID];
  qRR[ID] = qLB[ID];
  if (s.cIso > 0)
  {
    qLL[IP] = qLL[ID] * s.cIso * s.cIso;
    qRL[IP] = qRL[ID] * s.cIso * s.cIso;
    qLR[IP] = qLR[ID] * s.cIso * s.cIso;
    qRR[IP] = qRR[ID] * s.cIso * s.cIso;
  }
  else
  {
    qLL[IP] = qRT[IP];
    qRL[IP] = qLT[IP];
    qLR[IP] = qRB[IP];
    qRR[IP] = qLB[IP];
  }
  // (first parallel v, second parallel v, orthogonal v) and the same for B, per EMF direction.
  int iu, iv, iw, ia, ib, ic;
  if (emf_dir == 2)
  {
    iu = IU; iv = IV; iw = IW; ia = IA; ib = IB; ic = IC;
  }
  else if (emf_dir == 1)
  {
    iu = IW; iv = IU; iw = IV; ia = IC; ib = IA; ic = IB;
  }
  else
  {
    iu = IV; iv = IW; iw = IU; ia = IB; ib = IC; ic = IA;
  }
  qLL[IU] = qRT[iu];
  qRL[IU] = qLT[iu];
  qLR[IU] = qRB[iu];
  qRR[IU] = qLB[iu];
  qLL[IV] = qRT[iv];
  qRL[IV] = qLT[iv];
  qLR[IV] = qRB[iv];
  qRR[IV] = qLB[iv];
  qLL[IA] = 0.5 * (qRT[ia] + qLT[ia]);
  qRL[IA] = 0.5 * (qRT[ia] + qLT[ia]);
  qLR[IA] = 0.5 * (qRB[ia] + qLB[ia]);
  qRR[IA] = 0.5 * (qRB[ia] + qLB[ia]);
  qLL[IB] = 0.5 * (qRT[ib] + qRB[ib]);
  qRL[IB] = 0.5 * (qLT[ib] + qLB[ib]);
  qLR[IB] = 0.5 * (qRT[ib] + qRB[ib]);
  qRR[IB] = 0.5 * (qLT[ib] + qLB[ib]);
  qLL[IW] = qRT[iw];
  qRL[IW] = qLT[iw];
  qLR[IW] = qRB[iw];
  qRR[IW] = qLB[iw];
  qLL[IC] = qRT[ic];
  qRL[IC] = qLT[ic];
  qLR[IC] = qRB[ic];
  qRR[IC] = qLB[ic];

  double e[4];
  e[SLL] = qLL[IU] * qLL[IB] - qLL[IV] * qLL[IA];
  e[SRL] = qRL[IU] * qRL[IB] - qRL[IV] * qRL[IA];
  e[SLR] = qLR[IU] * qLR[IB] - qLR[IV] * qLR[IA];
  e[SRR] = qRR[IU] * qRR[IB] - qRR[IV] * qRR[IA];
  return mag_riemann2d_hlld(qq, e, s);
}

} // namespace oracle

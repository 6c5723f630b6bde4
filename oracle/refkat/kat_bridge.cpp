// Known-answer bridge (test infrastructure): exposes the reference's own per-cell math —
// models/mhd_utils.h, models/RiemannSolvers_MHD.h, models/HydroSettings.cpp, compiled unmodified
// from the reference tree — through a C ABI so tests can compare the oracle against it and so
// tests/golden/make_golden.py can record golden vectors. Built only where the reference tree is
// present; nothing in the product uses it.
#include <cstdio>
#include <cstdint>
#include <string>

#include <godunov_mhd_ct/models/RiemannSolvers_MHD.h>
#include <godunov_mhd_ct/models/mhd_utils.h>

using namespace kalypsso;
using namespace kalypsso::godunov_mhd_ct;

namespace
{
std::string
num(double x)
{
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.17g", x);
  return buf;
}

const char *
riemann_name(int id)
{
  switch (id)
  {
    case 2: return "LLF";
    case 3: return "HLL";
    case 4: return "HLLC";
    case 5: return "HLLD";
    default: return "UNKNOWN";
  }
}

MHDSettings
make(double gamma0, double slope_type, double smallr, double smallc, int riemann)
{
  ConfigMap cm;
  cm.set("hydro", "gamma0", num(gamma0));
  cm.set("hydro", "slope_type", num(slope_type));
  cm.set("hydro", "smallr", num(smallr));
  cm.set("hydro", "smallc", num(smallc));
  cm.set("hydro", "riemann", riemann_name(riemann));
  return MHDSettings(cm);
}

template <typename A>
void
load(A & a, const double * p)
{
  for (std::size_t i = 0; i < A::size(); ++i)
    a[i] = p[i];
}
} // namespace

extern "C" {

// derived settings: out = {gamma0, cfl, slope_type, smallr, smallc, smallp, smallpp, cIso, riemann}
void
ref_settings(double gamma0, double slope_type, double smallr, double smallc, int riemann, double * out)
{
  const MHDSettings s = make(gamma0, slope_type, smallr, smallc, riemann);
  out[0] = s.hydro.gamma0;
  out[1] = s.hydro.cfl;
  out[2] = s.hydro.slope_type;
  out[3] = s.hydro.smallr;
  out[4] = s.hydro.smallc;
  out[5] = s.hydro.smallp;
  out[6] = s.hydro.smallpp;
  out[7] = s.hydro.cIso;
  out[8] = static_cast<int>(s.hydro.riemannSolverType);
}

// flux = riemann_mhd(qL, qR) for n state pairs (8 doubles each). Components the solver does not
// write are returned as 0.
void
ref_riemann_batch(double gamma0, double smallr, double smallc, int riemann, int64_t n,
                  const double * qL, const double * qR, double * flux)
{
  const MHDSettings s = make(gamma0, 1.0, smallr, smallc, riemann);
  for (int64_t i = 0; i < n; ++i)
  {
    MHDStateCell l, r, f;
    load(l, qL + 8 * i);
    load(r, qR + 8 * i);
    for (int v = 0; v < 8; ++v)
      f[v] = 0.0;
    riemann_mhd(l, r, f, s);
    for (int v = 0; v < 8; ++v)
      flux[8 * i + v] = f[v];
  }
}

// emf = compute_emf<dir>(qEdge) for n edges; q holds, per edge, the states RT, LT, RB, LB.
void
ref_compute_emf_batch(double gamma0, double smallr, double smallc, int64_t n, int dir,
                      const double * q, double * out)
{
  const MHDSettings s = make(gamma0, 1.0, smallr, smallc, 5);
  for (int64_t i = 0; i < n; ++i)
  {
    MHDStateCell qe[4];
    load(qe[IRT], q + 32 * i + 0);
    load(qe[ILT], q + 32 * i + 8);
    load(qe[IRB], q + 32 * i + 16);
    load(qe[ILB], q + 32 * i + 24);
    if (dir == 0)
      out[i] = compute_emf<EMFX>(qe, s);
    else if (dir == 1)
      out[i] = compute_emf<EMFY>(qe, s);
    else
      out[i] = compute_emf<EMFZ>(qe, s);
  }
}

// q = compute_primitives(u), c = sound speed
void
ref_compute_primitives_batch(double gamma0, double smallr, double smallc, int64_t n,
                             const double * u, double * q, double * c)
{
  const MHDSettings s = make(gamma0, 1.0, smallr, smallc, 5);
  for (int64_t i = 0; i < n; ++i)
  {
    MHDStateCell uu;
    load(uu, u + 8 * i);
    real_t     cc = 0;
    const auto qq = models::mhd::compute_primitives(uu, cc, s);
    for (int v = 0; v < 8; ++v)
      q[8 * i + v] = qq[v];
    c[i] = cc;
  }
}

// find_speed_info<dim>
void
ref_find_speed_info_batch(double gamma0, int64_t n, int dim, const double * q, double * out)
{
  const MHDSettings s = make(gamma0, 1.0, 1e-10, 1e-10, 5);
  for (int64_t i = 0; i < n; ++i)
  {
    MHDStateCell qq;
    load(qq, q + 8 * i);
    if (dim == 2)
    {
      const auto v = models::mhd::find_speed_info<2>(qq, s);
      out[3 * i + 0] = v[0];
      out[3 * i + 1] = v[1];
      out[3 * i + 2] = 0.0;
    }
    else
    {
      const auto v = models::mhd::find_speed_info<3>(qq, s);
      out[3 * i + 0] = v[0];
      out[3 * i + 1] = v[1];
      out[3 * i + 2] = v[2];
    }
  }
}

// find_speed_fast<dir>
void
ref_find_speed_fast_batch(double gamma0, int64_t n, int dir, const double * q, double * out)
{
  const MHDSettings s = make(gamma0, 1.0, 1e-10, 1e-10, 5);
  for (int64_t i = 0; i < n; ++i)
  {
    MHDStateCell qq;
    load(qq, q + 8 * i);
    out[i] = dir == 0 ? models::mhd::find_speed_fast<IX>(qq, s)
                      : (dir == 1 ? models::mhd::find_speed_fast<IY>(qq, s)
                                  : models::mhd::find_speed_fast<IZ>(qq, s));
  }
}

} // extern "C"

// Functor bridge (test infrastructure): runs the reference's own stage functors — limited slopes,
// Hancock predictor, edge electric field, half-step face source, face fluxes and edge EMFs
// (scheme/*Functor.cpp, compiled unmodified from the reference tree against the stub headers in
// shim/) — on one block whose ghosted stage inputs come from the caller, so that tests can compare the oracle's
// restatement of those stages with the reference code itself. Built only where the reference tree
// is present; nothing in the product uses it.
#include <cstdio>
#include <cstring>
#include <string>

#include <godunov_mhd_ct/scheme/ComputeElectricFieldFunctor.h>
#include <godunov_mhd_ct/scheme/ComputeEmfAndStoreFunctor.h>
#include <godunov_mhd_ct/scheme/ComputeHydroFluxesAndStoreFunctor.h>
#include <godunov_mhd_ct/scheme/ComputeLimitedSlopesFunctor.h>
#include <godunov_mhd_ct/scheme/ComputeSourceFaceMagFunctor.h>
#include <godunov_mhd_ct/scheme/ComputeUpdatedPrimitiveVariablesFunctor.h>

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

template <std::size_t dim>
int
run(const int * b, int level, const double * prm, const int * flags, const double * grav, double dt, const double * q_in,
    double * slopes, double * q2, double * efield, double * sf)
{
  // prm: gamma0, slope_type, smallr, smallc, scaling_factor, mu; flags: riemann, rk2, gravity, viscosity, predictor
  ConfigMap cm;
  const char * rs[] = {"UNKNOWN", "APPROX", "LLF", "HLL", "HLLC", "HLLD"};
  cm.set("hydro", "gamma0", num(prm[0]));
  cm.set("hydro", "slope_type", num(prm[1]));
  cm.set("hydro", "smallr", num(prm[2]));
  cm.set("hydro", "smallc", num(prm[3]));
  cm.set("hydro", "riemann", rs[flags[0]]);
  cm.set("mesh", "scaling_factor", num(prm[4]));
  cm.set("amr", "time_integrator", flags[1] ? "RK2_SSP" : "HANCOCK");
  cm.set("gravity", "enabled", flags[2] ? "true" : "false");
  cm.set("gravity", "uniform_gx", num(grav[0]));
  cm.set("gravity", "uniform_gy", num(grav[1]));
  cm.set("gravity", "uniform_gz", num(grav[2]));
  cm.set("viscosity", "enabled", flags[3] ? "true" : "false");
  cm.set("viscosity", "mu", num(prm[5]));
  cm.set("viscosity", "hancock_predictor_enabled", flags[4] ? "true" : "false");
  const MHDSettings     st(cm);
  const ViscosityParams visc(cm);
  FieldMap<models::MHD> fm;

  using Arr = DataArrayGhostedBlock<dim, real_t, DefaultDevice>;
  block_size_t<dim> bs;
  for (std::size_t d = 0; d < dim; ++d)
    bs[d] = b[d];
  const int nvs = 8, nsf = dim == 3 ? 3 : 2, ne = dim == 3 ? 3 : 1;
  Arr q(bs, 2, 11, 1), sx(bs, 1, nvs, 1), sy(bs, 1, nvs, 1), sz(bs, 1, nvs, 1), qq2(bs, 1, nvs, 1),
    e(bs, 2, ne, 1), s(bs, 1, nsf, 1);
  std::memcpy(q.data(), q_in, sizeof(double) * q.num_cells() * 11);
  typename orchard_key_base_t<DefaultDevice>::view_t keys;
  keys.keys->push_back((uint64_t)level);

  ComputeLimitedSlopesFunctor<dim, DefaultDevice>::apply_on_group(q, sx, sy, sz, fm, 1, st);
  ComputeUpdatedPrimitiveVariablesFunctor<dim, DefaultDevice>::apply_on_group(cm, keys, q, qq2, sx, sy, sz, fm, 1, st,
                                                                             visc, dt);
  ComputeElectricFieldFunctor<dim, DefaultDevice>::apply_on_group(q, e, fm, 1);
  ComputeSourceFaceMagFunctor<dim, DefaultDevice>::apply_on_group(s, e, fm, 1, dt, cm, keys);

  const std::size_t ns = (std::size_t)sx.num_cells() * nvs;
  std::memcpy(slopes, sx.data(), sizeof(double) * ns);
  std::memcpy(slopes + ns, sy.data(), sizeof(double) * ns);
  if (dim == 3)
    std::memcpy(slopes + 2 * ns, sz.data(), sizeof(double) * ns);
  std::memcpy(q2, qq2.data(), sizeof(double) * ns);
  std::memcpy(efield, e.data(), sizeof(double) * e.num_cells() * ne);
  std::memcpy(sf, s.data(), sizeof(double) * s.num_cells() * nsf);
  return 0;
}

// settings + config of a bridge call (prm, flags, grav as in run())
ConfigMap
config_of(const double * prm, const int * flags, const double * grav)
{
  ConfigMap    cm;
  const char * rs[] = {"UNKNOWN", "APPROX", "LLF", "HLL", "HLLC", "HLLD"};
  cm.set("hydro", "gamma0", num(prm[0]));
  cm.set("hydro", "slope_type", num(prm[1]));
  cm.set("hydro", "smallr", num(prm[2]));
  cm.set("hydro", "smallc", num(prm[3]));
  cm.set("hydro", "riemann", rs[flags[0]]);
  cm.set("mesh", "scaling_factor", num(prm[4]));
  cm.set("amr", "time_integrator", flags[1] ? "RK2_SSP" : "HANCOCK");
  cm.set("gravity", "enabled", flags[2] ? "true" : "false");
  cm.set("gravity", "uniform_gx", num(grav[0]));
  cm.set("gravity", "uniform_gy", num(grav[1]));
  cm.set("gravity", "uniform_gz", num(grav[2]));
  cm.set("viscosity", "enabled", flags[3] ? "true" : "false");
  cm.set("viscosity", "mu", num(prm[5]));
  cm.set("viscosity", "hancock_predictor_enabled", flags[4] ? "true" : "false");
  return cm;
}

template <std::size_t dim>
int
run_fluxes(const int * b, int level, const double * prm, const int * flags, const double * grav, double dt,
           const double * q_in, const double * q2_in, const double * slopes_in, const double * sf_in, double * fluxes,
           double * emf)
{
  const ConfigMap       cm = config_of(prm, flags, grav);
  const MHDSettings     st(cm);
  FieldMap<models::MHD> fm;
  AMRMeshInfo           info;
  using Arr = DataArrayGhostedBlock<dim, real_t, DefaultDevice>;
  block_size_t<dim> bs;
  for (std::size_t d = 0; d < dim; ++d)
    bs[d] = b[d];
  const int nsf = dim == 3 ? 3 : 2;
  Arr       q(bs, 2, 11, 1), q2(bs, 1, 8, 1), sx(bs, 1, 8, 1), sy(bs, 1, 8, 1), sz(bs, 1, 8, 1), sf(bs, 1, nsf, 1);
  const std::size_t n1 = (std::size_t)sx.num_cells() * 8;
  std::memcpy(q.data(), q_in, sizeof(double) * q.num_cells() * 11);
  std::memcpy(q2.data(), q2_in, sizeof(double) * n1);
  std::memcpy(sx.data(), slopes_in, sizeof(double) * n1);
  std::memcpy(sy.data(), slopes_in + n1, sizeof(double) * n1);
  if (dim == 3)
    std::memcpy(sz.data(), slopes_in + 2 * n1, sizeof(double) * n1);
  std::memcpy(sf.data(), sf_in, sizeof(double) * sf.num_cells() * nsf);
  typename orchard_key_base_t<DefaultDevice>::view_t keys;
  keys.keys->push_back((uint64_t)level);

  // face fluxes per direction, 8 variables on the (b + 1 along the direction) face box
  std::size_t off = 0;
  for (int dir = 0; dir < (int)dim; ++dir)
  {
    block_size_t<dim> fs = bs;
    fs[dir]++;
    Arr f(fs, 0, 8, 1);
    ComputeHydroFluxesAndStoreFunctor<dim, DefaultDevice>::apply(cm, keys, info, f, q, q2, sx, sy, sz, sf, fm, 0, 1, dir,
                                                                 st, dt);
    std::memcpy(fluxes + off, f.data(), sizeof(double) * f.num_cells() * 8);
    off += (std::size_t)f.num_cells() * 8;
  }
  // raw edge EMFs on the (b + 1)^d edge box, components by edge direction (2D: along z)
  block_size_t<dim> es;
  for (std::size_t d = 0; d < dim; ++d)
    es[d] = b[d] + 1;
  Arr e(es, 0, 3, 1);
  ComputeEmfAndStoreFunctor<dim, DefaultDevice>::apply(cm, keys, info, e, q, q2, sx, sy, sz, sf, fm, 0, 1, st, dt);
  std::memcpy(emf, e.data(), sizeof(double) * e.num_cells() * 3);
  return 0;
}
} // namespace

extern "C" {

// One block: the ghosted stage arrays (as ref_block_stages returns them) in, the reference's face
// fluxes (times dt/dx; per direction [8][faces], directions concatenated) and raw edge EMFs (times
// dt/dx; [3][(b+1)^d], components by edge direction) out.
int
ref_block_fluxes_emf(int dim, const int * b, int level, const double * prm, const int * flags, const double * grav,
                     double dt, const double * q, const double * q2, const double * slopes, const double * sf,
                     double * fluxes, double * emf)
{
  if (dim == 2)
    return run_fluxes<2>(b, level, prm, flags, grav, dt, q, q2, slopes, sf, fluxes, emf);
  if (dim == 3)
    return run_fluxes<3>(b, level, prm, flags, grav, dt, q, q2, slopes, sf, fluxes, emf);
  return -1;
}


// One block: q_in [11][(b+4)^d] ghosted primitives (ghost width 2; variable-major, x fastest) in, the
// reference's slopes [dim][8][(b+2)^d], predictor [8][(b+2)^d], edge field [ncomp][(b+4)^d] and face
// source [2|3][(b+2)^d] out.
int
ref_block_stages(int dim, const int * b, int level, const double * prm, const int * flags, const double * grav,
                 double dt, const double * q_in, double * slopes, double * q2, double * efield, double * sf)
{
  if (dim == 2)
    return run<2>(b, level, prm, flags, grav, dt, q_in, slopes, q2, efield, sf);
  if (dim == 3)
    return run<3>(b, level, prm, flags, grav, dt, q_in, slopes, q2, efield, sf);
  return -1;
}

} // extern "C"

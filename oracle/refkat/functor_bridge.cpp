// Functor bridge (test infrastructure): runs the reference's own stage functors — limited slopes,
// Hancock predictor, edge electric field, half-step face source, face fluxes, edge EMFs, the CT
// update of the face field, the CFL reduction, the viscous face fluxes, the gravity source term, the
// conservative update by face fluxes (on coarse/fine meshes too), the border EMF correction, the
// primitive variables of a ghosted block with its ghost cells from same-level, finer and coarser leaves
// and the fill of the leaves beyond non-periodic domain borders (scheme/*Functor.cpp and
// border_conditions/FillOutside.cpp, compiled unmodified from the reference tree against the stub headers in
// shim/) — on one block whose ghosted stage inputs come from the caller, so that tests can compare the oracle's
// restatement of those stages with the reference code itself. Built only where the reference tree
// is present; nothing in the product uses it.
#include <cstdio>
#include <cstring>
#include <string>

#include <godunov_mhd_ct/scheme/ComputeElectricFieldFunctor.h>
#include <godunov_mhd_ct/scheme/ConvertToPrimitivesVariablesFunctor.h>
#include <godunov_mhd_ct/scheme/CorrectEmfAtBlockBorderFunctor.h>
#include <godunov_mhd_ct/scheme/ComputeEmfAndStoreFunctor.h>
#include <godunov_mhd_ct/scheme/ComputeHydroFluxesAndStoreFunctor.h>
#include <godunov_mhd_ct/scheme/ComputeLimitedSlopesFunctor.h>
#include <godunov_mhd_ct/scheme/ComputeSourceFaceMagFunctor.h>
#include <godunov_mhd_ct/scheme/ComputeUpdatedPrimitiveVariablesFunctor.h>
#include <godunov_mhd_ct/scheme/AddGravitySourceTerm.h>
#include <godunov_mhd_ct/scheme/ComputeDtMHDFunctor.h>
#include <godunov_mhd_ct/scheme/ComputeViscousFluxesAndStoreFunctor.h>
#include <godunov_mhd_ct/scheme/ReadEmfAndUpdateFunctor.h>
#include <godunov_mhd_ct/scheme/ReadFluxesAndConservativeUpdateFunctor.h>
#include <godunov_mhd_ct/border_conditions/FillOutside.h>

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
template <std::size_t dim>
int
run_viscous(const int * b, int level, const double * prm, const int * flags, const double * grav, double dt,
            const double * q_in, double * fluxes)
{
  const ConfigMap       cm = config_of(prm, flags, grav);
  const ViscosityParams visc(cm);
  FieldMap<models::MHD> fm;
  AMRMeshInfo           info;
  using Arr = DataArrayGhostedBlock<dim, real_t, DefaultDevice>;
  block_size_t<dim> bs;
  for (std::size_t d = 0; d < dim; ++d)
    bs[d] = b[d];
  Arr q(bs, 2, 11, 1);
  std::memcpy(q.data(), q_in, sizeof(double) * q.num_cells() * 11);
  typename orchard_key_base_t<DefaultDevice>::view_t keys;
  keys.keys->push_back((uint64_t)level);
  std::size_t off = 0;
  for (int dir = 0; dir < (int)dim; ++dir)
  {
    block_size_t<dim> fs = bs;
    fs[dir]++;
    Arr f(fs, 0, 8, 1);
    ComputeViscousFluxesAndStoreFunctor<dim, DefaultDevice>::apply(cm, keys, info, f, q, fm, 0, 1, dir, visc, dt);
    std::memcpy(fluxes + off, f.data(), sizeof(double) * f.num_cells() * 8);
    off += (std::size_t)f.num_cells() * 8;
  }
  return 0;
}

template <std::size_t dim>
int
run_inv_dt(const int * b, int n_blocks, const int * levels, const double * prm, const int * flags,
           const double * grav, const double * U_in, const double * B_in, double * inv_dt)
{
  const ConfigMap       cm = config_of(prm, flags, grav);
  const MHDSettings     st(cm);
  FieldMap<models::MHD> fm;
  block_size_t<dim>     bs;
  for (std::size_t d = 0; d < dim; ++d)
    bs[d] = b[d];
  DataArrayBlock<dim, real_t, DefaultDevice>     U(bs, 0, 5, n_blocks);
  FaceDataArrayBlock<dim, real_t, DefaultDevice> B(bs, n_blocks);
  std::memcpy(U.data(), U_in, sizeof(double) * (std::size_t)U.num_cells() * 5 * n_blocks);
  std::memcpy(B.data(), B_in, sizeof(double) * (std::size_t)B.num_elements_per_octant() * n_blocks);
  typename orchard_key_base_t<DefaultDevice>::view_t keys;
  for (int i = 0; i < n_blocks; ++i)
    keys.keys->push_back((uint64_t)levels[i]);
  real_t v = 0;
  ComputeDtMHDFunctor<dim, DefaultDevice>::apply(cm, keys, n_blocks, st, fm, bs, U, B, v);
  *inv_dt = v;
  return 0;
}

template <std::size_t dim>
int
run_gravity(const int * b, int n_blocks, const double * grav, double dt, const double * Uold_in, double * Unew_io)
{
  const double prm[6] = {1.4, 1.0, 1e-10, 1e-10, 1.0, 0.0};
  const int    flags[5] = {5, 0, 1, 0, 0};
  const ConfigMap       cm = config_of(prm, flags, grav);
  FieldMap<models::MHD> fm;
  block_size_t<dim>     bs;
  for (std::size_t d = 0; d < dim; ++d)
    bs[d] = b[d];
  DataArrayBlock<dim, real_t, DefaultDevice> Uold(bs, 0, 5, n_blocks), Unew(bs, 0, 5, n_blocks);
  const std::size_t                          n = (std::size_t)Uold.num_cells() * 5 * n_blocks;
  std::memcpy(Uold.data(), Uold_in, sizeof(double) * n);
  std::memcpy(Unew.data(), Unew_io, sizeof(double) * n);
  AddGravitySourceTerm<dim, DefaultDevice>::apply(cm, Uold, Unew, fm, n_blocks, dt);
  std::memcpy(Unew_io, Unew.data(), sizeof(double) * n);
  return 0;
}

template <std::size_t dim>
int
run_update(const int * b, const double * prm, const int * flags, const double * grav, double dt,
           const double * fluxes, double * U_io, double * B_io)
{
  const ConfigMap       cm = config_of(prm, flags, grav);
  const MHDSettings     st(cm);
  FieldMap<models::MHD> fm;
  AMRMeshInfo           info;
  block_size_t<dim>     bs;
  brick_size_t<dim>     bricks;
  Kokkos::Array<bool, dim> periodic;
  for (std::size_t d = 0; d < dim; ++d)
  {
    bs[d] = b[d];
    bricks[d] = 1;
    periodic[d] = true;
  }
  DataArrayBlock<dim, real_t, DefaultDevice>     U(bs, 0, 5, 1);
  FaceDataArrayBlock<dim, real_t, DefaultDevice> B(bs, 1);
  std::memcpy(U.data(), U_io, sizeof(double) * (std::size_t)U.num_cells() * 5);
  std::memcpy(B.data(), B_io, sizeof(double) * (std::size_t)B.num_elements_per_octant());
  typename orchard_key_base_t<DefaultDevice>::view_t keys;
  keys.keys->push_back(0);
  conformal_status_view_t<dim, DefaultDevice> status;
  status.bits->push_back(0); // conforming: no finer neighbour across any face
  typename hashmap_base_t<DefaultDevice>::map_t map;
  std::size_t                                   off = 0;
  for (int dir = 0; dir < (int)dim; ++dir)
  {
    block_size_t<dim> fs = bs;
    fs[dir]++;
    DataArrayBlock<dim, real_t, DefaultDevice> f(fs, 0, 8, 1);
    std::memcpy(f.data(), fluxes + off, sizeof(double) * f.num_cells() * 8);
    off += (std::size_t)f.num_cells() * 8;
    ReadFluxesAndConservativeUpdateFunctor<dim, DefaultDevice>::apply(cm, map, keys, status, info, U, B, f, fm, dir,
                                                                      bricks, periodic, st, dt);
  }
  std::memcpy(U_io, U.data(), sizeof(double) * (std::size_t)U.num_cells() * 5);
  std::memcpy(B_io, B.data(), sizeof(double) * (std::size_t)B.num_elements_per_octant());
  return 0;
}

template <std::size_t dim>
int
run_ct(const int * b, int n_blocks, const double * emf_in, double * B_io)
{
  block_size_t<dim> bs, es;
  for (std::size_t d = 0; d < dim; ++d)
  {
    bs[d] = b[d];
    es[d] = b[d] + 1;
  }
  FaceDataArrayBlock<dim, real_t, DefaultDevice> B(bs, n_blocks);
  DataArrayBlock<dim, real_t, DefaultDevice>     emf(es, 0, 3, n_blocks);
  const std::size_t                              nf = (std::size_t)B.num_elements_per_octant() * n_blocks;
  std::memcpy(B.data(), B_io, sizeof(double) * nf);
  std::memcpy(emf.data(), emf_in, sizeof(double) * (std::size_t)emf.num_cells() * 3 * n_blocks);
  AMRMeshInfo info;
  info.nb_owned = n_blocks;
  ReadEmfAndUpdateFunctor<dim, DefaultDevice>::apply(info, B, emf);
  std::memcpy(B_io, B.data(), sizeof(double) * nf);
  return 0;
}
// the bridge's mesh tables and the per-block flags derived from them (orchard keys = levels; one
// conformal-status bit per face whose neighbour region is split into finer leaves)
template <std::size_t dim>
struct MeshCtx
{
  BridgeMesh                                          mesh;
  typename hashmap_base_t<DefaultDevice>::map_t       map;
  typename orchard_key_base_t<DefaultDevice>::view_t  keys;
  conformal_status_view_t<dim, DefaultDevice>         status;
  AMRMeshInfo                                         info;
  brick_size_t<dim>                                   bricks;
  Kokkos::Array<bool, dim>                            periodic;

  MeshCtx(int n_blocks, int n_owned, const int * level, const int * neighbor, const int * fine, const int * coord)
  {
    mesh.dim = (int)dim;
    mesh.n_owned = n_owned;
    mesh.n_blocks = n_blocks;
    mesh.level = level;
    mesh.neighbor = neighbor;
    mesh.fine = fine;
    mesh.coord = coord;
    map.mesh = &mesh;
    for (int b = 0; b < n_blocks; ++b)
      keys.keys->push_back((uint64_t)level[b]);
    for (int b = 0; b < n_blocks; ++b)
    {
      uint8_t bits = 0;
      for (int f = 0; f < 2 * (int)dim; ++f)
      {
        int o[3] = {0, 0, 0};
        o[f / 2] = (f & 1) ? 1 : -1;
        const int s = (o[2] + 1) * 9 + (o[1] + 1) * 3 + (o[0] + 1);
        bool      finer = false;
        if (fine && b < n_owned && neighbor[(int64_t)b * 27 + s] < 0)
          for (int c = 0; c < 8; ++c)
            finer = finer || fine[((int64_t)b * 27 + s) * 8 + c] >= 0;
        bits |= (uint8_t)((finer ? 1 : 0) << f);
      }
      status.bits->push_back(bits);
    }
    info.nb_owned = n_owned;
    info.nb_ghosts = 0;
    info.nb_outside = n_blocks - n_owned;
    for (std::size_t d = 0; d < dim; ++d)
    {
      bricks[d] = 1;
      periodic[d] = true;
    }
  }
};

template <std::size_t dim>
int
run_correct_emf(const int * b, int n_blocks, int n_owned, const int * level, const int * neighbor, const int * fine,
                const int * coord, const double * emf_in, double * emf_out)
{
  MeshCtx<dim>      mc(n_blocks, n_owned, level, neighbor, fine, coord);
  ConfigMap         cm;
  block_size_t<dim> bs, es;
  for (std::size_t d = 0; d < dim; ++d)
  {
    bs[d] = b[d];
    es[d] = b[d] + 1;
  }
  DataArrayBlock<dim, real_t, DefaultDevice> emf(es, 0, 3, n_blocks), emf2(es, 0, 3, n_blocks);
  const std::size_t                          n = (std::size_t)emf.num_cells() * 3 * n_blocks;
  std::memcpy(emf.data(), emf_in, sizeof(double) * n);
  std::memcpy(emf2.data(), emf_in, sizeof(double) * n); // deep_copy(emf2, emf), GodunovImplemV0.cpp:606
  ParallelEnv pe;
  CorrectEmfAtBlockBorderFunctor<dim, DefaultDevice>::apply(cm, mc.map, mc.keys, mc.status, mc.info, bs, emf, emf2,
                                                            mc.bricks, mc.periodic, pe);
  std::memcpy(emf_out, emf2.data(), sizeof(double) * n);
  return 0;
}

template <std::size_t dim>
int
run_update_mesh(const int * b, int n_blocks, int n_owned, const int * level, const int * neighbor, const int * fine,
                const int * coord, const double * prm, const int * flags, const double * grav, double dt,
                const double * fluxes, double * U_io, double * B_io)
{
  MeshCtx<dim>          mc(n_blocks, n_owned, level, neighbor, fine, coord);
  const ConfigMap       cm = config_of(prm, flags, grav);
  const MHDSettings     st(cm);
  FieldMap<models::MHD> fm;
  block_size_t<dim>     bs;
  for (std::size_t d = 0; d < dim; ++d)
    bs[d] = b[d];
  DataArrayBlock<dim, real_t, DefaultDevice>     U(bs, 0, 5, n_owned);
  FaceDataArrayBlock<dim, real_t, DefaultDevice> B(bs, n_owned);
  std::memcpy(U.data(), U_io, sizeof(double) * (std::size_t)U.num_cells() * 5 * n_owned);
  std::memcpy(B.data(), B_io, sizeof(double) * (std::size_t)B.num_elements_per_octant() * n_owned);
  // fluxes [block][dir][8][faces] of every owned block, regrouped per direction
  std::size_t per_block = 0;
  for (int dir = 0; dir < (int)dim; ++dir)
  {
    std::size_t nf = 1;
    for (std::size_t d = 0; d < dim; ++d)
      nf *= (std::size_t)(b[d] + ((int)d == dir ? 1 : 0));
    per_block += 8 * nf;
  }
  std::size_t off = 0;
  for (int dir = 0; dir < (int)dim; ++dir)
  {
    block_size_t<dim> fs = bs;
    fs[dir]++;
    DataArrayBlock<dim, real_t, DefaultDevice> f(fs, 0, 8, n_blocks);
    const std::size_t                          nfb = (std::size_t)f.num_cells() * 8;
    for (int blk = 0; blk < n_owned; ++blk)
      std::memcpy(f.data() + nfb * blk, fluxes + per_block * blk + off, sizeof(double) * nfb);
    off += nfb;
    ReadFluxesAndConservativeUpdateFunctor<dim, DefaultDevice>::apply(cm, mc.map, mc.keys, mc.status, mc.info, U, B,
                                                                      f, fm, dir, mc.bricks, mc.periodic, st, dt);
  }
  std::memcpy(U_io, U.data(), sizeof(double) * (std::size_t)U.num_cells() * 5 * n_owned);
  std::memcpy(B_io, B.data(), sizeof(double) * (std::size_t)B.num_elements_per_octant() * n_owned);
  return 0;
}
template <std::size_t dim>
int
run_primitives(const int * b, int n_blocks, int n_owned, const int * level, const int * neighbor, const int * fine,
               const int * coord, const double * prm, int prolongation, const double * U_in, const double * Bg_in,
               int blk, double * q_out)
{
  MeshCtx<dim> mc(n_blocks, n_owned, level, neighbor, fine, coord);
  const int    flags[5] = {5, 0, 0, 0, 0};
  const double grav[3] = {0.0, 0.0, 0.0};
  ConfigMap    cm = config_of(prm, flags, grav);
  cm.set("amr", "cell_centered_prolongation_type", prolongation ? "EXTRAPOLATE_LINEAR_MINMOD" : "SIMPLE_COPY");
  const MHDSettings st(cm);
  block_size_t<dim> bs, gs;
  for (std::size_t d = 0; d < dim; ++d)
  {
    bs[d] = b[d];
    gs[d] = b[d] + 4;
  }
  DataArrayBlock<dim, real_t, DefaultDevice>      U(bs, 0, 5, n_blocks);
  FaceDataArrayBlock<dim, real_t, DefaultDevice>  Bg(gs, n_blocks, 2);
  DataArrayGhostedBlock<dim, real_t, DefaultDevice> q(bs, 2, 11, 1);
  std::memcpy(U.data(), U_in, sizeof(double) * (std::size_t)U.num_cells() * 5 * n_blocks);
  std::memcpy(Bg.data(), Bg_in, sizeof(double) * (std::size_t)Bg.num_elements_per_octant() * n_blocks);
  ParallelEnv pe;
  ConvertToPrimitivesVariablesFunctor<dim, DefaultDevice>::apply_on_group(cm, mc.map, mc.keys, mc.info, blk, 1, U, Bg,
                                                                          q, mc.bricks, mc.periodic, st, pe);
  std::memcpy(q_out, q.data(), sizeof(double) * (std::size_t)q.num_cells() * 11);
  return 0;
}
// keys of every block: level, coordinates at that level and, for the blocks beyond a non-periodic
// border, the axes along which they lie outside [0, bricks << level)
template <std::size_t dim>
std::vector<uint64_t>
block_keys(int n_blocks, const int * level, const int * coord, const int * bricks)
{
  std::vector<uint64_t> k((std::size_t)n_blocks);
  for (int b = 0; b < n_blocks; ++b)
  {
    int64_t  c[3] = {0, 0, 0};
    unsigned bits = 0;
    for (int a = 0; a < (int)dim; ++a)
    {
      c[a] = coord[3 * b + a];
      const int64_t e = (int64_t)bricks[a] << level[b];
      if (c[a] < 0 || c[a] >= e)
        bits |= 1u << a;
    }
    k[b] = orchard_key_t<dim>::pack(level[b], c, bits);
  }
  return k;
}

template <std::size_t dim>
int
run_fill_outside(const int * b, int n_blocks, int n_owned, const int * level, const int * neighbor, const int * coord,
                 const int * bc, double * U_io, double * B_io)
{
  MeshCtx<dim>      mc(n_blocks, n_owned, level, neighbor, nullptr, coord);
  const int         bricks[3] = {1, 1, 1};
  std::vector<uint64_t> keys = block_keys<dim>(n_blocks, level, coord, bricks);
  mc.mesh.keys = keys.data();
  mc.keys.keys->assign(keys.begin(), keys.end());
  ConfigMap    cm;
  const char * names[5] = {"NONE", "PERIODIC", "ZERO_GRADIENT", "WALL", "CUSTOM"};
  const char * faces[6] = {"xmin", "xmax", "ymin", "ymax", "zmin", "zmax"};
  const char * per[3] = {"periodic_x", "periodic_y", "periodic_z"};
  for (int f = 0; f < 2 * (int)dim; ++f)
    cm.set("border_conditions", faces[f], names[bc[f] >= 0 && bc[f] < 5 ? bc[f] : 0]);
  for (int a = 0; a < (int)dim; ++a)
    cm.set("p4est_connectivity", per[a], bc[2 * a] == 1 ? "1" : "0");
  block_size_t<dim> bs;
  for (std::size_t d = 0; d < dim; ++d)
    bs[d] = b[d];
  DataArrayBlock<dim, real_t, DefaultDevice>     U(bs, 0, 5, n_blocks);
  FaceDataArrayBlock<dim, real_t, DefaultDevice> B(bs, n_blocks);
  const std::size_t nu = (std::size_t)U.num_cells() * 5 * n_blocks;
  const std::size_t nb = (std::size_t)B.num_elements_per_octant() * n_blocks;
  std::memcpy(U.data(), U_io, sizeof(double) * nu);
  std::memcpy(B.data(), B_io, sizeof(double) * nb);
  FieldMap<models::MHD> fm;
  ParallelEnv           pe;
  FillOutsideCellFunctor<dim, DefaultDevice>::apply(U, B, mc.info, mc.keys, mc.map, fm, cm, pe);
  std::memcpy(U_io, U.data(), sizeof(double) * nu);
  std::memcpy(B_io, B.data(), sizeof(double) * nb);
  return 0;
}
} // namespace

extern "C" {

// The reference's fill of the leaves beyond non-periodic domain borders (FillOutsideCellFunctor::apply):
// mesh tables as for ref_correct_emf, the outside blocks after the owned ones with their coordinates
// beyond the domain (-1 or 2^level), border conditions bc[6] per domain face (0 NONE, 1 PERIODIC,
// 2 ZERO_GRADIENT, 3 WALL, 4 CUSTOM); U [n_blocks][5][cells] and B [n_blocks][faces] updated in place.
int
ref_fill_outside(int dim, const int * b, int n_blocks, int n_owned, const int * level, const int * neighbor,
                 const int * coord, const int * bc, double * U, double * B)
{
  if (dim == 2)
    return run_fill_outside<2>(b, n_blocks, n_owned, level, neighbor, coord, bc, U, B);
  if (dim == 3)
    return run_fill_outside<3>(b, n_blocks, n_owned, level, neighbor, coord, bc, U, B);
  return -1;
}

// The reference's primitive variables of owned block blk on its (b+4)^d ghosted box
// (ConvertToPrimitivesVariablesFunctor::apply_on_group, ghosts from same-level leaves, the sibling
// average of finer ones, a coarser one copied or extrapolated with minmod slopes): mesh tables as for
// ref_correct_emf, U [n_blocks][5][cells], Bg [n_blocks][ghosted faces] (per block the face arrays of a
// (b+4)^d cell box, first face at index -2, components concatenated), q_out [11][(b+4)^d].
int
ref_block_primitives(int dim, const int * b, int n_blocks, int n_owned, const int * level, const int * neighbor,
                     const int * fine, const int * coord, const double * prm, int prolongation, const double * U,
                     const double * Bg, int blk, double * q_out)
{
  if (dim == 2)
    return run_primitives<2>(b, n_blocks, n_owned, level, neighbor, fine, coord, prm, prolongation, U, Bg, blk, q_out);
  if (dim == 3)
    return run_primitives<3>(b, n_blocks, n_owned, level, neighbor, fine, coord, prm, prolongation, U, Bg, blk, q_out);
  return -1;
}

// The reference's border EMF correction (CorrectEmfAtBlockBorderFunctor::apply) on a mesh given by its
// tables (levels [n_blocks], neighbour table [n_blocks][27], children of finer regions [n_blocks][27][8]
// or NULL, coordinates [n_blocks][3]): emf_in [n_blocks][3][(b+1)^d] raw EMFs (components by edge
// direction, 2D: z), emf_out the corrected copy (only the owned blocks' border edges change).
int
ref_correct_emf(int dim, const int * b, int n_blocks, int n_owned, const int * level, const int * neighbor,
                const int * fine, const int * coord, const double * emf_in, double * emf_out)
{
  if (dim == 2)
    return run_correct_emf<2>(b, n_blocks, n_owned, level, neighbor, fine, coord, emf_in, emf_out);
  if (dim == 3)
    return run_correct_emf<3>(b, n_blocks, n_owned, level, neighbor, fine, coord, emf_in, emf_out);
  return -1;
}

// The reference's conservative update (ReadFluxesAndConservativeUpdateFunctor::apply per direction) of
// all owned blocks of a mesh given by its tables, coarse cells next to finer leaves taking the sum of
// the fine face fluxes: fluxes [n_owned][dir][8][faces] (times dt/dx), U [n_owned][5][cells] and B
// [n_owned][faces] (2D: the cell-centred Bz) updated in place.
int
ref_update_mesh(int dim, const int * b, int n_blocks, int n_owned, const int * level, const int * neighbor,
                const int * fine, const int * coord, const double * prm, const int * flags, const double * grav,
                double dt, const double * fluxes, double * U, double * B)
{
  if (dim == 2)
    return run_update_mesh<2>(b, n_blocks, n_owned, level, neighbor, fine, coord, prm, flags, grav, dt, fluxes, U, B);
  if (dim == 3)
    return run_update_mesh<3>(b, n_blocks, n_owned, level, neighbor, fine, coord, prm, flags, grav, dt, fluxes, U, B);
  return -1;
}

// One block: ghosted primitives q [11][(b+4)^d] (as ref_block_stages takes them) in, the reference's
// viscous face fluxes (times dt/dx; per direction [8][faces], directions concatenated) out.
int
ref_block_viscous_fluxes(int dim, const int * b, int level, const double * prm, const int * flags,
                         const double * grav, double dt, const double * q, double * fluxes)
{
  if (dim == 2)
    return run_viscous<2>(b, level, prm, flags, grav, dt, q, fluxes);
  if (dim == 3)
    return run_viscous<3>(b, level, prm, flags, grav, dt, q, fluxes);
  return -1;
}

// The reference's CFL reduction (ComputeDtMHDFunctor::apply) over n_blocks unghosted blocks of the
// C ABI layout: U [n_blocks][5][cells], B [n_blocks][Bx|By|Bz faces], block levels on the unit
// brick. Writes max over cells of the inverse time step (before the CFL number).
int
ref_inv_dt(int dim, const int * b, int n_blocks, const int * levels, const double * prm, const int * flags,
           const double * grav, const double * U, const double * B, double * inv_dt)
{
  if (dim == 2)
    return run_inv_dt<2>(b, n_blocks, levels, prm, flags, grav, U, B, inv_dt);
  if (dim == 3)
    return run_inv_dt<3>(b, n_blocks, levels, prm, flags, grav, U, B, inv_dt);
  return -1;
}

// The reference's gravity source term (AddGravitySourceTerm::apply): Unew [n_blocks][5][cells]
// updated in place from Uold, uniform field grav[3], time step dt.
int
ref_gravity_source(int dim, const int * b, int n_blocks, const double * grav, double dt, const double * Uold,
                   double * Unew)
{
  if (dim == 2)
    return run_gravity<2>(b, n_blocks, grav, dt, Uold, Unew);
  if (dim == 3)
    return run_gravity<3>(b, n_blocks, grav, dt, Uold, Unew);
  return -1;
}

// The reference's conservative update (ReadFluxesAndConservativeUpdateFunctor::apply, direction by
// direction) of one conforming block: U [5][cells] and faces B (2D: the cell-centred Bz) updated in
// place by the face fluxes (per direction [8][faces] concatenated, times dt/dx).
int
ref_block_update(int dim, const int * b, const double * prm, const int * flags, const double * grav, double dt,
                 const double * fluxes, double * U, double * B)
{
  if (dim == 2)
    return run_update<2>(b, prm, flags, grav, dt, fluxes, U, B);
  if (dim == 3)
    return run_update<3>(b, prm, flags, grav, dt, fluxes, U, B);
  return -1;
}

// The reference's CT update (ReadEmfAndUpdateFunctor::apply): B [n_blocks][Bx|By|Bz faces] (C ABI
// layout) updated in place by the curl of emf [n_blocks][3][(b+1)^d] (components by edge direction;
// 2D: along z), which already carries dt/dx.
int
ref_ct_update(int dim, const int * b, int n_blocks, const double * emf, double * B)
{
  if (dim == 2)
    return run_ct<2>(b, n_blocks, emf, B);
  if (dim == 3)
    return run_ct<3>(b, n_blocks, emf, B);
  return -1;
}

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

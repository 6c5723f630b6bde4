"""Record golden stage arrays from the reference's own stage functors.

Runs the functor bridge (oracle/refkat/functor_bridge.cpp: the reference's
ComputeLimitedSlopesFunctor, ComputeUpdatedPrimitiveVariablesFunctor, ComputeElectricFieldFunctor,
ComputeSourceFaceMagFunctor, ComputeHydroFluxesAndStoreFunctor, ComputeEmfAndStoreFunctor,
ReadEmfAndUpdateFunctor, ComputeDtMHDFunctor, ComputeViscousFluxesAndStoreFunctor,
AddGravitySourceTerm and ReadFluxesAndConservativeUpdateFunctor compiled unmodified against stub headers) on the
ghosted primitive variables the oracle builds for one block, and writes ``functor_stages.npz`` next
to this script: per case the mesh and state (U, B), dt, the settings, and the reference's slopes,
predictor, edge field, face source, face fluxes and raw edge EMFs (the fluxes and EMFs computed from
the reference's own stage arrays), the block's faces after the reference's CT update by those EMFs
(``ct_B``), the reference's CFL reduction over the mesh (``inv_dt``), with viscosity its viscous
face fluxes (``visc``) and with gravity its source term on the owned blocks (``grav_U``, inputs from
``gravity_inputs``), and the block's U and faces after the reference's conservative update by
those fluxes, then by the viscous ones (``upd_U``, ``upd_B``). Needs the reference tree (default /root/reference, or
$GMHD_REFERENCE_TREE); the committed npz is what tests use.

    python tests/golden/make_golden_stages.py
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from godunov_mhd_ct_gb300 import workloads as wl  # noqa: E402
from godunov_mhd_ct_gb300.mesh import BlockMesh  # noqa: E402
from oracle import oracle as orc  # noqa: E402

BRIDGE = os.path.join(ROOT, "oracle", "_ref", "libref_functors.so")

# name: dim, state, gamma, slope_type, rk2, gravity, viscosity mu (None: off), viscous predictor
CASES = {
    "2d_smooth_mc": (2, "smooth", 1.4, 2.0, 0, None, None, False),
    "2d_ot_minmod": (2, "ot", 5.0 / 3.0, 1.0, 0, None, None, False),
    "2d_blast_mc_grav_visc": (2, "blast", 5.0 / 3.0, 2.0, 0, (0.3, -0.7, 0.0), 2e-3, True),
    "2d_smooth_rk2": (2, "smooth", 1.4, 2.0, 1, None, None, False),
    "3d_smooth_mc": (3, "smooth", 1.4, 2.0, 0, None, None, False),
    "3d_ot_minmod_grav": (3, "ot", 5.0 / 3.0, 1.0, 0, (0.2, 0.1, -0.4), None, False),
    "3d_smooth_visc_pred": (3, "smooth", 1.4, 2.0, 0, None, 3e-3, True),
    "3d_smooth_rk2": (3, "smooth", 1.4, 2.0, 1, None, None, False),
}


def case_mesh(dim):
    if dim == 2:
        return BlockMesh.uniform(2, level=1, block=(8, 8, 1))
    return BlockMesh.uniform(3, level=1, block=(4, 4, 4))


def case_state(mesh, kind, gamma):
    if kind == "smooth":
        return wl.random_smooth(mesh, gamma=gamma, seed=17)
    if kind == "ot":
        return wl.orszag_tang(mesh, gamma=gamma, rho_perturbation=1e-3, seed=5)
    # front r = 0.3 around the domain centre (it crosses every block), three oracle steps on: the
    # initial step profile has zero limited slopes
    U, B = wl.blast(mesh, gamma=gamma, radius=0.3)
    st = orc.settings(gamma0=gamma, cfl=0.4, slope_type=2.0, riemann=5)
    U, B, _ = orc.run(orc.Mesh.from_block_mesh(mesh), st, U, B, 3)
    return U, B


def oracle_settings(gamma, slope, rk2, grav, mu, pred):
    return orc.settings(gamma0=gamma, cfl=0.4, slope_type=slope, riemann=5, time_integrator=rk2, gravity=grav,
                        viscosity_mu=mu, viscous_predictor=pred)


def reference_stages(dim, block, level, gamma, slope, rk2, grav, mu, pred, dt, q):
    """The reference functors on the oracle's ghosted primitives q of one block."""
    L = ctypes.CDLL(BRIDGE)
    dp = ctypes.POINTER(ctypes.c_double)
    b = (ctypes.c_int * 3)(*block)
    prm = (ctypes.c_double * 6)(gamma, slope, 1e-10, 1e-10, 1.0, 0.0 if mu is None else mu)
    flags = (ctypes.c_int * 5)(5, rk2, int(grav is not None), int(mu is not None), int(bool(pred)))
    g = (ctypes.c_double * 3)(*(tuple(grav) + (0.0,) * 3)[:3] if grav is not None else (0.0, 0.0, 0.0))
    n1 = int(np.prod([v + 2 for v in block[:dim]]))
    n2 = int(np.prod([v + 4 for v in block[:dim]]))
    out = {"slopes": np.zeros(dim * 8 * n1), "q2": np.zeros(8 * n1), "e": np.zeros((3 if dim == 3 else 1) * n2),
           "sf": np.zeros((3 if dim == 3 else 2) * n1)}
    q = np.ascontiguousarray(q, dtype=np.float64)
    rc = L.ref_block_stages(dim, b, level, prm, flags, g, ctypes.c_double(dt), q.ctypes.data_as(dp),
                            *(out[k].ctypes.data_as(dp) for k in ("slopes", "q2", "e", "sf")))
    if rc != 0:
        raise RuntimeError(f"ref_block_stages failed: {rc}")
    return out


def reference_fluxes_emf(dim, block, level, gamma, slope, rk2, grav, mu, pred, dt, stages):
    """The reference flux and EMF functors on the stage arrays `stages` (q, q2, slopes, sf) of one
    block: fluxes per direction [8][faces] concatenated, EMFs [3][(b+1)^d] by edge direction."""
    L = ctypes.CDLL(BRIDGE)
    dp = ctypes.POINTER(ctypes.c_double)
    b = (ctypes.c_int * 3)(*block)
    prm = (ctypes.c_double * 6)(gamma, slope, 1e-10, 1e-10, 1.0, 0.0 if mu is None else mu)
    flags = (ctypes.c_int * 5)(5, rk2, int(grav is not None), int(mu is not None), int(bool(pred)))
    g = (ctypes.c_double * 3)(*(tuple(grav) + (0.0,) * 3)[:3] if grav is not None else (0.0, 0.0, 0.0))
    nf = sum(int(np.prod([block[d] + (d == dr) for d in range(dim)])) for dr in range(dim))
    ne = int(np.prod([v + 1 for v in block[:dim]]))
    fl = np.zeros(8 * nf)
    emf = np.zeros(3 * ne)
    arrs = [np.ascontiguousarray(stages[k], dtype=np.float64) for k in ("q", "q2", "slopes", "sf")]
    rc = L.ref_block_fluxes_emf(dim, b, level, prm, flags, g, ctypes.c_double(dt), *(a.ctypes.data_as(dp) for a in arrs),
                                fl.ctypes.data_as(dp), emf.ctypes.data_as(dp))
    if rc != 0:
        raise RuntimeError(f"ref_block_fluxes_emf failed: {rc}")
    return fl, emf


def _bridge_args(gamma, slope, rk2, grav, mu, pred):
    prm = (ctypes.c_double * 6)(gamma, slope, 1e-10, 1e-10, 1.0, 0.0 if mu is None else mu)
    flags = (ctypes.c_int * 5)(5, rk2, int(grav is not None), int(mu is not None), int(bool(pred)))
    g = (ctypes.c_double * 3)(*(tuple(grav) + (0.0,) * 3)[:3] if grav is not None else (0.0, 0.0, 0.0))
    return prm, flags, g


def reference_viscous_fluxes(dim, block, level, gamma, slope, rk2, grav, mu, pred, dt, q):
    """The reference viscous flux functor (ComputeViscousFluxesAndStoreFunctor) on the ghosted
    primitives q of one block: per direction [8][faces], concatenated."""
    L = ctypes.CDLL(BRIDGE)
    dp = ctypes.POINTER(ctypes.c_double)
    b = (ctypes.c_int * 3)(*block)
    nf = sum(int(np.prod([block[d] + (d == dr) for d in range(dim)])) for dr in range(dim))
    fl = np.zeros(8 * nf)
    q = np.ascontiguousarray(q, dtype=np.float64)
    rc = L.ref_block_viscous_fluxes(dim, b, level, *_bridge_args(gamma, slope, rk2, grav, mu, pred), ctypes.c_double(dt),
                                    q.ctypes.data_as(dp), fl.ctypes.data_as(dp))
    if rc != 0:
        raise RuntimeError(f"ref_block_viscous_fluxes failed: {rc}")
    return fl


def reference_update(dim, block, gamma, slope, rk2, grav, mu, pred, dt, fluxes, Ublk, Bblk):
    """The reference conservative update (ReadFluxesAndConservativeUpdateFunctor, direction by
    direction) of one conforming block by its face fluxes, on copies; returns (U, B)."""
    L = ctypes.CDLL(BRIDGE)
    dp = ctypes.POINTER(ctypes.c_double)
    b = (ctypes.c_int * 3)(*block)
    U = np.array(Ublk, dtype=np.float64, copy=True)
    B = np.array(Bblk, dtype=np.float64, copy=True)
    fl = np.ascontiguousarray(fluxes, dtype=np.float64)
    rc = L.ref_block_update(dim, b, *_bridge_args(gamma, slope, rk2, grav, mu, pred), ctypes.c_double(dt),
                            fl.ctypes.data_as(dp), U.ctypes.data_as(dp), B.ctypes.data_as(dp))
    if rc != 0:
        raise RuntimeError(f"ref_block_update failed: {rc}")
    return U, B


def gravity_inputs(mesh, U):
    """(Uold, Unew) for the gravity source check: the owned blocks of U, and a copy with the density
    raised by 1 % and the momenta shifted (a stand-in for the hydro update)."""
    n = mesh.n_owned
    Uold = np.ascontiguousarray(U[:n], dtype=np.float64)
    Unew = Uold.copy()
    Unew[:, 0] *= 1.01
    Unew[:, 2:5] += 0.05
    return Uold, Unew


def reference_gravity(dim, block, grav, dt, Uold, Unew):
    """The reference gravity source term (AddGravitySourceTerm) on a copy of Unew."""
    L = ctypes.CDLL(BRIDGE)
    dp = ctypes.POINTER(ctypes.c_double)
    b = (ctypes.c_int * 3)(*block)
    g = (ctypes.c_double * 3)(*(tuple(grav) + (0.0,) * 3)[:3])
    Unew = np.array(Unew, dtype=np.float64, copy=True)
    Uold = np.ascontiguousarray(Uold, dtype=np.float64)
    rc = L.ref_gravity_source(dim, b, int(Unew.shape[0]), g, ctypes.c_double(dt), Uold.ctypes.data_as(dp),
                              Unew.ctypes.data_as(dp))
    if rc != 0:
        raise RuntimeError(f"ref_gravity_source failed: {rc}")
    return Unew


def reference_inv_dt(mesh, gamma, slope, rk2, grav, mu, pred, U, B):
    """The reference CFL reduction (ComputeDtMHDFunctor) over the owned blocks of `mesh`."""
    L = ctypes.CDLL(BRIDGE)
    dp = ctypes.POINTER(ctypes.c_double)
    n = mesh.n_owned
    b = (ctypes.c_int * 3)(*mesh.block)
    lev = np.ascontiguousarray(mesh.level[:n], dtype=np.int32)
    Uo = np.ascontiguousarray(U[:n], dtype=np.float64)
    Bo = np.ascontiguousarray(B[:n], dtype=np.float64)
    out = ctypes.c_double(0.0)
    rc = L.ref_inv_dt(mesh.dim, b, n, lev.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                      *_bridge_args(gamma, slope, rk2, grav, mu, pred), Uo.ctypes.data_as(dp), Bo.ctypes.data_as(dp),
                      ctypes.byref(out))
    if rc != 0:
        raise RuntimeError(f"ref_inv_dt failed: {rc}")
    return out.value


def reference_ct(dim, block, emf, B):
    """The reference CT update (ReadEmfAndUpdateFunctor) of one block's faces B by its edge EMFs
    emf [3][(b+1)^d] (2D: component 2 is the z one). Returns the updated B."""
    L = ctypes.CDLL(BRIDGE)
    dp = ctypes.POINTER(ctypes.c_double)
    b = (ctypes.c_int * 3)(*block)
    B = np.array(B, dtype=np.float64, copy=True)
    emf = np.ascontiguousarray(emf, dtype=np.float64)
    rc = L.ref_ct_update(dim, b, 1, emf.ctypes.data_as(dp), B.ctypes.data_as(dp))
    if rc != 0:
        raise RuntimeError(f"ref_ct_update failed: {rc}")
    return B


def main():
    if not orc.build_refkat() or not os.path.exists(BRIDGE):
        sys.exit("the reference tree is needed to record the golden stages")
    out = {}
    for name, (dim, kind, gamma, slope, rk2, grav, mu, pred) in CASES.items():
        mesh = case_mesh(dim)
        U, B = case_state(mesh, kind, gamma)
        om = orc.Mesh.from_block_mesh(mesh)
        st = oracle_settings(gamma, slope, rk2, grav, mu, pred)
        dt = 0.4 / orc.inv_dt(om, st, U, B)
        blk = 1
        q = orc.block_stages(om, st, U, B, dt, blk)["q"]
        ref = reference_stages(dim, mesh.block, int(mesh.level[blk]), gamma, slope, rk2, grav, mu, pred, dt, q)
        ref["fluxes"], ref["emf"] = reference_fluxes_emf(dim, mesh.block, int(mesh.level[blk]), gamma, slope, rk2,
                                                         grav, mu, pred, dt, dict(ref, q=q))
        if mu is not None:
            ref["visc"] = reference_viscous_fluxes(dim, mesh.block, int(mesh.level[blk]), gamma, slope, rk2, grav, mu,
                                                   pred, dt, q)
        if grav is not None:
            ref["grav_U"] = reference_gravity(dim, mesh.block, grav, dt, *gravity_inputs(mesh, U))
        args = (dim, mesh.block, gamma, slope, rk2, grav, mu, pred, dt)
        ref["upd_U"], ref["upd_B"] = reference_update(*args, ref["fluxes"], U[blk], B[blk])
        if mu is not None:
            ref["upd_U"], ref["upd_B"] = reference_update(*args, ref["visc"], ref["upd_U"], ref["upd_B"])
        ref["inv_dt"] = np.float64(reference_inv_dt(mesh, gamma, slope, rk2, grav, mu, pred, U, B))
        ref["ct_B"] = reference_ct(dim, mesh.block, ref["emf"], B[blk])
        out[f"{name}_U"] = U
        out[f"{name}_B"] = B
        out[f"{name}_dt"] = np.float64(dt)
        out[f"{name}_q"] = q
        for k, v in ref.items():
            out[f"{name}_{k}"] = v
    path = os.path.join(HERE, "functor_stages.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({len(CASES)} cases)")


if __name__ == "__main__":
    main()

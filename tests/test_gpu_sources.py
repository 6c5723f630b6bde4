"""Gravity and viscosity source terms on the GPU against the oracle.

FP64 path bit for bit: the Hancock predictor's gravity kick and viscous term
(ComputeUpdatedPrimitiveVariablesFunctor.cpp:174-280, 372-383, 505-517), the viscous face fluxes
applied after the hydro fluxes (ComputeViscousFluxesAndStoreFunctor.cpp:168-344,
GodunovImplemV0.cpp:179-192; on coarse/fine meshes the fine-side flux sums), the gravity source
after the update (AddGravitySourceTerm.cpp:47-99) and the CFL with gravity and viscosity
(ComputeDtMHDFunctor.cpp:86-249), on uniform and coarse/fine meshes, Hancock and RK2_SSP. The mixed
path stays within its tolerance.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_mhd_ct_gb300 import _native as nat  # noqa: E402
from godunov_mhd_ct_gb300 import workloads as wl  # noqa: E402
from godunov_mhd_ct_gb300.mesh import BlockMesh  # noqa: E402
from godunov_mhd_ct_gb300.solver import GodunovImplemGB300  # noqa: E402

from .helpers import l1_rel, oracle_settings, same_level_face_mismatch, settings  # noqa: E402
from .test_gpu_amr import MESHES  # noqa: E402

pytestmark = pytest.mark.gpu

SOURCES = {
    "gravity": dict(gravity=(0.4, -0.9, 0.3)),
    "viscosity": dict(viscosity_mu=2e-3),
    "viscous_predictor": dict(viscosity_mu=2e-3, viscous_predictor=True),
    "both": dict(gravity=(-0.5, 0.7, -0.2), viscosity_mu=1e-3, viscous_predictor=True),
}

UNIFORM = {
    "2d_b16": lambda: BlockMesh.uniform(2, level=2, block=(16, 16, 1)),
    "2d_b8": lambda: BlockMesh.uniform(2, level=2, block=(8, 8, 1)),
    "3d_b8": lambda: BlockMesh.uniform(3, level=1, block=(8, 8, 8)),
    "3d_b4": lambda: BlockMesh.uniform(3, level=1, block=(4, 4, 4)),
}


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _settings(src, **kw):
    st = settings(gamma0=1.4, cfl=0.4, **kw)
    st.gravity = src.get("gravity")
    st.viscosity_mu = src.get("viscosity_mu")
    st.viscous_predictor = src.get("viscous_predictor", False)
    return st


@pytest.mark.parametrize("name", sorted(UNIFORM))
@pytest.mark.parametrize("src", sorted(SOURCES))
def test_sources_step_fp64_bit_exact(oracle_lib, name, src):
    mesh = UNIFORM[name]()
    st = _settings(SOURCES[src])
    U, B = wl.random_smooth(mesh, seed=21)
    om = oracle_lib.Mesh.from_block_mesh(mesh)
    ost = oracle_settings(oracle_lib, st)
    dt = 0.4 / oracle_lib.inv_dt(om, ost, U, B)
    Uo, Bo = oracle_lib.step(om, ost, U, B, dt)
    impl = GodunovImplemGB300(st, mesh, precision="fp64")
    dU, dB = _dev(U), _dev(B)
    dU2, dB2 = dU.clone(), dB.clone()
    impl.do_time_step(dU, dU2, dB, dB2, dt)
    torch.cuda.synchronize()
    n = mesh.n_owned
    assert np.array_equal(dU2.cpu().numpy()[:n], Uo[:n])
    assert np.array_equal(dB2.cpu().numpy()[:n], Bo[:n])
    # the CFL with the source terms
    assert impl.compute_inv_dt(dU, dB) == oracle_lib.inv_dt(om, ost, U, B)


@pytest.mark.parametrize("name", ["2d_b16", "3d_b8"])
@pytest.mark.parametrize("integrator", ["HANCOCK", "RK2_SSP"])
def test_sources_run_fp64_bit_exact(oracle_lib, name, integrator):
    """Solver loop (CUDA graph, device dt from the fused CFL) against the oracle's run."""
    mesh = UNIFORM[name]()
    st = _settings(SOURCES["both"])
    st.time_integrator = integrator
    U, B = wl.random_smooth(mesh, seed=23)
    nsteps = 5
    Uo, Bo, dto = oracle_lib.run(oracle_lib.Mesh.from_block_mesh(mesh), oracle_settings(oracle_lib, st), U, B, nsteps)
    impl = GodunovImplemGB300(st, mesh, precision="fp64")
    dU, dB = _dev(U), _dev(B)
    dtg, _ = impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), nsteps)
    n = mesh.n_owned
    assert np.array_equal(dtg[:, 0], dto)
    assert np.array_equal(dU.cpu().numpy()[:n], Uo[:n])
    assert np.array_equal(dB.cpu().numpy()[:n], Bo[:n])


@pytest.mark.parametrize("name", sorted(MESHES))
@pytest.mark.parametrize("src", ["viscosity", "both"])
def test_sources_amr_step_fp64_bit_exact(oracle_lib, name, src):
    """Coarse/fine meshes: the viscous fluxes of coarse cells next to finer blocks are the fine-side
    sums, as the hydro fluxes."""
    mesh = MESHES[name]()
    st = _settings(SOURCES[src])
    U, B = wl.random_smooth(mesh, seed=25)
    om = oracle_lib.Mesh.from_block_mesh(mesh)
    ost = oracle_settings(oracle_lib, st)
    dt = 0.4 / oracle_lib.inv_dt(om, ost, U, B)
    Uo, Bo = oracle_lib.step(om, ost, U, B, dt)
    impl = GodunovImplemGB300(st, mesh, precision="fp64")
    dU, dB = _dev(U), _dev(B)
    dU2, dB2 = dU.clone(), dB.clone()
    impl.do_time_step(dU, dU2, dB, dB2, dt)
    torch.cuda.synchronize()
    assert impl.last_status() & ~16 == 0
    n = mesh.n_owned
    assert np.array_equal(dU2.cpu().numpy()[:n], Uo[:n])
    assert np.array_equal(dB2.cpu().numpy()[:n], Bo[:n])


@pytest.mark.parametrize("name", ["2d_b16", "3d_b8", "3d_b4"])
def test_sources_mixed_accuracy(oracle_lib, name):
    mesh = UNIFORM[name]()
    st = _settings(SOURCES["both"])
    U, B = wl.random_smooth(mesh, seed=27)
    nsteps = 10
    Uo, Bo, _ = oracle_lib.run(oracle_lib.Mesh.from_block_mesh(mesh), oracle_settings(oracle_lib, st), U, B, nsteps)
    impl = GodunovImplemGB300(st, mesh, precision="mixed")
    dU, dB = _dev(U), _dev(B)
    impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), nsteps)
    n = mesh.n_owned
    Ug, Bg = dU.cpu().numpy(), dB.cpu().numpy()
    assert l1_rel(Ug[:n, 0], Uo[:n, 0]) <= 1e-6
    assert l1_rel(Ug[:n, 1], Uo[:n, 1]) <= 1e-6
    assert l1_rel(Ug[:n, 2], Uo[:n, 2]) <= 1e-5
    assert same_level_face_mismatch(mesh, Bg) == 0.0


def test_sources_amr_mixed(oracle_lib):
    mesh = MESHES["3d_b8"]()
    st = _settings(SOURCES["both"])
    U, B = wl.random_smooth(mesh, seed=29)
    nsteps = 6
    Uo, _, _ = oracle_lib.run(oracle_lib.Mesh.from_block_mesh(mesh), oracle_settings(oracle_lib, st), U, B, nsteps)
    impl = GodunovImplemGB300(st, mesh, precision="mixed")
    dU, dB = _dev(U), _dev(B)
    impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), nsteps)
    n = mesh.n_owned
    assert l1_rel(dU.cpu().numpy()[:n, 0], Uo[:n, 0]) <= 1e-6


@pytest.mark.parametrize("src", ["gravity", "viscosity", "both"])
def test_noalloc_cfl_with_sources(oracle_lib, src):
    mesh = UNIFORM["3d_b8"]()
    st = _settings(SOURCES[src])
    U, B = wl.random_smooth(mesh, seed=31)
    dU, dB = _dev(U), _dev(B)
    p = nat.GmhdParams(st.gamma0, st.cfl, st.slope_type, st.smallr, st.smallc, mesh.scaling_factor, st.riemann_id, 0)
    if st.gravity is not None:
        p.gravity_enabled = 1
        p.gravity = (ctypes.c_double * 3)(*st.gravity)
    if st.viscosity_mu is not None:
        p.viscosity_enabled = 1
        p.viscosity_mu = st.viscosity_mu
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    nat.check(nat.lib().gmhd_inv_dt_noalloc(ctypes.byref(p), mesh.dim, 8, 8, 8, mesh.n_owned, int(mesh.level[0]), None,
                                            1, dU.data_ptr(), dB.data_ptr(), out.data_ptr(), None), "noalloc")
    torch.cuda.synchronize()
    want = oracle_lib.inv_dt(oracle_lib.Mesh.from_block_mesh(mesh), oracle_settings(oracle_lib, st), U, B)
    assert float(out.cpu()[0]) == want

"""RK2_SSP on the GPU (gmhd_advance with time_integrator RK2_SSP) against the oracle's RK2 loop."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_mhd_ct_gb300 import workloads as wl  # noqa: E402
from godunov_mhd_ct_gb300.mesh import BlockMesh  # noqa: E402
from godunov_mhd_ct_gb300.solver import GodunovImplemGB300  # noqa: E402

from .helpers import l1_rel, oracle_settings, settings  # noqa: E402
from .test_gpu_amr import MESHES  # noqa: E402

pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


CASES = {
    "uniform_2d": lambda: BlockMesh.uniform(2, level=2, block=(16, 16, 1)),
    "uniform_3d": lambda: BlockMesh.uniform(3, level=1, block=(8, 8, 8)),
    "amr_2d": MESHES["2d_b8"],
    "amr_3d": MESHES["3d_b8"],
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_rk2_run_fp64_bit_exact(oracle_lib, name):
    mesh = CASES[name]()
    st = settings(gamma0=1.4, cfl=0.4)
    st.time_integrator = "RK2_SSP"
    U, B = wl.random_smooth(mesh, seed=8)
    nsteps = 5
    om = oracle_lib.Mesh.from_block_mesh(mesh)
    Uo, Bo, dto = oracle_lib.run(om, oracle_settings(oracle_lib, st), U, B, nsteps)
    impl = GodunovImplemGB300(st, mesh, precision="fp64")
    dU, dB = _dev(U), _dev(B)
    dtg, _ = impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), nsteps)
    n = mesh.n_owned
    assert np.array_equal(dtg[:, 0], dto)
    assert np.array_equal(dU.cpu().numpy()[:n], Uo[:n])
    assert np.array_equal(dB.cpu().numpy()[:n], Bo[:n])


def test_rk2_single_stage_matches_oracle_step(oracle_lib):
    """do_time_step under RK2_SSP (no predictor, no half-step source in the edge states)."""
    mesh = BlockMesh.uniform(3, level=1, block=(8, 8, 8))
    st = settings(gamma0=1.4)
    st.time_integrator = "RK2_SSP"
    U, B = wl.orszag_tang(mesh, gamma=st.gamma0)
    om = oracle_lib.Mesh.from_block_mesh(mesh)
    Uo, Bo = oracle_lib.step(om, oracle_settings(oracle_lib, st), U, B, 2e-3)
    impl = GodunovImplemGB300(st, mesh, precision="fp64")
    dU, dB = _dev(U), _dev(B)
    dU2, dB2 = dU.clone(), dB.clone()
    impl.do_time_step(dU, dU2, dB, dB2, 2e-3)
    n = mesh.n_owned
    assert np.array_equal(dU2.cpu().numpy()[:n], Uo[:n])
    assert np.array_equal(dB2.cpu().numpy()[:n], Bo[:n])


@pytest.mark.parametrize("name", ["uniform_3d", "amr_2d"])
def test_rk2_mixed_accuracy(oracle_lib, name):
    mesh = CASES[name]()
    st = settings(gamma0=1.4, cfl=0.4)
    st.time_integrator = "RK2_SSP"
    U, B = wl.random_smooth(mesh, seed=9)
    nsteps = 8
    Uo, _, _ = oracle_lib.run(oracle_lib.Mesh.from_block_mesh(mesh), oracle_settings(oracle_lib, st), U, B, nsteps)
    impl = GodunovImplemGB300(st, mesh, precision="mixed")
    dU, dB = _dev(U), _dev(B)
    impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), nsteps)
    n = mesh.n_owned
    assert l1_rel(dU.cpu().numpy()[:n, 0], Uo[:n, 0]) <= 1e-6

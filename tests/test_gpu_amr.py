"""Coarse/fine (AMR) meshes on the GPU against the oracle.

The FP64 path must match the oracle bit for bit through the ghost prepass (restriction,
SIMPLE_COPY and EXTRAPOLATE_LINEAR_MINMOD prolongation, face-B ghosts), the fine-flux sums of coarse
cells (ReadFluxesAndConservativeUpdateFunctor.cpp:141-172) and the coarse/fine EMF correction
(CorrectEmfAtBlockBorderFunctor.cpp:94-360); the mixed path must stay within its tolerance and keep
div B at round-off and mass conserved.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_mhd_ct_gb300 import workloads as wl  # noqa: E402
from godunov_mhd_ct_gb300.mesh import BlockMesh  # noqa: E402
from godunov_mhd_ct_gb300.solver import GodunovImplemGB300  # noqa: E402

from .helpers import l1_rel, oracle_settings, same_level_face_mismatch, settings  # noqa: E402

pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def refine_ball(center, radius):
    c = np.asarray(center, dtype=np.float64)

    def f(level, lo, hi):
        dim = 3 if hi[2] - lo[2] < 1.0 else 2
        p = np.clip(c, lo, hi)
        near = np.sqrt(((p - c)[:dim] ** 2).sum())
        far = np.sqrt((np.maximum(np.abs(lo - c), np.abs(hi - c))[:dim] ** 2).sum())
        return near < radius < far

    return f


MESHES = {
    # 2D, 8^2 blocks (8x8 tiles: one tile per block), three levels
    "2d_b8": lambda: BlockMesh.amr(2, refine_ball((0.5, 0.5, 0.5), 0.3), base_level=2, max_level=4, block=(8, 8, 1)),
    # 2D, 16^2 blocks, two levels
    "2d_b16": lambda: BlockMesh.amr(2, refine_ball((0.4, 0.55, 0.5), 0.25), base_level=1, max_level=3,
                                    block=(16, 16, 1)),
    # 3D, 8^3 blocks (several tiles per block on the FP64 path)
    "3d_b8": lambda: BlockMesh.amr(3, refine_ball((0.3, 0.3, 0.3), 0.2), base_level=1, max_level=2, block=(8, 8, 8)),
    # 3D, 4^3 blocks, three levels
    "3d_b4": lambda: BlockMesh.amr(3, refine_ball((0.3, 0.3, 0.3), 0.2), base_level=1, max_level=3, block=(4, 4, 4)),
}


def _totals(m, U):
    vol = (m.block_dx() ** m.dim)[: m.n_owned, None, None, None]
    return [float((U[: m.n_owned, v] * vol).sum()) for v in (0, 1)]


def _div_b(m, B):
    Bx, By, Bz = m.split_faces(B)
    d = (Bx[..., 1:] - Bx[..., :-1]) + (By[..., 1:, :] - By[..., :-1, :])
    if m.dim == 3:
        d = d + (Bz[:, 1:] - Bz[:, :-1])
    return float(np.abs(d / m.block_dx()[:, None, None, None])[: m.n_owned].max())


@pytest.mark.parametrize("name", sorted(MESHES))
@pytest.mark.parametrize("prolongation", ["SIMPLE_COPY", "EXTRAPOLATE_LINEAR_MINMOD"])
def test_amr_step_fp64_bit_exact(oracle_lib, name, prolongation):
    mesh = MESHES[name]()
    assert mesh.fine_neighbor is not None
    st = settings(gamma0=1.4)
    st.prolongation = prolongation
    U, B = wl.random_smooth(mesh, seed=5)
    om = oracle_lib.Mesh.from_block_mesh(mesh, prolongation=1 if prolongation != "SIMPLE_COPY" else 0)
    dt = 0.4 / oracle_lib.inv_dt(om, oracle_settings(oracle_lib, st), U, B)
    Uo, Bo = oracle_lib.step(om, oracle_settings(oracle_lib, st), U, B, dt)
    impl = GodunovImplemGB300(st, mesh, precision="fp64")
    dU, dB = _dev(U), _dev(B)
    dU2, dB2 = dU.clone(), dB.clone()
    impl.do_time_step(dU, dU2, dB, dB2, dt)
    torch.cuda.synchronize()
    assert impl.last_status() & ~16 == 0
    n = mesh.n_owned
    assert np.array_equal(dU2.cpu().numpy()[:n], Uo[:n])
    assert np.array_equal(dB2.cpu().numpy()[:n], Bo[:n])


@pytest.mark.parametrize("name", ["2d_b8", "3d_b8"])
@pytest.mark.parametrize("riemann", ["HLLD", "LLF"])
def test_amr_run_fp64_bit_exact(oracle_lib, name, riemann):
    """Solver loop (CUDA graph, device dt) against the oracle's run, bit for bit."""
    mesh = MESHES[name]()
    st = settings(gamma0=1.4, cfl=0.4, riemann=riemann)
    U, B = wl.random_smooth(mesh, seed=7)
    nsteps = 6
    om = oracle_lib.Mesh.from_block_mesh(mesh)
    Uo, Bo, dto = oracle_lib.run(om, oracle_settings(oracle_lib, st), U, B, nsteps)
    impl = GodunovImplemGB300(st, mesh, precision="fp64")
    dU, dB = _dev(U), _dev(B)
    dtg, _ = impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), nsteps)
    n = mesh.n_owned
    assert np.array_equal(dtg[:, 0], dto)
    assert np.array_equal(dU.cpu().numpy()[:n], Uo[:n])
    assert np.array_equal(dB.cpu().numpy()[:n], Bo[:n])
    assert same_level_face_mismatch(mesh, dB.cpu().numpy()) == 0.0


@pytest.mark.parametrize("name", sorted(MESHES))
def test_amr_mixed_accuracy_and_invariants(oracle_lib, name):
    mesh = MESHES[name]()
    st = settings(gamma0=1.4, cfl=0.4)
    U, B = wl.random_smooth(mesh, seed=11)
    nsteps = 10
    om = oracle_lib.Mesh.from_block_mesh(mesh)
    Uo, Bo, _ = oracle_lib.run(om, oracle_settings(oracle_lib, st), U, B, nsteps)
    impl = GodunovImplemGB300(st, mesh, precision="mixed")
    dU, dB = _dev(U), _dev(B)
    impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), nsteps)
    n = mesh.n_owned
    Ug, Bg = dU.cpu().numpy(), dB.cpu().numpy()
    assert l1_rel(Ug[:n, 0], Uo[:n, 0]) <= 1e-6
    assert l1_rel(Ug[:n, 1], Uo[:n, 1]) <= 1e-6
    assert _div_b(mesh, Bg) <= 1e-10
    assert same_level_face_mismatch(mesh, Bg) == 0.0
    t0, t1 = _totals(mesh, U), _totals(mesh, Ug)
    assert abs(t1[0] - t0[0]) <= 1e-10 * abs(t0[0])


def test_amr_walls_fp64_bit_exact(oracle_lib):
    """Refinement inside a domain with reflecting y borders (outside blocks at the border level)."""
    mesh = BlockMesh.amr(2, refine_ball((0.5, 0.5, 0.5), 0.2), base_level=2, max_level=3, block=(8, 8, 1),
                         periodic=(True, False, True))
    bc = (1, 1, 3, 3, 1, 1)
    st = settings(gamma0=1.4, cfl=0.4)
    U, B = wl.kelvin_helmholtz(mesh, seed=2)
    nsteps = 5
    om = oracle_lib.Mesh.from_block_mesh(mesh, bc=bc)
    Uo, Bo, dto = oracle_lib.run(om, oracle_settings(oracle_lib, st), U, B, nsteps)
    impl = GodunovImplemGB300(st, mesh, precision="fp64", bc=bc)
    dU, dB = _dev(U), _dev(B)
    dtg, _ = impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), nsteps)
    n = mesh.n_owned
    assert np.array_equal(dtg[:, 0], dto)
    assert np.array_equal(dU.cpu().numpy()[:n], Uo[:n])
    assert np.array_equal(dB.cpu().numpy()[:n], Bo[:n])


def test_amr_blast_fp64_bit_exact(oracle_lib):
    """Magnetised blast (strong pressure jump on the refined front), solver loop, bit for bit."""
    mesh = wl.blast_mesh(base_level=2, max_level=4, block=8, radius=0.15, band=0.05)
    st = settings(gamma0=5.0 / 3.0, cfl=0.5)
    U, B = wl.blast(mesh, gamma=st.gamma0, radius=0.15)
    nsteps = 8
    om = oracle_lib.Mesh.from_block_mesh(mesh)
    Uo, Bo, dto = oracle_lib.run(om, oracle_settings(oracle_lib, st), U, B, nsteps)
    impl = GodunovImplemGB300(st, mesh, precision="fp64")
    dU, dB = _dev(U), _dev(B)
    dtg, _ = impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), nsteps)
    n = mesh.n_owned
    assert np.array_equal(dtg[:, 0], dto)
    assert np.array_equal(dU.cpu().numpy()[:n], Uo[:n])
    assert np.array_equal(dB.cpu().numpy()[:n], Bo[:n])

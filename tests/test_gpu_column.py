"""The column step (16 x 8 columns walking each block along z; mixed precision, 3D, conforming meshes)
against the 8x8x8-tile step of the same path and against the FP64 oracle.

Both kernels compute the same cells with the same formulas in the same order, compiled separately, so
their FP32 contractions may differ in the last bits: one step agrees to 1e-6 relative (L1) and 1e-5 of
the field's largest magnitude, as for any two tiles of the mixed path. Over a run the column step must
stay within the mixed path's bar against the oracle: L1(rho) <= 1e-6, max|div B| <= 1e-12, and mass and
energy conserved to 1e-13 on periodic meshes."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_mhd_ct_gb300 import workloads as wl  # noqa: E402
from godunov_mhd_ct_gb300.mesh import BlockMesh  # noqa: E402
from godunov_mhd_ct_gb300.solver import GodunovImplemGB300  # noqa: E402

from .helpers import accuracy_block, oracle_mesh, oracle_settings, settings  # noqa: E402

pytestmark = pytest.mark.gpu
COLUMN, TILE8 = 16, 8


def _close(got, ref, n):
    for a, b in zip(got, ref):
        a, b = a[:n], b[:n]
        assert np.abs(a - b).sum() <= 1e-6 * np.abs(b).sum()
        assert np.max(np.abs(a - b)) <= 1e-5 * np.max(np.abs(b))


def _step(impl, U, B, dt):
    dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    dU2, dB2 = dU.clone(), dB.clone()
    impl.do_time_step(dU, dU2, dB, dB2, dt)
    torch.cuda.synchronize()
    assert impl.last_status() & ~16 == 0
    return dU2.cpu().numpy(), dB2.cpu().numpy()


@pytest.mark.parametrize("block,level", [((32, 32, 32), 1), ((16, 16, 16), 1), ((16, 8, 8), 2), ((32, 16, 48), 1)])
@pytest.mark.parametrize("extra", ["none", "gravity", "rk2", "minmod_hll"])
def test_column_step_matches_tile_step(block, level, extra):
    kw = {}
    if extra == "minmod_hll":
        kw = dict(slope_type=1.0, riemann="HLL")
    st = settings(gamma0=1.4, **kw)
    if extra == "gravity":
        st.gravity = (0.2, -0.7, 0.4)
    if extra == "rk2":
        st.time_integrator = "RK2_SSP"
    mesh = BlockMesh.uniform(3, level=level, block=block)
    U, B = wl.random_smooth(mesh, gamma=st.gamma0, seed=9, amp=0.3)
    impl = GodunovImplemGB300(st, mesh, precision="mixed")
    dt = 0.5 * impl.compute_dt(torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda())
    impl.set_tile(TILE8 if block[2] % 8 == 0 else 4)
    ref = _step(impl, U, B, dt)
    impl.set_tile(COLUMN)
    got = _step(impl, U, B, dt)
    _close(got, ref, mesh.n_owned)
    impl.close()


def test_column_run_matches_oracle_and_conserves(oracle_lib):
    """3D Orszag-Tang 64^3 (8 blocks of 32^3), 20 solver iterations: graph-replayed loop with the fused
    CFL of the column step."""
    mesh = BlockMesh.uniform(3, level=1, block=(32, 32, 32))
    st = settings()
    U, B = wl.orszag_tang(mesh, gamma=st.gamma0, rho_perturbation=1e-3, seed=5)
    n = mesh.n_owned
    Uo, Bo, dto = oracle_lib.run(oracle_mesh(oracle_lib, mesh), oracle_settings(oracle_lib, st), U, B, 20)
    outs = {}
    for tile in (TILE8, COLUMN):
        impl = GodunovImplemGB300(st, mesh, precision="mixed")
        impl.set_tile(tile)
        dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
        dtg, _ = impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), 20)
        assert impl.last_status() & ~16 == 0
        outs[tile] = (dU.cpu().numpy(), dB.cpu().numpy(), dtg[:, 0])
        impl.close()
    Ug, Bg, dtg = outs[COLUMN]
    acc = accuracy_block(mesh, U, mesh, Ug, Bg, Uo, Bo)
    print("column vs oracle:", acc)
    assert acc["l1_rho"] <= 1e-6 and acc["max_divB"] <= 1e-12
    assert acc["mass_drift"] <= 1e-13 and acc["energy_drift"] <= 1e-13
    assert np.max(np.abs(dtg - dto) / dto) <= 1e-5
    # the CFL estimates of the two mixed kernels agree closely
    assert np.max(np.abs(dtg - outs[TILE8][2]) / outs[TILE8][2]) <= 1e-5


def test_column_with_walls(oracle_lib):
    """Reflecting walls in y (outside blocks filled each step) on a uniform 3D mesh."""
    mesh = BlockMesh.uniform(3, level=1, block=(16, 16, 16), periodic=(True, False, True))
    st = settings(gamma0=1.4)
    U, B = wl.random_smooth(mesh, gamma=st.gamma0, seed=13, amp=0.2)
    bc = (1, 1, 3, 3, 1, 1)
    n = mesh.n_owned
    Uo, Bo, _ = oracle_lib.run(oracle_lib.Mesh.from_block_mesh(mesh, bc=list(bc)), oracle_settings(oracle_lib, st),
                               U, B, 10)
    impl = GodunovImplemGB300(st, mesh, precision="mixed", bc=bc)
    impl.set_tile(COLUMN)
    dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), 10)
    assert impl.last_status() & ~16 == 0
    acc = accuracy_block(mesh, U, mesh, dU.cpu().numpy(), dB.cpu().numpy(), Uo, Bo)
    assert acc["l1_rho"] <= 1e-6 and acc["max_divB"] <= 1e-12
    impl.close()


def test_column_batch_with_staggered_end_times(oracle_lib):
    """Problems ending at different times: a finished problem's columns are carried over unchanged."""
    st = settings(gamma0=1.4, cfl=0.4, slope_type=2.0)
    meshes = [BlockMesh.uniform(3, level=1, block=(16, 16, 16)), BlockMesh.uniform(3, level=1, block=(16, 16, 16)),
              BlockMesh.uniform(3, level=2, block=(16, 16, 16))]
    states = [wl.random_smooth(m, seed=40 + p) for p, m in enumerate(meshes)]
    mesh, problem = BlockMesh.batch(meshes)
    U = np.concatenate([s[0] for s in states])
    B = np.concatenate([s[1] for s in states])
    t_end = np.array([5e-3, 1.5e-2, 1e-2])
    impl = GodunovImplemGB300(st, mesh, precision="mixed", problem=problem, n_problems=len(meshes))
    impl.set_tile(COLUMN)
    dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    dtlog, t = impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), 12, t=0.0, t_end=t_end)
    Ug, Bg = dU.cpu().numpy(), dB.cpu().numpy()
    assert np.allclose(t, t_end, rtol=0, atol=1e-15)
    off = 0
    for p, (m, (Up, Bp)) in enumerate(zip(meshes, states)):
        Uo, Bo, dto, _ = oracle_lib.run_to(oracle_mesh(oracle_lib, m), oracle_settings(oracle_lib, st), Up, Bp, 12,
                                           0.0, t_end[p])
        sl = slice(off, off + m.n_owned)
        off += m.n_owned
        l1 = float(np.abs(Ug[sl, 0] - Uo[:, 0]).sum() / np.abs(Uo[:, 0]).sum())
        assert l1 <= 1e-6
        assert np.count_nonzero(dtlog[:, p]) == np.count_nonzero(dto)


def test_column_not_offered_where_it_does_not_apply():
    """Blocks narrower than a column, viscous runs and coarse/fine meshes fall back to the tile step."""
    st = settings()
    mesh = BlockMesh.uniform(3, level=1, block=(8, 8, 8))
    U, B = wl.random_smooth(mesh, gamma=st.gamma0, seed=1)
    impl = GodunovImplemGB300(st, mesh, precision="mixed")
    dt = 0.5 * impl.compute_dt(torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda())
    impl.set_tile(COLUMN)  # falls back to the largest tile that divides the block
    got = _step(impl, U, B, dt)
    impl.set_tile(TILE8)
    ref = _step(impl, U, B, dt)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    impl.close()

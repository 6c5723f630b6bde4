"""Tile choice and the autotuner (gmhd_set_tile, gmhd_autotune).

Every tile configuration computes the same cells with the same formulas. On the FP64 path (no FMA
contraction) a step must give bit-identical U2, B2 whatever tile runs it, on uniform and coarse/fine
meshes, equal to the oracle's. On the mixed path each tile is its own compiled kernel whose FP32
contractions may differ in the last bits: results must agree to 1e-6 relative (L1) and to 1e-5 of the
field's largest magnitude. The autotuner must return one of the configured tiles and keep it for the following steps and
across a new mesh of the same block size.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_mhd_ct_gb300 import workloads as wl  # noqa: E402
from godunov_mhd_ct_gb300.mesh import BlockMesh  # noqa: E402
from godunov_mhd_ct_gb300.solver import GodunovImplemGB300  # noqa: E402

from .helpers import oracle_mesh, oracle_settings, settings  # noqa: E402

pytestmark = pytest.mark.gpu


def _same(precision, got, ref, n):
    for a, b in zip(got, ref):
        a, b = a[:n], b[:n]
        if precision == "fp64":
            assert np.array_equal(a, b)
        else:
            assert np.abs(a - b).sum() <= 1e-6 * np.abs(b).sum()
            assert np.max(np.abs(a - b)) <= 1e-5 * np.max(np.abs(b))


def _step(impl, U, B, dt):
    dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    dU2, dB2 = dU.clone(), dB.clone()
    impl.do_time_step(dU, dU2, dB, dB2, dt)
    torch.cuda.synchronize()
    assert impl.last_status() & ~16 == 0
    return dU2.cpu().numpy(), dB2.cpu().numpy()


CASES = [
    # dim, block, tiles the block admits
    (3, (16, 16, 16), (8, 4, 16)),
    (2, (16, 16, 1), (16, 8, 4)),
]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("dim,block,tiles", CASES)
def test_results_do_not_depend_on_the_tile(oracle_lib, precision, dim, block, tiles):
    mesh = BlockMesh.uniform(dim, level=1, block=block)
    st = settings()
    U, B = wl.random_smooth(mesh, gamma=st.gamma0, seed=3, amp=0.3)
    impl = GodunovImplemGB300(st, mesh, precision=precision)
    dt = 0.5 * impl.compute_dt(torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda())
    outs = []
    for t in tiles:
        impl.set_tile(t)
        outs.append(_step(impl, U, B, dt))
    n = mesh.n_owned
    for out in outs[1:]:
        _same(precision, out, outs[0], n)
    if precision == "fp64":
        U2o, B2o = oracle_lib.step(oracle_mesh(oracle_lib, mesh), oracle_settings(oracle_lib, st), U, B, dt)
        assert np.array_equal(outs[0][0][:n], U2o[:n]) and np.array_equal(outs[0][1][:n], B2o[:n])
    impl.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("dim", [2, 3])
def test_tile_choice_on_a_coarse_fine_mesh(oracle_lib, precision, dim):
    """Two-level meshes: the two-pass tile lists are rebuilt for each tile (3D: the persistent kernel on
    both tiles); FP64 steps agree bit for bit and with the oracle."""
    if dim == 2:
        mesh = BlockMesh.amr(2, wl.refine_band((0.5, 0.5, 0.5), 0.1, 0.2), base_level=2, max_level=3,
                             block=(16, 16, 1))
        tiles = (16, 8, 4)
    else:
        mesh = BlockMesh.amr(3, wl.refine_band((0.3, 0.3, 0.3), 0.0, 0.1, axes=3), base_level=2, max_level=3,
                             block=(8, 8, 8))
        tiles = (8, 4)
    assert mesh.is_amr
    st = settings()
    U, B = wl.random_smooth(mesh, gamma=st.gamma0, seed=5, amp=0.2)
    impl = GodunovImplemGB300(st, mesh, precision=precision)
    dt = 0.5 * impl.compute_dt(torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda())
    outs = []
    for t in tiles:
        impl.set_tile(t)
        outs.append(_step(impl, U, B, dt))
    n = mesh.n_owned
    for out in outs[1:]:
        _same(precision, out, outs[0], n)
    if precision == "fp64":
        om = oracle_lib.Mesh.from_block_mesh(mesh)
        U2o, B2o = oracle_lib.step(om, oracle_settings(oracle_lib, st), U, B, dt)
        assert np.array_equal(outs[0][0][:n], U2o[:n]) and np.array_equal(outs[0][1][:n], B2o[:n])
    impl.close()


def test_autotune_picks_a_configured_tile_and_keeps_it():
    mesh = BlockMesh.uniform(3, level=1, block=(32, 32, 32))
    st = settings()
    U, B = wl.orszag_tang(mesh, gamma=st.gamma0)
    impl = GodunovImplemGB300(st, mesh, precision="mixed")
    dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    dU2, dB2 = torch.empty_like(dU), torch.empty_like(dB)
    dt = impl.compute_dt(dU, dB)
    ref = _step(impl, U, B, dt)
    tile, ms = impl.autotune(dU, dU2, dB, dB2, dt)
    assert tile in (8, 4, 16) and ms > 0.0
    tuned = _step(impl, U, B, dt)
    _same("mixed", tuned, ref, mesh.n_owned)
    # a graph-replayed loop after the tuning (the cached graph is rebuilt for the chosen kernel), and a
    # new mesh of the same block size keep the choice: the same bits as right after the tuning
    impl.advance(dU, dU2, dB, dB2, 3)
    impl.resize_auxiliary_data(mesh)
    got = _step(impl, U, B, dt)
    assert np.array_equal(got[0], tuned[0]) and np.array_equal(got[1], tuned[1])
    impl.close()


def test_autotune_on_a_coarse_fine_mesh_keeps_fp64_exact(oracle_lib):
    """The autotuner on a two-level 2D mesh (tile lists rebuilt per candidate): the FP64 step afterwards
    still equals the oracle's bit for bit; an empty mesh tunes without work."""
    mesh = BlockMesh.amr(2, wl.refine_band((0.5, 0.5, 0.5), 0.1, 0.2), base_level=2, max_level=3, block=(16, 16, 1))
    st = settings()
    U, B = wl.random_smooth(mesh, gamma=st.gamma0, seed=8, amp=0.2)
    impl = GodunovImplemGB300(st, mesh, precision="fp64")
    dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    dt = 0.5 * impl.compute_dt(dU, dB)
    tile, _ = impl.autotune(dU, torch.empty_like(dU), dB, torch.empty_like(dB), dt)
    assert tile in (16, 8, 4)
    U2, B2 = _step(impl, U, B, dt)
    U2o, B2o = oracle_lib.step(oracle_lib.Mesh.from_block_mesh(mesh), oracle_settings(oracle_lib, st), U, B, dt)
    n = mesh.n_owned
    assert np.array_equal(U2[:n], U2o[:n]) and np.array_equal(B2[:n], B2o[:n])
    impl.close()
    empty = BlockMesh(dim=2, block=(16, 16, 1), level=np.zeros(0, np.int32), neighbor=np.zeros((0, 27), np.int32),
                      coords=np.zeros((0, 3), np.int64), n_owned=0, grid=(1, 1, 1), periodic=(True, True, True))
    impl = GodunovImplemGB300(st, empty, precision="mixed")
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    tile, _ = impl.autotune(x, x.clone(), x.clone(), x.clone(), 1e-3)
    assert tile in (16, 8, 4)
    impl.close()

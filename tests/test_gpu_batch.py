"""Batched independent problems (configuration 3: field loops of uneven sizes) in one launch per
step, each with its own CFL dt and end time, against the oracle run problem by problem."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_mhd_ct_gb300 import workloads as wl  # noqa: E402
from godunov_mhd_ct_gb300.mesh import BlockMesh  # noqa: E402
from godunov_mhd_ct_gb300.solver import GodunovImplemGB300  # noqa: E402

from .helpers import max_rel_diff, oracle_mesh, oracle_settings, settings  # noqa: E402

pytestmark = pytest.mark.gpu
TOL_FP64 = 1e-12


def _batch(n, seed, sizes):
    meshes, states, params = wl.field_loop_batch(n, seed=seed, sizes=sizes)
    mesh, problem = BlockMesh.batch(meshes)
    U = np.concatenate([s[0] for s in states])
    B = np.concatenate([s[1] for s in states])
    return meshes, states, mesh, problem, U, B


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_field_loop_batch_matches_per_problem_oracle(oracle_lib, precision):
    st = settings(gamma0=5.0 / 3.0, slope_type=2.0)
    meshes, states, mesh, problem, U, B = _batch(7, seed=3, sizes=(32, 64))
    assert len({m.n_owned for m in meshes}) > 1  # uneven sizes
    t_end, nsteps = 0.01, 12
    impl = GodunovImplemGB300(st, mesh, precision=precision, problem=problem, n_problems=len(meshes))
    dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    dtlog, t = impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), nsteps, t=0.0, t_end=t_end)
    Ug, Bg = dU.cpu().numpy(), dB.cpu().numpy()
    assert np.allclose(t, t_end, rtol=0, atol=1e-15)
    off = 0
    for p, (m, (Up, Bp)) in enumerate(zip(meshes, states)):
        Uo, Bo, dto, to = oracle_lib.run_to(oracle_mesh(oracle_lib, m), oracle_settings(oracle_lib, st), Up, Bp,
                                            nsteps, 0.0, t_end)
        sl = slice(off, off + m.n_owned)
        off += m.n_owned
        assert dto[-1] == 0.0 and to == t_end  # every problem finished inside the step budget
        if precision == "fp64":
            assert max_rel_diff(dtlog[:, p], dto) <= TOL_FP64
            assert max_rel_diff(Ug[sl], Uo) <= TOL_FP64
            assert max_rel_diff(Bg[sl], Bo) <= TOL_FP64
        else:
            l1 = float(np.abs(Ug[sl, 0] - Uo[:, 0]).sum() / np.abs(Uo[:, 0]).sum())
            assert l1 <= 1e-6
            assert np.all(np.abs(dtlog[:, p] - dto) <= 1e-6 * np.max(dto))


def test_batch_rejects_cross_problem_neighbours():
    from godunov_mhd_ct_gb300._native import NativeError

    meshes, _, mesh, problem, _, _ = _batch(3, seed=1, sizes=(32,))
    bad = problem.copy()
    bad[0] = 1  # block 0 now claims problem 1 while its neighbours belong to problem 0
    with pytest.raises(NativeError):
        GodunovImplemGB300(settings(), mesh, problem=bad, n_problems=3)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_3d_batch_with_staggered_end_times(oracle_lib, precision):
    """3D problems of 8^3 tiles (the mixed path's persistent kernel) ending at different times: a
    finished problem's tiles are carried over unchanged while the others keep stepping."""
    st = settings(gamma0=1.4, cfl=0.4, slope_type=2.0)
    meshes = [BlockMesh.uniform(3, level=1, block=(16, 16, 16)), BlockMesh.uniform(3, level=1, block=(16, 16, 16)),
              BlockMesh.uniform(3, level=2, block=(16, 16, 16))]
    states = [wl.random_smooth(m, seed=40 + p) for p, m in enumerate(meshes)]
    mesh, problem = BlockMesh.batch(meshes)
    U = np.concatenate([s[0] for s in states])
    B = np.concatenate([s[1] for s in states])
    t_end = np.array([5e-3, 1.5e-2, 1e-2])  # about 2, 6 and 8 steps
    nsteps = 12
    impl = GodunovImplemGB300(st, mesh, precision=precision, problem=problem, n_problems=len(meshes))
    dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    dtlog, t = impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), nsteps, t=0.0, t_end=t_end)
    Ug, Bg = dU.cpu().numpy(), dB.cpu().numpy()
    assert np.allclose(t, t_end, rtol=0, atol=1e-15)
    off = 0
    for p, (m, (Up, Bp)) in enumerate(zip(meshes, states)):
        Uo, Bo, dto, to = oracle_lib.run_to(oracle_mesh(oracle_lib, m), oracle_settings(oracle_lib, st), Up, Bp,
                                            nsteps, 0.0, t_end[p])
        sl = slice(off, off + m.n_owned)
        off += m.n_owned
        n_active = int(np.count_nonzero(dto))
        assert n_active < nsteps  # finished inside the step budget, later steps carried the state over
        if precision == "fp64":
            assert max_rel_diff(Ug[sl], Uo) <= TOL_FP64
            assert max_rel_diff(Bg[sl], Bo) <= TOL_FP64
        else:
            l1 = float(np.abs(Ug[sl, 0] - Uo[:, 0]).sum() / np.abs(Uo[:, 0]).sum())
            assert l1 <= 1e-6
            assert np.count_nonzero(dtlog[:, p]) == n_active


@pytest.mark.parametrize("dim", [2, 3])
def test_finished_problems_skipped_across_calls(dim):
    """A finished problem is copied through by one step and then skipped; the state stays exact when the
    run is split into calls of odd and even lengths whose scratch buffers start as NaN (each call's first
    step copies a finished problem through again)."""
    st = settings(gamma0=5.0 / 3.0, cfl=0.4, slope_type=2.0)
    if dim == 2:
        meshes, states, mesh, problem, U, B = _batch(5, seed=8, sizes=(32, 64))
        t_end = np.array([4e-3, 1e-2, 6e-3, 2e-2, 8e-3])
    else:
        meshes = [BlockMesh.uniform(3, level=1, block=(16, 16, 16)) for _ in range(3)]
        states = [wl.random_smooth(m, seed=60 + p) for p, m in enumerate(meshes)]
        mesh, problem = BlockMesh.batch(meshes)
        U = np.concatenate([s[0] for s in states])
        B = np.concatenate([s[1] for s in states])
        t_end = np.array([5e-3, 1.5e-2, 1e-2])
    n = len(meshes)
    ref = GodunovImplemGB300(st, mesh, precision="fp64", problem=problem, n_problems=n)
    rU, rB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    ref.advance(rU, torch.empty_like(rU), rB, torch.empty_like(rB), 30, t=0.0, t_end=t_end, use_graph=False)
    impl = GodunovImplemGB300(st, mesh, precision="fp64", problem=problem, n_problems=n)
    dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    t = np.zeros(n)
    logs = []
    for k in (3, 4, 5, 2, 7, 9):
        U2 = torch.full_like(dU, float("nan"))
        B2 = torch.full_like(dB, float("nan"))
        dtlog, t = impl.advance(dU, U2, dB, B2, k, t=t, t_end=t_end)
        logs.append(dtlog)
    dtlog = np.concatenate(logs)
    assert np.allclose(t, t_end, rtol=0, atol=1e-15)
    assert not np.signbit(dtlog).any()  # the log holds +0 for finished problems
    assert (dtlog[-1] == 0.0).all()
    assert np.array_equal(dU.cpu().numpy(), rU.cpu().numpy())
    assert np.array_equal(dB.cpu().numpy(), rB.cpu().numpy())

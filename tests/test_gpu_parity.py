"""GPU parity: the CUDA path, called through the C ABI (libgmhd.so), against the FP64 oracle.

FP64 path: the oracle restates the reference in FP64 with its operand order; the kernel is built
without FMA contraction, so results are expected to be identical. The bar written here is
1e-12 relative per field; the test also records whether they are bit-identical. Mixed path: L1(rho) <= 1e-6 relative to FP64 and max|div B| <= 1e-12.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_mhd_ct_gb300 import workloads as wl  # noqa: E402
from godunov_mhd_ct_gb300.mesh import BlockMesh  # noqa: E402
from godunov_mhd_ct_gb300.solver import GodunovImplemGB300  # noqa: E402

from .helpers import (div_b, l1_rel, max_rel_diff, oracle_mesh, oracle_settings, settings,  # noqa: E402
                      shared_face_mismatch)

pytestmark = pytest.mark.gpu
TOL_FP64 = 1e-12


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _one_step_pair(oracle_lib, mesh, st, U, B, dt, precision="fp64"):
    impl = GodunovImplemGB300(st, mesh, precision=precision)
    dU, dB = _dev(U), _dev(B)
    dU2, dB2 = dU.clone(), dB.clone()
    impl.do_time_step(dU, dU2, dB, dB2, dt)
    torch.cuda.synchronize()
    assert impl.last_status() & ~16 == 0
    U2g, B2g = dU2.cpu().numpy(), dB2.cpu().numpy()
    U2o, B2o = oracle_lib.step(oracle_mesh(oracle_lib, mesh), oracle_settings(oracle_lib, st), U, B, dt)
    n = mesh.n_owned
    return U2g[:n], B2g[:n], U2o[:n], B2o[:n]


@pytest.mark.parametrize("dim,block,level", [(2, (16, 16, 1), 2), (2, (8, 8, 1), 2), (3, (8, 8, 8), 1),
                                             (3, (16, 8, 8), 1), (3, (4, 4, 4), 1)])
@pytest.mark.parametrize("riemann", ["HLLD", "HLL", "LLF", "HLLC"])
@pytest.mark.parametrize("slope_type", [1.0, 2.0])
def test_single_step_fp64_matches_oracle(oracle_lib, dim, block, level, riemann, slope_type):
    mesh = BlockMesh.uniform(dim, level=level, block=block)
    st = settings(gamma0=1.4, slope_type=slope_type, riemann=riemann)
    U, B = wl.random_smooth(mesh, gamma=1.4, seed=dim * 7 + level)
    dt = 0.3 * mesh.cell_length()
    U2g, B2g, U2o, B2o = _one_step_pair(oracle_lib, mesh, st, U, B, dt)
    assert max_rel_diff(U2g, U2o) <= TOL_FP64
    assert max_rel_diff(B2g, B2o) <= TOL_FP64


@pytest.mark.parametrize("dim,block,level,nsteps", [(2, (16, 16, 1), 3, 200), (3, (32, 32, 32), 1, 5)])
def test_orszag_tang_run_fp64_matches_oracle(oracle_lib, dim, block, level, nsteps):
    """Config 0 in full (2D OT 128^2, 200 steps) and a reduced config 1 (3D OT 64^3)."""
    mesh = BlockMesh.uniform(dim, level=level, block=block)
    st = settings()
    U, B = wl.orszag_tang(mesh, gamma=st.gamma0, rho_perturbation=1e-3 if dim == 3 else 0.0, seed=12345)
    Uo, Bo, dto = oracle_lib.run(oracle_mesh(oracle_lib, mesh), oracle_settings(oracle_lib, st), U, B, nsteps)
    impl = GodunovImplemGB300(st, mesh, precision="fp64")
    dU, dB = _dev(U), _dev(B)
    dU2, dB2 = torch.empty_like(dU), torch.empty_like(dB)
    dtg, _ = impl.advance(dU, dU2, dB, dB2, nsteps)
    Ug, Bg = dU.cpu().numpy(), dB.cpu().numpy()
    assert max_rel_diff(dtg[:, 0], dto) <= TOL_FP64
    assert max_rel_diff(Ug, Uo) <= TOL_FP64
    assert max_rel_diff(Bg, Bo) <= TOL_FP64
    print(f"bit-identical U: {np.array_equal(Ug, Uo)}  B: {np.array_equal(Bg, Bo)}  dt: {np.array_equal(dtg[:, 0], dto)}")
    assert np.max(np.abs(div_b(mesh, Bg))) <= 1e-12
    assert shared_face_mismatch(mesh, Bg) == 0.0


def test_inv_dt_matches_oracle(oracle_lib):
    for dim, block, level in [(2, (16, 16, 1), 3), (3, (8, 8, 8), 1)]:
        mesh = BlockMesh.uniform(dim, level=level, block=block)
        st = settings()
        U, B = wl.orszag_tang(mesh, gamma=st.gamma0, rho_perturbation=1e-3, seed=3)
        impl = GodunovImplemGB300(st, mesh)
        g = impl.compute_inv_dt(_dev(U), _dev(B))
        o = oracle_lib.inv_dt(oracle_mesh(oracle_lib, mesh), oracle_settings(oracle_lib, st), U, B)
        assert g == o


def test_step_host_buffers(oracle_lib):
    mesh = BlockMesh.uniform(2, level=2, block=(16, 16, 1))
    st = settings()
    U, B = wl.orszag_tang(mesh, gamma=st.gamma0)
    impl = GodunovImplemGB300(st, mesh)
    dt = st.cfl / impl.compute_inv_dt(_dev(U), _dev(B))
    U2, B2 = impl.step_host(U, B, dt)
    U2o, B2o = oracle_lib.step(oracle_mesh(oracle_lib, mesh), oracle_settings(oracle_lib, st), U, B, dt)
    assert max_rel_diff(U2, U2o) <= TOL_FP64 and max_rel_diff(B2, B2o) <= TOL_FP64


@pytest.mark.parametrize("dim,level,block,precision,tile", [
    (3, 2, (16, 16, 16), "mixed", 0), (3, 2, (16, 16, 16), "fp64", 0), (3, 2, (32, 32, 32), "mixed", 16),
    (2, 4, (16, 16, 1), "mixed", 0), (2, 4, (16, 16, 1), "fp64", 0)])
def test_step_host_chunked_matches_step(dim, level, block, precision, tile):
    """gmhd_step_host copies in, steps and copies out in chunks of blocks that overlap one another:
    the result equals gmhd_step on device buffers bit for bit (pinned and pageable host buffers)."""
    mesh = BlockMesh.uniform(dim, level=level, block=block)
    assert mesh.n_owned >= 16
    st = settings()
    U, B = wl.orszag_tang(mesh, gamma=st.gamma0, rho_perturbation=1e-3 if dim == 3 else 0.0, seed=2)
    impl = GodunovImplemGB300(st, mesh, precision=precision)
    if tile:
        impl.set_tile(tile)
    dU, dB = _dev(U), _dev(B)
    dU2, dB2 = torch.empty_like(dU), torch.empty_like(dB)
    dt = impl.compute_dt(dU, dB)
    impl.do_time_step(dU, dU2, dB, dB2, dt)
    torch.cuda.synchronize()
    ref_U, ref_B = dU2.cpu().numpy(), dB2.cpu().numpy()
    n = mesh.n_owned
    U2, B2 = impl.step_host(U, B, dt)
    assert np.array_equal(U2[:n], ref_U[:n]) and np.array_equal(B2[:n], ref_B[:n])
    hU, hB = torch.from_numpy(U).pin_memory(), torch.from_numpy(B).pin_memory()
    hU2, hB2 = torch.zeros_like(hU).pin_memory(), torch.zeros_like(hB).pin_memory()
    impl.step_host(hU.numpy(), hB.numpy(), dt, hU2.numpy(), hB2.numpy())
    assert np.array_equal(hU2.numpy()[:n], ref_U[:n]) and np.array_equal(hB2.numpy()[:n], ref_B[:n])


@pytest.mark.parametrize("case", ["batch", "walls"])
def test_step_host_batched_and_walled(case):
    """gmhd_step_host on a batch of independent problems (chunks by each problem's extent) and on a mesh
    with outside blocks (no chunking: the outside fill needs every block): equal to gmhd_step."""
    st = settings()
    if case == "batch":
        meshes, states, _ = wl.field_loop_batch(6, seed=5, sizes=(32, 64))
        mesh, problem = BlockMesh.batch(meshes)
        U = np.concatenate([s_[0] for s_ in states])
        B = np.concatenate([s_[1] for s_ in states])
        impl = GodunovImplemGB300(st, mesh, problem=problem, n_problems=len(meshes))
        dt = 1e-3
    else:
        mesh = BlockMesh.uniform(3, level=2, block=(8, 8, 8), periodic=(True, False, True))
        U, B = wl.kelvin_helmholtz(mesh, seed=3)
        impl = GodunovImplemGB300(settings(gamma0=1.4), mesh, bc=(1, 1, 3, 3, 1, 1))
        dU0, dB0 = _dev(U), _dev(B)
        impl.fill_outside(dU0, dB0)
        U, B = dU0.cpu().numpy(), dB0.cpu().numpy()
        dt = 0.2 / float(np.max(impl.compute_inv_dt(dU0, dB0)))
    assert mesh.n_owned >= 16
    dU, dB = _dev(U), _dev(B)
    dU2, dB2 = torch.empty_like(dU), torch.empty_like(dB)
    impl.do_time_step(dU, dU2, dB, dB2, dt)
    torch.cuda.synchronize()
    n = mesh.n_owned
    U2, B2 = impl.step_host(U, B, dt)
    assert np.array_equal(U2[:n], dU2.cpu().numpy()[:n]) and np.array_equal(B2[:n], dB2.cpu().numpy()[:n])


@pytest.mark.parametrize("dim", [2, 3])
def test_uniform_state_preserved(dim):
    mesh = BlockMesh.uniform(dim, level=1 if dim == 3 else 2, block=(16, 16, 16) if dim == 3 else (16, 16, 1))
    st = settings(gamma0=1.4)
    U, B = wl.uniform_state(mesh)
    for prec in ("fp64", "mixed"):
        impl = GodunovImplemGB300(st, mesh, precision=prec)
        dU, dB = _dev(U), _dev(B)
        impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), 4)
        assert np.array_equal(dB.cpu().numpy(), B)
        assert np.max(np.abs(dU.cpu().numpy() - U)) <= (0.0 if prec == "fp64" else 1e-12)


@pytest.mark.parametrize("dim,block,level,nsteps", [(2, (16, 16, 1), 3, 100), (3, (32, 32, 32), 1, 20)])
def test_mixed_precision_accuracy(dim, block, level, nsteps):
    mesh = BlockMesh.uniform(dim, level=level, block=block)
    st = settings()
    U, B = wl.orszag_tang(mesh, gamma=st.gamma0, rho_perturbation=1e-3 if dim == 3 else 0.0, seed=1)
    out = {}
    for prec in ("fp64", "mixed"):
        impl = GodunovImplemGB300(st, mesh, precision=prec)
        dU, dB = _dev(U), _dev(B)
        impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), nsteps)
        out[prec] = (dU.cpu().numpy(), dB.cpu().numpy())
    n = mesh.n_owned
    l1_rho = l1_rel(out["mixed"][0][:n, 0], out["fp64"][0][:n, 0])
    l1_e = l1_rel(out["mixed"][0][:n, 1], out["fp64"][0][:n, 1])
    l1_b = l1_rel(out["mixed"][1][:n], out["fp64"][1][:n])
    divb = float(np.max(np.abs(div_b(mesh, out["mixed"][1]))))
    print(f"mixed vs fp64 after {nsteps} steps: L1(rho)={l1_rho:.3e} L1(E)={l1_e:.3e} L1(B)={l1_b:.3e} "
          f"max|divB|={divb:.3e}")
    assert l1_rho <= 1e-6
    assert divb <= 1e-12
    # conservation on a periodic mesh: exact to FP64 round-off on both paths (the mixed path sums each
    # cell's face-flux terms error-free in FP32, a head and a tail, and adds both to U in FP64)
    for v in (0, 1):
        m0 = U[:n, v].sum()
        drift64 = abs(out["fp64"][0][:n, v].sum() - m0) / abs(m0)
        drift32 = abs(out["mixed"][0][:n, v].sum() - m0) / abs(m0)
        print(f"var {v}: relative drift fp64 {drift64:.2e} mixed {drift32:.2e}")
        assert drift64 <= 1e-13
        assert drift32 <= 1e-13


def test_alias_and_argument_errors():
    from godunov_mhd_ct_gb300._native import NativeError

    mesh = BlockMesh.uniform(2, level=1, block=(8, 8, 1))
    impl = GodunovImplemGB300(settings(), mesh)
    U, B = wl.uniform_state(mesh)
    dU, dB = _dev(U), _dev(B)
    with pytest.raises(NativeError):
        impl.do_time_step(dU, dU, dB, dB.clone(), 1e-3)
    with pytest.raises(NativeError):
        impl.do_time_step(dU, dU.clone(), dB, dB.clone(), float("nan"))


def test_step_host_async_matches_step(oracle_lib):
    """gmhd_step_host_async: consecutive overlapped calls give the same results as gmhd_step."""
    import ctypes

    from godunov_mhd_ct_gb300 import _native as nat

    mesh = BlockMesh.uniform(3, level=1, block=(16, 16, 16))
    st = settings()
    U, B = wl.orszag_tang(mesh, gamma=st.gamma0)
    impl = GodunovImplemGB300(st, mesh, precision="mixed")
    dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    dU2, dB2 = torch.empty_like(dU), torch.empty_like(dB)
    dt = impl.compute_dt(dU, dB)
    impl.do_time_step(dU, dU2, dB, dB2, dt)
    torch.cuda.synchronize()
    ref_U, ref_B = dU2.cpu().numpy(), dB2.cpu().numpy()
    hU, hB = torch.from_numpy(U).pin_memory(), torch.from_numpy(B).pin_memory()
    outs = [(torch.zeros_like(hU).pin_memory(), torch.zeros_like(hB).pin_memory()) for _ in range(5)]
    s = torch.cuda.current_stream()
    for hU2, hB2 in outs:
        nat.check(nat.lib().gmhd_step_host_async(impl._ctx, hU.data_ptr(), hU2.data_ptr(), hB.data_ptr(),
                                                 hB2.data_ptr(), ctypes.c_double(dt), ctypes.c_void_p(s.cuda_stream)),
                  "gmhd_step_host_async")
    s.synchronize()
    n = mesh.n_owned
    for hU2, hB2 in outs:
        assert np.array_equal(hU2.numpy()[:n], ref_U[:n])
        assert np.array_equal(hB2.numpy()[:n], ref_B[:n])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_empty_mesh_is_a_no_op(precision):
    """A mesh without blocks (a rank that owns no leaves): every call succeeds and touches nothing."""
    mesh = BlockMesh(dim=3, block=(8, 8, 8), level=np.zeros(0, np.int32), neighbor=np.zeros((0, 27), np.int32),
                     coords=np.zeros((0, 3), np.int64), n_owned=0, grid=(1, 1, 1), periodic=(True, True, True))
    assert not mesh.is_amr
    impl = GodunovImplemGB300(settings(), mesh, precision=precision)
    sentinel = torch.full((16,), 7.0, dtype=torch.float64, device="cuda")
    U, U2, B, B2 = (sentinel.clone() for _ in range(4))
    impl.do_time_step(U, U2, B, B2, 1e-3)
    impl.fill_outside(U, B)
    assert impl.compute_inv_dt(U, B) == 0.0
    torch.cuda.synchronize()
    for x in (U, U2, B, B2):
        assert torch.equal(x, sentinel)
    assert impl.last_status() == 0
    hU2, hB2 = impl.step_host(np.zeros(0), np.zeros(0), 1e-3)
    assert hU2.size == 0 and hB2.size == 0
    impl.close()

"""Outside-block fill (border_conditions/FillOutside.cpp) and non-periodic meshes: GPU vs oracle."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_mhd_ct_gb300 import workloads as wl  # noqa: E402
from godunov_mhd_ct_gb300.mesh import BlockMesh  # noqa: E402
from godunov_mhd_ct_gb300.solver import GodunovImplemGB300  # noqa: E402

from .helpers import max_rel_diff, oracle_mesh, oracle_settings, settings  # noqa: E402

pytestmark = pytest.mark.gpu
TOL_FP64 = 1e-12
WALL, ZG, PER = 3, 2, 1


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


CASES = [
    # dim, block, level, periodic, bc per face (XMIN..ZMAX)
    (3, (8, 8, 8), 1, (True, False, True), (PER, PER, WALL, WALL, PER, PER)),
    (2, (16, 16, 1), 2, (False, False, True), (ZG, ZG, WALL, WALL, PER, PER)),
    (2, (8, 8, 1), 2, (False, True, True), (ZG, WALL, PER, PER, PER, PER)),
    (3, (8, 8, 8), 1, (False, False, False), (ZG, ZG, ZG, ZG, ZG, ZG)),
]


@pytest.mark.parametrize("dim,block,level,periodic,bc", CASES)
def test_fill_outside_matches_oracle(oracle_lib, dim, block, level, periodic, bc):
    mesh = BlockMesh.uniform(dim, level=level, block=block, periodic=periodic)
    assert mesh.n_blocks > mesh.n_owned
    st = settings(gamma0=1.4)
    U, B = wl.kelvin_helmholtz(mesh, seed=4)
    impl = GodunovImplemGB300(st, mesh, bc=bc)
    dU, dB = _dev(U), _dev(B)
    impl.fill_outside(dU, dB)
    torch.cuda.synchronize()
    Uo, Bo = oracle_lib.fill_outside(oracle_mesh(oracle_lib, mesh, bc), U, B)
    assert np.array_equal(dU.cpu().numpy(), Uo)
    assert np.array_equal(dB.cpu().numpy(), Bo)


@pytest.mark.parametrize("dim,block,level,periodic,bc", CASES)
def test_non_periodic_run_fp64_matches_oracle(oracle_lib, dim, block, level, periodic, bc):
    """Solver loop with walls / zero-gradient borders: fill outside, then step, every iteration."""
    mesh = BlockMesh.uniform(dim, level=level, block=block, periodic=periodic)
    st = settings(gamma0=1.4)
    U, B = wl.kelvin_helmholtz(mesh, seed=9)
    nsteps = 8
    Uo, Bo, dto = oracle_lib.run(oracle_mesh(oracle_lib, mesh, bc), oracle_settings(oracle_lib, st), U, B, nsteps)
    impl = GodunovImplemGB300(st, mesh, precision="fp64", bc=bc)
    dU, dB = _dev(U), _dev(B)
    dtg, _ = impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), nsteps)
    n = mesh.n_owned
    Ug, Bg = dU.cpu().numpy()[:n], dB.cpu().numpy()[:n]
    assert max_rel_diff(dtg[:, 0], dto) <= TOL_FP64
    assert max_rel_diff(Ug, Uo[:n]) <= TOL_FP64
    assert max_rel_diff(Bg, Bo[:n]) <= TOL_FP64
    print(f"bit-identical U: {np.array_equal(Ug, Uo[:n])} B: {np.array_equal(Bg, Bo[:n])}")


def test_mixed_walls_accuracy(oracle_lib):
    mesh = BlockMesh.uniform(3, level=2, block=(8, 8, 8), periodic=(True, False, True))
    bc = (PER, PER, WALL, WALL, PER, PER)
    st = settings(gamma0=1.4)
    U, B = wl.kelvin_helmholtz(mesh, seed=2)
    out = {}
    for prec in ("fp64", "mixed"):
        impl = GodunovImplemGB300(st, mesh, precision=prec, bc=bc)
        dU, dB = _dev(U), _dev(B)
        impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), 10)
        out[prec] = dU.cpu().numpy()[: mesh.n_owned]
    l1 = float(np.abs(out["mixed"][:, 0] - out["fp64"][:, 0]).sum() / np.abs(out["fp64"][:, 0]).sum())
    assert l1 <= 1e-6


def _golden_outside():
    import importlib.util
    import os
    here = os.path.dirname(__file__)
    spec = importlib.util.spec_from_file_location("make_golden_outside",
                                                  os.path.join(here, "golden", "make_golden_outside.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    return gen, np.load(os.path.join(here, "golden", "functor_outside.npz"))


@pytest.mark.parametrize("name", ["2d_walls", "2d_zero_gradient", "2d_mixed", "2d_mixed_amr", "3d_mixed",
                                  "3d_yz_amr"])
def test_fill_outside_matches_reference_golden(name):
    """The GPU outside fill on the recorded cases (ZERO_GRADIENT and WALL mixed per face, uniform and
    two-level meshes) reproduces the digests of the reference's FillOutsideCellFunctor."""
    import hashlib
    gen, golden = _golden_outside()
    mesh, _, bc, U, B = gen.case_inputs(name)
    impl = GodunovImplemGB300(settings(gamma0=gen.GAMMA), mesh, bc=tuple(bc))
    dU, dB = _dev(U), _dev(B)
    impl.fill_outside(dU, dB)
    torch.cuda.synchronize()
    n = mesh.n_owned
    Ug, Bg = dU.cpu().numpy(), dB.cpu().numpy()
    assert hashlib.sha256(np.ascontiguousarray(Ug[n:]).tobytes()).hexdigest() == str(golden[f"{name}_sha_U"])
    assert hashlib.sha256(np.ascontiguousarray(Bg[n:]).tobytes()).hexdigest() == str(golden[f"{name}_sha_B"])

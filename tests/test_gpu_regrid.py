"""AMR cycle on the GPU (refinement flags, remap, new tables) against the oracle, bit for bit, and a
solver loop with a regrid every few steps (SolverGodunovMHD::next_iteration_impl, .cpp:407-420)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_mhd_ct_gb300 import workloads as wl  # noqa: E402
from godunov_mhd_ct_gb300.mesh import BlockMesh  # noqa: E402
from godunov_mhd_ct_gb300.solver import GodunovImplemGB300  # noqa: E402

from .helpers import oracle_settings, same_level_face_mismatch, settings  # noqa: E402
from .test_gpu_amr import MESHES  # noqa: E402

pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


CRIT = [("LOHNER_UNSPLIT", ("rho",), 0.05, 0.01), ("SIMPLE_GRADIENT", ("rho", "pressure"), 0.05, 0.005)]


@pytest.mark.parametrize("name", ["2d_b8", "3d_b8", "2d_b16"])
@pytest.mark.parametrize("crit,variables,er,ec", CRIT)
def test_refine_flags_bit_exact(oracle_lib, name, crit, variables, er, ec):
    mesh = MESHES[name]()
    st = settings(gamma0=1.4)
    U, B = wl.random_smooth(mesh, seed=6)
    lv = np.unique(mesh.level[: mesh.n_owned])
    impl = GodunovImplemGB300(st, mesh, precision="fp64")
    fg = impl.refine_flags(_dev(U), _dev(B), criterion=crit, level_min=int(lv[0]), level_max=int(lv[-1]) + 1,
                           eps_refine=er, eps_coarsen=ec, variables=variables)
    fo = oracle_lib.refine_flags(oracle_lib.Mesh.from_block_mesh(mesh), oracle_settings(oracle_lib, st), U, B,
                                 criterion=crit, level_min=int(lv[0]), level_max=int(lv[-1]) + 1, eps_refine=er,
                                 eps_coarsen=ec, use_rho="rho" in variables, use_pressure="pressure" in variables)
    assert np.array_equal(fg, fo)


@pytest.mark.parametrize("name", ["2d_b8", "3d_b8", "3d_b4"])
@pytest.mark.parametrize("mode", ["refine_coarse", "coarsen_fine", "mixed"])
def test_remap_bit_exact(oracle_lib, name, mode):
    mesh = MESHES[name]()
    st = settings(gamma0=1.4)
    U, B = wl.random_smooth(mesh, seed=2)
    lv = mesh.level[: mesh.n_owned]
    lo, hi = int(lv.min()), int(lv.max())
    if mode == "refine_coarse":
        flags = np.where(lv == lo, 1, 0)
    elif mode == "coarsen_fine":
        flags = np.where(lv == hi, -1, 0)
    else:
        flags = np.random.default_rng(3).integers(-1, 2, mesh.n_owned)
    new, table = mesh.adapt(flags, lo, hi + 1)
    us, bs = new.alloc_state()
    Uo, Bo = oracle_lib.remap(oracle_lib.Mesh.from_block_mesh(mesh), oracle_lib.Mesh.from_block_mesh(new), table,
                              U, B, (us.shape, bs.shape))
    impl = GodunovImplemGB300(st, mesh, precision="fp64")
    from godunov_mhd_ct_gb300 import _native as nat

    Un = torch.zeros(us.shape, dtype=torch.float64, device="cuda")
    Bn = torch.zeros(bs.shape, dtype=torch.float64, device="cuda")
    t = np.ascontiguousarray(table, dtype=np.int32)
    bx, by, bz = mesh.block
    dU, dB = _dev(U), _dev(B)
    nat.check(nat.lib().gmhd_remap(mesh.dim, bx, by, bz, mesh.n_blocks, new.n_owned, t.ctypes.data, dU.data_ptr(),
                                   dB.data_ptr(), Un.data_ptr(), Bn.data_ptr(), None), "gmhd_remap")
    n = new.n_owned
    assert np.array_equal(Un.cpu().numpy()[:n], Uo[:n])
    assert np.array_equal(Bn.cpu().numpy()[:n], Bo[:n])
    assert same_level_face_mismatch(new, Bn.cpu().numpy()) == 0.0
    del impl


@pytest.mark.parametrize("dim", [2, 3])
def test_run_with_regrid_bit_exact(oracle_lib, dim):
    """steps, AMR cycle, steps, AMR cycle, ... on GPU and oracle."""
    if dim == 2:
        mesh = wl.blast_mesh(base_level=2, max_level=3, block=8, radius=0.15, band=0.05)
        U, B = wl.blast(mesh, radius=0.15)
        lmin, lmax = 2, 4
    else:
        mesh = MESHES["3d_b4"]()
        U, B = wl.random_smooth(mesh, seed=4)
        lmin, lmax = 1, 3
    st = settings(gamma0=5.0 / 3.0, cfl=0.4)
    crit = dict(criterion="LOHNER_UNSPLIT", eps_refine=0.1, eps_coarsen=0.02, eps_lohner=0.02)
    impl = GodunovImplemGB300(st, mesh, precision="fp64")
    dU, dB = _dev(U), _dev(B)
    om, Uo, Bo = mesh, U.copy(), B.copy()
    changed = 0
    for cycle in range(3):
        # GPU
        dtg, _ = impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), 3)
        new_g, dU, dB = impl.regrid(dU, dB, lmin, lmax, **crit)
        # oracle
        orm = oracle_lib.Mesh.from_block_mesh(om)
        Uo, Bo, dto = oracle_lib.run(orm, oracle_settings(oracle_lib, st), Uo, Bo, 3)
        fl = oracle_lib.refine_flags(orm, oracle_settings(oracle_lib, st), Uo, Bo, level_min=lmin, level_max=lmax,
                                     **{k: v for k, v in crit.items() if k != "criterion"},
                                     criterion=crit["criterion"])
        om2, table = om.adapt(fl, lmin, lmax)
        changed += int(np.any(table[:, 0] != 0))
        us, bs = om2.alloc_state()
        Uo, Bo = oracle_lib.remap(orm, oracle_lib.Mesh.from_block_mesh(om2), table, Uo, Bo, (us.shape, bs.shape))
        om = om2
        assert np.array_equal(dtg[:, 0], dto)
        assert new_g.n_owned == om.n_owned
        n = om.n_owned
        assert np.array_equal(dU.cpu().numpy()[:n], Uo[:n])
        assert np.array_equal(dB.cpu().numpy()[:n], Bo[:n])
    assert changed > 0

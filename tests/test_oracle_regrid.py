"""AMR cycle on the oracle (CPU): BlockMesh.adapt + refinement flags + remap keep mass and energy,
keep div B at round-off, and leave the copies of same-level shared faces identical."""
import numpy as np
import pytest

from godunov_mhd_ct_gb300 import workloads as wl
from godunov_mhd_ct_gb300.mesh import BlockMesh

from .helpers import same_level_face_mismatch
from .test_oracle_amr import amr_mesh, div_b, totals

orc = pytest.importorskip("oracle.oracle")


def _remap(m, flags, lmin, lmax, U, B):
    new, table = m.adapt(flags, lmin, lmax)
    us, bs = new.alloc_state()
    U2, B2 = orc.remap(orc.Mesh.from_block_mesh(m), orc.Mesh.from_block_mesh(new), table, U, B, (us.shape, bs.shape))
    return new, table, U2, B2


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("mode", ["indicator", "refine_coarse", "coarsen_fine", "random"])
def test_regrid_invariants(dim, mode):
    m = amr_mesh(dim)
    U, B = wl.random_smooth(m, seed=3)
    st = orc.settings(gamma0=1.4, cfl=0.4, slope_type=2.0, riemann=5)
    lv = m.level[: m.n_owned]
    lmin, lmax = int(lv.min()), int(lv.max())
    if mode == "indicator":
        flags = orc.refine_flags(orc.Mesh.from_block_mesh(m), st, U, B, level_min=lmin, level_max=lmax + 1,
                                 eps_refine=0.05, eps_coarsen=0.01)
    elif mode == "refine_coarse":
        flags = np.where(lv == lmin, 1, 0)
    elif mode == "coarsen_fine":
        flags = np.where(lv == lmax, -1, 0)
    else:
        flags = np.random.default_rng(5).integers(-1, 2, m.n_owned)
    new, table, U2, B2 = _remap(m, flags, lmin, lmax + 1, U, B)
    t0, t1 = totals(m, U), totals(new, U2)
    assert abs(t1[0] - t0[0]) <= 1e-14 * abs(t0[0])
    assert abs(t1[1] - t0[1]) <= 1e-14 * abs(t0[1])
    assert div_b(new, B2) < 1e-12
    assert same_level_face_mismatch(new, B2) == 0.0
    # and the scheme runs on the adapted mesh with the same invariants
    U3, B3, _ = orc.run(orc.Mesh.from_block_mesh(new), st, U2, B2, 3)
    assert div_b(new, B3) < 1e-11
    assert same_level_face_mismatch(new, B3) == 0.0


def test_adapt_refine_then_coarsen_is_identity_on_u():
    """Refining every leaf then coarsening every family gives back U exactly (copy, then mean of
    equal values) and B up to the mean of prolonged faces."""
    m = BlockMesh.uniform(2, level=2, block=(8, 8, 1))
    U, B = wl.random_smooth(m, seed=1)
    fine, t1, Uf, Bf = _remap(m, np.ones(m.n_owned), 2, 3, U, B)
    assert np.bincount(t1[:, 0], minlength=3)[1] == fine.n_owned
    back, t2, Ub, Bb = _remap(fine, -np.ones(fine.n_owned), 2, 3, Uf, Bf)
    assert back.n_owned == m.n_owned
    np.testing.assert_array_equal(Ub[: m.n_owned], U[: m.n_owned])
    np.testing.assert_allclose(Bb[: m.n_owned], B[: m.n_owned], rtol=0, atol=1e-15)


def test_refine_flags_thresholds():
    m = amr_mesh(2)
    U, B = wl.uniform_state(m)
    st = orc.settings(gamma0=1.4)
    lv = m.level[: m.n_owned]
    flags = orc.refine_flags(orc.Mesh.from_block_mesh(m), st, U, B, level_min=int(lv.min()),
                             level_max=int(lv.max()) + 1)
    # a uniform state has zero error: every block above level_min coarsens, the others are kept
    assert np.array_equal(flags, np.where(lv > lv.min(), -1, 0).astype(np.int8))

"""Oracle on 2:1-balanced AMR meshes (CPU): the invariants the reference scheme guarantees by
construction hold across coarse/fine borders.

* an exactly uniform state is preserved;
* discrete div B stays at round-off (ReadEmfAndUpdateFunctor.cpp:118-161 is an exact curl, and the
  coarse/fine EMF correction of CorrectEmfAtBlockBorderFunctor.cpp:94-360 keeps shared faces
  consistent);
* total mass and energy are conserved on periodic meshes (the fine-flux sum of
  ReadFluxesAndConservativeUpdateFunctor.cpp:141-172 replaces the coarse face flux);
* a coarse face on a coarse/fine border stays the mean of the fine faces covering it;
* both hydro prolongations ([amr] cell_centered_prolongation_type) run.
"""
import numpy as np
import pytest

from godunov_mhd_ct_gb300 import workloads as wl
from godunov_mhd_ct_gb300.mesh import BlockMesh, nb_slot

from .helpers import same_level_face_mismatch

orc = pytest.importorskip("oracle.oracle")


def refine_ball(center, radius):
    """Refine the leaves whose box crosses the sphere |x - center| = radius (2D: circle)."""
    c = np.asarray(center, dtype=np.float64)

    def f(level, lo, hi):
        dim = 3 if hi[2] - lo[2] < 1.0 else 2
        p = np.clip(c, lo, hi)
        near = np.sqrt(((p - c)[:dim] ** 2).sum())
        far = np.sqrt((np.maximum(np.abs(lo - c), np.abs(hi - c))[:dim] ** 2).sum())
        return near < radius < far

    return f


def amr_mesh(dim):
    if dim == 2:
        return BlockMesh.amr(2, refine_ball((0.5, 0.5, 0.5), 0.3), base_level=2, max_level=4, block=(8, 8, 1))
    return BlockMesh.amr(3, refine_ball((0.3, 0.3, 0.3), 0.2), base_level=1, max_level=3, block=(4, 4, 4))


def div_b(m, B):
    Bx, By, Bz = m.split_faces(B)
    d = (Bx[..., 1:] - Bx[..., :-1]) + (By[..., 1:, :] - By[..., :-1, :])
    if m.dim == 3:
        d = d + (Bz[:, 1:] - Bz[:, :-1])
    return float(np.abs(d / m.block_dx()[:, None, None, None])[: m.n_owned].max())


def totals(m, U):
    vol = (m.block_dx() ** m.dim)[: m.n_owned, None, None, None]
    return [float((U[: m.n_owned, v] * vol).sum()) for v in (0, 1)]


def coarse_fine_face_gap(m, B):
    """max |coarse face - mean of the fine faces covering it| over x faces on coarse/fine borders."""
    Bx = m.split_faces(B)[0]
    bx, by, bz = m.block
    worst = 0.0
    for b in range(m.n_owned):
        for side in (-1, 1):
            s = nb_slot(side, 0, 0)
            if m.fine_neighbor is None or m.neighbor[b, s] >= 0:
                continue
            for c in range(1 << m.dim):
                child = m.fine_neighbor[b, s, c]
                cc = (c & 1, (c >> 1) & 1, (c >> 2) & 1)
                if child < 0 or cc[0] != (1 if side < 0 else 0):
                    continue
                ff = Bx[child][..., bx if side < 0 else 0]
                cf = Bx[b][..., 0 if side < 0 else bx]
                if m.dim == 2:
                    avg = 0.5 * (ff[:, 0::2] + ff[:, 1::2])
                    sub = cf[:, cc[1] * by // 2: (cc[1] + 1) * by // 2]
                else:
                    avg = 0.25 * (ff[0::2, 0::2] + ff[0::2, 1::2] + ff[1::2, 0::2] + ff[1::2, 1::2])
                    sub = cf[cc[2] * bz // 2: (cc[2] + 1) * bz // 2, cc[1] * by // 2: (cc[1] + 1) * by // 2]
                worst = max(worst, float(np.abs(sub - avg).max()))
    return worst


@pytest.mark.parametrize("dim", [2, 3])
def test_mesh_is_balanced_and_consistent(dim):
    m = amr_mesh(dim)
    assert m.fine_neighbor is not None
    assert len(set(m.level[: m.n_owned].tolist())) > 1
    n_jumps = 0
    for b in range(m.n_owned):
        for s in range(27):
            n = m.neighbor[b, s]
            if n >= 0:
                assert abs(int(m.level[n]) - int(m.level[b])) <= 1
                n_jumps += m.level[n] != m.level[b]
            elif s != 13 and (dim == 3 or 9 <= s < 18):
                ch = m.fine_neighbor[b, s][: 1 << dim]
                assert (ch >= 0).any()
                assert all(m.level[c] == m.level[b] + 1 for c in ch if c >= 0)
    assert n_jumps > 0


@pytest.mark.parametrize("dim", [2, 3])
def test_uniform_state_is_preserved(dim):
    m = amr_mesh(dim)
    om = orc.Mesh.from_block_mesh(m)
    st = orc.settings(gamma0=1.4, cfl=0.4, slope_type=2.0, riemann=5)
    U, B = wl.uniform_state(m)
    U2, B2 = orc.step(om, st, U, B, 1e-3)
    np.testing.assert_array_equal(U2[: m.n_owned], U[: m.n_owned])
    np.testing.assert_array_equal(B2[: m.n_owned], B[: m.n_owned])


@pytest.mark.parametrize("dim,prolongation", [(2, 0), (2, 1), (3, 0), (3, 1)])
def test_conservation_and_div_b(dim, prolongation):
    m = amr_mesh(dim)
    om = orc.Mesh.from_block_mesh(m, prolongation=prolongation)
    st = orc.settings(gamma0=1.4, cfl=0.4, slope_type=2.0, riemann=5)
    U, B = wl.random_smooth(m, seed=3)
    t0 = totals(m, U)
    assert div_b(m, B) < 1e-12
    U2, B2, dts = orc.run(om, st, U, B, 10)
    t1 = totals(m, U2)
    assert np.all(dts > 0)
    assert abs(t1[0] - t0[0]) <= 1e-13 * abs(t0[0])
    assert abs(t1[1] - t0[1]) <= 1e-13 * abs(t0[1])
    assert div_b(m, B2) < 1e-11
    assert coarse_fine_face_gap(m, B2) < 1e-14
    # every block sees one value per face, so same-level copies of shared faces stay identical
    assert same_level_face_mismatch(m, B) == 0.0
    assert same_level_face_mismatch(m, B2) == 0.0


def test_prolongation_types_differ():
    m = amr_mesh(2)
    st = orc.settings(gamma0=1.4, cfl=0.4, slope_type=2.0, riemann=5)
    U, B = wl.random_smooth(m, seed=3)
    a, _, _ = orc.run(orc.Mesh.from_block_mesh(m, prolongation=0), st, U, B, 3)
    b, _, _ = orc.run(orc.Mesh.from_block_mesh(m, prolongation=1), st, U, B, 3)
    assert np.abs(a - b).max() > 1e-6

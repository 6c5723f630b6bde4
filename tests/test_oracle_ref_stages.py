"""Pin the oracle's per-block stages against the reference's own stage functors.

The golden arrays (tests/golden/functor_stages.npz, recorded by tests/golden/make_golden_stages.py)
are the output of the reference's ComputeLimitedSlopesFunctor, ComputeUpdatedPrimitiveVariablesFunctor
(Hancock predictor with the gravity and viscous terms, and the RK2_SSP identity),
ComputeElectricFieldFunctor, ComputeSourceFaceMagFunctor, ComputeHydroFluxesAndStoreFunctor (HLLD),
ComputeEmfAndStoreFunctor (edge reconstruction + 2D HLLD), ComputeViscousFluxesAndStoreFunctor,
ReadEmfAndUpdateFunctor (CT update), ComputeDtMHDFunctor (CFL with the gravity and viscous
limits), AddGravitySourceTerm and ReadFluxesAndConservativeUpdateFunctor, compiled unmodified, on the ghosted primitive variables the oracle builds for one block. The
oracle must reproduce the slopes, the predictor, the edge electric field, the half-step face source,
the face fluxes, the raw edge EMFs, the viscous fluxes, the conservative update by the fluxes, the CT
update, the CFL reduction and the gravity source bit for bit (2D fluxes: the variables the reference stores, rho, E, rho u, rho v, rho w, Bz). Where the reference tree
is present the same comparison also runs live on further states.
"""
import os

import numpy as np
import pytest


orc = pytest.importorskip("oracle.oracle")
HERE = os.path.dirname(__file__)
GOLDEN = os.path.join(HERE, "golden", "functor_stages.npz")

import importlib.util  # noqa: E402

_spec = importlib.util.spec_from_file_location("make_golden_stages", os.path.join(HERE, "golden", "make_golden_stages.py"))
gen = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(gen)


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("name", sorted(gen.CASES))
def test_oracle_stages_match_reference_functors(golden, name):
    dim, kind, gamma, slope, rk2, grav, mu, pred = gen.CASES[name]
    mesh = gen.case_mesh(dim)
    om = orc.Mesh.from_block_mesh(mesh)
    st = gen.oracle_settings(gamma, slope, rk2, grav, mu, pred)
    out = orc.block_stages(om, st, golden[f"{name}_U"], golden[f"{name}_B"], float(golden[f"{name}_dt"]), 1)
    assert np.array_equal(out["q"], golden[f"{name}_q"])
    for k in ("slopes", "q2", "e", "sf"):
        assert np.array_equal(out[k], golden[f"{name}_{k}"]), k
    fl, emf = orc.block_fluxes_emf(om, st, golden[f"{name}_U"], golden[f"{name}_B"], float(golden[f"{name}_dt"]), 1)
    _same_fluxes_emf(dim, fl, emf, golden[f"{name}_fluxes"], golden[f"{name}_emf"])
    # CT update of the block's faces by the reference's EMFs, and the CFL reduction over the mesh
    assert np.array_equal(_oracle_ct(dim, mesh.block, golden[f"{name}_emf"], golden[f"{name}_B"][1]),
                          golden[f"{name}_ct_B"])
    assert orc.inv_dt(om, st, golden[f"{name}_U"], golden[f"{name}_B"]) == float(golden[f"{name}_inv_dt"])
    if mu is not None:
        vf = orc.block_viscous_fluxes(om, st, golden[f"{name}_U"], golden[f"{name}_B"], float(golden[f"{name}_dt"]), 1)
        _same_fluxes(dim, vf, golden[f"{name}_visc"])
    U1, B1 = orc.block_update(om, 1, golden[f"{name}_fluxes"], golden[f"{name}_U"][1], golden[f"{name}_B"][1])
    if mu is not None:
        U1, B1 = orc.block_update(om, 1, golden[f"{name}_visc"], U1, B1)
    assert np.array_equal(U1, golden[f"{name}_upd_U"]) and np.array_equal(B1, golden[f"{name}_upd_B"])
    if grav is not None:
        Uold, Unew = gen.gravity_inputs(mesh, golden[f"{name}_U"])
        got = orc.gravity_source(dim, mesh.block, grav, float(golden[f"{name}_dt"]), Uold, Unew)
        assert np.array_equal(got, golden[f"{name}_grav_U"])


def _same_fluxes(dim, fl, ref_fl, block=None):
    """Per direction [8][faces]; in 2D only the variables the reference stores (rho, E, rho u, rho v,
    rho w, Bz)."""
    block = block or ((8, 8, 1) if dim == 2 else (4, 4, 4))
    stored = list(range(8)) if dim == 3 else [0, 1, 2, 3, 4, 7]
    off = 0
    for dr in range(dim):
        n = int(np.prod([block[d] + (d == dr) for d in range(dim)]))
        a = fl[off:off + 8 * n].reshape(8, n)
        b = ref_fl[off:off + 8 * n].reshape(8, n)
        for v in stored:
            assert np.array_equal(a[v], b[v]), ("flux", dr, v)
        off += 8 * n


def _oracle_ct(dim, block, ref_emf, B):
    """The oracle's CT update on one block, fed the reference's [3][(b+1)^d] edge array (2D: z only)."""
    ne = ref_emf.size // 3
    emf = ref_emf[2 * ne:] if dim == 2 else ref_emf
    return orc.ct_update(dim, block, emf, B[None])[0]


def _same_fluxes_emf(dim, fl, emf, ref_fl, ref_emf, block=None):
    """Oracle fluxes / EMFs against the reference's: per direction a [8][faces] block; in 2D the
    reference stores six flux variables, and its single EMF component is the z one of its edge array."""
    block = block or ((8, 8, 1) if dim == 2 else (4, 4, 4))
    stored = list(range(8)) if dim == 3 else [0, 1, 2, 3, 4, 7]
    off = 0
    for dr in range(dim):
        n = int(np.prod([block[d] + (d == dr) for d in range(dim)]))
        a = fl[off:off + 8 * n].reshape(8, n)
        b = ref_fl[off:off + 8 * n].reshape(8, n)
        for v in stored:
            assert np.array_equal(a[v], b[v]), ("flux", dr, v)
        off += 8 * n
    ne = emf.size // (3 if dim == 3 else 1)
    want = ref_emf[2 * ne:3 * ne] if dim == 2 else ref_emf
    assert np.array_equal(emf, want), "emf"


@pytest.mark.skipif(not os.path.isdir(os.environ.get("GMHD_REFERENCE_TREE", "/root/reference")),
                    reason="needs the reference tree")
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_stages_match_reference_functors_live(dim, seed):
    from godunov_mhd_ct_gb300 import workloads as wl

    if not orc.build_refkat() or not os.path.exists(gen.BRIDGE):
        pytest.skip("functor bridge not built")
    rng = np.random.default_rng(seed)
    mesh = gen.case_mesh(dim)
    gamma = [1.4, 5.0 / 3.0][seed % 2]
    slope = [1.0, 2.0][seed % 2]
    grav = tuple(rng.uniform(-1, 1, 3)) if seed == 2 else None
    mu, pred = (1e-3 * seed, seed != 1) if seed >= 2 else (None, False)
    rk2 = int(seed == 3)
    U, B = wl.random_smooth(mesh, gamma=gamma, seed=100 + seed, amp=0.4)
    om = orc.Mesh.from_block_mesh(mesh)
    st = gen.oracle_settings(gamma, slope, rk2, grav, mu, pred)
    dt = 0.4 / orc.inv_dt(om, st, U, B)
    for blk in range(mesh.n_owned):
        out = orc.block_stages(om, st, U, B, dt, blk)
        ref = gen.reference_stages(dim, mesh.block, int(mesh.level[blk]), gamma, slope, rk2, grav, mu, pred, dt,
                                   out["q"])
        for k in ("slopes", "q2", "e", "sf"):
            assert np.array_equal(out[k], ref[k]), (blk, k)
        fl, emf = orc.block_fluxes_emf(om, st, U, B, dt, blk)
        rfl, remf = gen.reference_fluxes_emf(dim, mesh.block, int(mesh.level[blk]), gamma, slope, rk2, grav, mu, pred,
                                             dt, out)
        _same_fluxes_emf(dim, fl, emf, rfl, remf)
        if mu is not None:
            vf = orc.block_viscous_fluxes(om, st, U, B, dt, blk)
            _same_fluxes(dim, vf, gen.reference_viscous_fluxes(dim, mesh.block, int(mesh.level[blk]), gamma, slope, rk2,
                                                               grav, mu, pred, dt, out["q"]))
        args = (dim, mesh.block, gamma, slope, rk2, grav, mu, pred, dt)
        want = gen.reference_update(*args, rfl, U[blk], B[blk])
        got = orc.block_update(om, blk, rfl, U[blk], B[blk])
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1]), blk


@pytest.mark.skipif(not os.path.isdir(os.environ.get("GMHD_REFERENCE_TREE", "/root/reference")),
                    reason="needs the reference tree")
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("opts", ["plain", "gravity", "viscosity"])
def test_oracle_cfl_and_ct_match_reference_functors_live(dim, opts):
    """CFL reduction on a two-level mesh (per-block cell sizes) and the CT update by random EMFs."""
    from godunov_mhd_ct_gb300 import workloads as wl
    from godunov_mhd_ct_gb300.mesh import BlockMesh

    if not orc.build_refkat() or not os.path.exists(gen.BRIDGE):
        pytest.skip("functor bridge not built")
    block = (8, 8, 1) if dim == 2 else (4, 4, 4)
    mesh = BlockMesh.amr(dim, wl.refine_band((0.3, 0.3, 0.3), 0.0, 0.05, axes=dim), base_level=2, max_level=3,
                         block=block)
    assert len(set(mesh.level[:mesh.n_owned].tolist())) == 2
    gamma = 5.0 / 3.0
    grav = (0.4, -0.9, 0.3) if opts == "gravity" else None
    mu = 2e-2 if opts == "viscosity" else None
    U, B = wl.random_smooth(mesh, gamma=gamma, seed=7 + dim, amp=0.4)
    om = orc.Mesh.from_block_mesh(mesh)
    st = gen.oracle_settings(gamma, 2.0, 0, grav, mu, False)
    assert orc.inv_dt(om, st, U, B) == gen.reference_inv_dt(mesh, gamma, 2.0, 0, grav, mu, False, U, B)
    if grav is not None:
        Uold, Unew = gen.gravity_inputs(mesh, U)
        assert np.array_equal(orc.gravity_source(dim, block, grav, 0.013, Uold, Unew),
                              gen.reference_gravity(dim, block, grav, 0.013, Uold, Unew))
    rng = np.random.default_rng(dim)
    ne = int(np.prod([v + 1 for v in block[:dim]]))
    for blk in range(3):
        emf = rng.standard_normal(3 * ne) * 1e-2
        assert np.array_equal(_oracle_ct(dim, block, emf, B[blk]), gen.reference_ct(dim, block, emf, B[blk]))

"""Pin the oracle's coarse/fine stage code against the reference's own functors.

The golden arrays (tests/golden/functor_amr.npz, recorded by tests/golden/make_golden_amr.py) are the
output of the reference's CorrectEmfAtBlockBorderFunctor (border EMF averaging with same-level, finer
and coarser siblings, CorrectEmfAtBlockBorderFunctor.cpp:94-360) and of the coarse/fine branch of
ReadFluxesAndConservativeUpdateFunctor (a coarse cell next to finer leaves takes their face-flux sum
/ 2^d, ReadFluxesAndConservativeUpdateFunctor.cpp:103-436 with .h:233-270) and of
ConvertToPrimitivesVariablesFunctor (ghost cells from same-level, outside, finer and coarser leaves,
.cpp:173-719), compiled unmodified, on
two-level 2D and 3D meshes (periodic, and with reflecting walls). Their kalypsso-core lookups (edge
siblings, the finer face neighbour, the fine-face sum) come from the bridge's stencil-helper stub,
which states this build's definitions. The inputs (raw EMFs, face fluxes) are the oracle's own; the
oracle's correction, update and ghosted primitives must reproduce the reference's results bit for bit. Where the
reference tree is present the comparison also runs live on every owned block of further states."""
import importlib.util
import os

import numpy as np
import pytest

orc = pytest.importorskip("oracle.oracle")
HERE = os.path.dirname(__file__)
GOLDEN = os.path.join(HERE, "golden", "functor_amr.npz")
_spec = importlib.util.spec_from_file_location("make_golden_amr", os.path.join(HERE, "golden", "make_golden_amr.py"))
gen = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(gen)


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("name", sorted(gen.CASES))
def test_oracle_emf_correction_matches_reference(golden, name):
    mesh, om, st, U, B, dt, emf, fluxes = gen.case_inputs(name)
    assert dt == float(golden[f"{name}_dt"])
    sel = golden[f"{name}_blocks"]
    assert len(sel) == 0 or mesh.is_amr
    got = orc.correct_emf(om, emf)
    assert np.array_equal(got[sel], golden[f"{name}_emf_ref"])


@pytest.mark.parametrize("name", sorted(gen.CASES))
def test_oracle_coarse_fine_update_matches_reference(golden, name):
    mesh, om, st, U, B, dt, emf, fluxes = gen.case_inputs(name)
    n = mesh.n_owned
    sel = golden[f"{name}_blocks"]
    Uu, Bu = orc.update_all(om, fluxes, U[:n], B[:n])
    assert np.array_equal(Uu[sel], golden[f"{name}_upd_U"])
    assert np.array_equal(Bu[sel], golden[f"{name}_upd_B"])


@pytest.mark.skipif(not os.path.isdir(os.environ.get("GMHD_REFERENCE_TREE", "/root/reference")),
                    reason="needs the reference tree")
@pytest.mark.parametrize("name", sorted(gen.CASES))
def test_oracle_coarse_fine_stages_match_reference_live(name):
    if not orc.build_refkat() or not os.path.exists(gen.BRIDGE):
        pytest.skip("functor bridge not built")
    mesh, om, st, U, B, dt, emf, fluxes = gen.case_inputs(name)
    n = mesh.n_owned
    assert np.array_equal(orc.correct_emf(om, emf), gen.reference_correct_emf(mesh, emf))
    Uu, Bu = orc.update_all(om, fluxes, U[:n], B[:n])
    Ur, Br = gen.reference_update(mesh, dt, fluxes, U, B)
    assert np.array_equal(Uu, Ur) and np.array_equal(Bu, Br)


@pytest.mark.parametrize("prolongation", [0, 1])
@pytest.mark.parametrize("name", sorted(gen.CASES))
def test_oracle_ghost_primitives_match_reference(golden, name, prolongation):
    """Ghosted primitive variables (ConvertToPrimitivesVariablesFunctor: same-level and outside copies,
    the sibling average of finer leaves, SIMPLE_COPY / EXTRAPOLATE_LINEAR_MINMOD from coarser ones) of the
    blocks next to a level change or to outside blocks: the oracle's block stage reproduces the
    reference's bit for bit (digests of the arrays; the first two blocks in full)."""
    mesh, om, st, U, B, dt, emf, fluxes = gen.case_inputs(name)
    om2 = gen.oracle_mesh_of(mesh, prolongation)
    pb = golden[f"{name}_prim_blocks"]
    want = golden[f"{name}_prim_sha_{prolongation}"]
    full = golden[f"{name}_prim_q_{prolongation}"]
    assert len(pb) == len(want) > 0
    for k, blk in enumerate(pb):
        q = orc.block_stages(om2, st, U, B, dt, int(blk))["q"]
        if k < len(full):
            assert np.array_equal(q, full[k]), blk
        assert gen.digest(q) == want[k], blk


@pytest.mark.skipif(not os.path.isdir(os.environ.get("GMHD_REFERENCE_TREE", "/root/reference")),
                    reason="needs the reference tree")
@pytest.mark.parametrize("name", sorted(gen.CASES))
def test_oracle_ghost_primitives_match_reference_live(name):
    if not orc.build_refkat() or not os.path.exists(gen.BRIDGE):
        pytest.skip("functor bridge not built")
    mesh, om, st, U, B, dt, emf, fluxes = gen.case_inputs(name)
    for prolongation in (0, 1):
        om2 = gen.oracle_mesh_of(mesh, prolongation)
        for blk in range(mesh.n_owned):
            q = orc.block_stages(om2, st, U, B, dt, blk)["q"]
            assert np.array_equal(q, gen.reference_primitives(mesh, U, B, blk, prolongation, om2)), (blk, prolongation)

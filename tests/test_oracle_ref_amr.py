"""Pin the oracle's coarse/fine stage code against the reference's own functors.

The golden arrays (tests/golden/functor_amr.npz, recorded by tests/golden/make_golden_amr.py) are the
output of the reference's CorrectEmfAtBlockBorderFunctor (border EMF averaging with same-level, finer
and coarser siblings, CorrectEmfAtBlockBorderFunctor.cpp:94-360) and of the coarse/fine branch of
ReadFluxesAndConservativeUpdateFunctor (a coarse cell next to finer leaves takes their face-flux sum
/ 2^d, ReadFluxesAndConservativeUpdateFunctor.cpp:103-436 with .h:233-270), compiled unmodified, on
two-level 2D and 3D meshes (periodic, and with reflecting walls). Their kalypsso-core lookups (edge
siblings, the finer face neighbour, the fine-face sum) come from the bridge's stencil-helper stub,
which states this build's definitions. The inputs (raw EMFs, face fluxes) are the oracle's own; the
oracle's correction and update must reproduce the reference's results bit for bit. Where the
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

"""gmhd_inv_dt_noalloc: the CFL reduction for callers that cannot allocate device memory (code under
CUDA-graph stream capture, frameworks that own every device allocation). It takes no context and
reduces into a fixed array inside the library, so it must give gmhd_inv_dt's result on every call,
including a second call whose answer is smaller than what the array held from the first.

This file is collected last so that a run stopping at the first failure has run everything else."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_mhd_ct_gb300 import _native as nat  # noqa: E402
from godunov_mhd_ct_gb300 import workloads as wl  # noqa: E402
from godunov_mhd_ct_gb300.mesh import BlockMesh  # noqa: E402
from godunov_mhd_ct_gb300.solver import GodunovImplemGB300  # noqa: E402

from .helpers import settings  # noqa: E402

pytestmark = pytest.mark.gpu
TOL = 1e-12  # the FP64 parity tolerance of the other tests; equality is expected


def _params(st, scaling_factor):
    p = nat.GmhdParams(st.gamma0, st.cfl, st.slope_type, st.smallr, st.smallc, scaling_factor, st.riemann_id, 0)
    if st.gravity is not None:
        p.gravity_enabled = 1
        p.gravity = (ctypes.c_double * 3)(*st.gravity)
    if st.viscosity_mu is not None:
        p.viscosity_enabled = 1
        p.viscosity_mu = st.viscosity_mu
    return p


def _noalloc(st, mesh, dU, dB, problem=None, n_problems=1):
    L = nat.lib()
    p = _params(st, mesh.scaling_factor)
    out = torch.full((n_problems,), -1.0, dtype=torch.float64, device="cuda")
    rc = L.gmhd_inv_dt_noalloc(ctypes.byref(p), mesh.dim, mesh.block[0], mesh.block[1], mesh.block[2], mesh.n_owned,
                               int(mesh.level[0]), problem.data_ptr() if problem is not None else None, n_problems,
                               dU.data_ptr(), dB.data_ptr(), out.data_ptr(), None)
    nat.check(rc, "gmhd_inv_dt_noalloc")
    torch.cuda.synchronize()
    return out.cpu().numpy()


SOURCES = {"none": {}, "gravity": {"gravity": (0.3, -1.0, 0.2)}, "viscosity": {"viscosity_mu": 2e-3},
           "both": {"gravity": (0.0, -0.5, 0.0), "viscosity_mu": 1e-3}}


@pytest.mark.parametrize("src", sorted(SOURCES))
@pytest.mark.parametrize("dim,block,level", [(3, (16, 16, 16), 1), (2, (16, 16, 1), 3)])
def test_noalloc_matches_inv_dt_on_two_calls(dim, block, level, src):
    mesh = BlockMesh.uniform(dim, level=level, block=block)
    st = settings()
    for k, v in SOURCES[src].items():
        setattr(st, k, v)
    impl = GodunovImplemGB300(st, mesh)
    Ua, Ba = wl.orszag_tang(mesh, gamma=st.gamma0, rho_perturbation=1e-3, seed=11)
    Ub, Bb = wl.uniform_state(mesh, gamma=st.gamma0, v=(0.01, 0.0, 0.0), b=(0.01, 0.0, 0.0))
    states = [(torch.from_numpy(Ua).cuda(), torch.from_numpy(Ba).cuda()),
              (torch.from_numpy(Ub).cuda(), torch.from_numpy(Bb).cuda())]
    expected = [impl.compute_inv_dt(dU, dB) for dU, dB in states]
    if src == "none":
        assert expected[1] < expected[0]  # the second call must not see the first call's maximum
    for (dU, dB), e in zip(states, expected):
        got = _noalloc(st, mesh, dU, dB)[0]
        assert abs(got - e) <= TOL * abs(e), (got, e)


def test_noalloc_per_problem_and_capacity():
    mesh = BlockMesh.uniform(2, level=2, block=(8, 8, 1))
    st = settings()
    U, B = wl.orszag_tang(mesh, gamma=st.gamma0)
    dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    single = _noalloc(st, mesh, dU, dB)[0]
    prob = torch.from_numpy((np.arange(mesh.n_owned) % 3).astype(np.int32)).cuda()
    per = _noalloc(st, mesh, dU, dB, problem=prob, n_problems=3)
    assert max(per) == single and np.all(per > 0)
    L = nat.lib()
    p = nat.GmhdParams(st.gamma0, st.cfl, st.slope_type, st.smallr, st.smallc, 1.0, 5, 0)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = L.gmhd_inv_dt_noalloc(ctypes.byref(p), 2, 8, 8, 1, mesh.n_owned, 2, prob.data_ptr(), 100000,
                               dU.data_ptr(), dB.data_ptr(), out.data_ptr(), None)
    assert rc == -6  # GMHD_ERR_TOO_LARGE


def test_noalloc_out_of_range_problem_id_gives_nan_then_recovers():
    """A problem id the call was not told about is skipped on the device and turns every output into
    NaN; the next, valid call is not affected. The bad id here equals n_problems, so even an unguarded
    kernel would stay inside the fixed array."""
    mesh = BlockMesh.uniform(2, level=2, block=(8, 8, 1))
    st = settings()
    U, B = wl.orszag_tang(mesh, gamma=st.gamma0)
    dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    ids = (np.arange(mesh.n_owned) % 2).astype(np.int32)
    good = _noalloc(st, mesh, dU, dB, problem=torch.from_numpy(ids).cuda(), n_problems=2)
    ids_bad = ids.copy()
    ids_bad[5] = 2  # == n_problems
    bad = _noalloc(st, mesh, dU, dB, problem=torch.from_numpy(ids_bad).cuda(), n_problems=2)
    assert np.all(np.isnan(bad)), bad
    again = _noalloc(st, mesh, dU, dB, problem=torch.from_numpy(ids).cuda(), n_problems=2)
    assert np.array_equal(again, good)

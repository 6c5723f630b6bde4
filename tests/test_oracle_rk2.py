"""RK2_SSP time integrator ([amr] time_integrator, SolverGodunovMHD.cpp:551-647) on the oracle (CPU):
no Hancock predictor, no half-step face source in the edge states, two stages and U = 1/2 U + 1/2 U2."""
import numpy as np
import pytest

from godunov_mhd_ct_gb300 import workloads as wl
from godunov_mhd_ct_gb300.mesh import BlockMesh

from .test_oracle_amr import amr_mesh, div_b, totals

orc = pytest.importorskip("oracle.oracle")


@pytest.mark.parametrize("dim", [2, 3])
def test_rk2_uniform_state_preserved(dim):
    m = BlockMesh.uniform(dim, level=1, block=(8, 8, 8 if dim == 3 else 1))
    U, B = wl.uniform_state(m)
    st = orc.settings(gamma0=1.4, cfl=0.4, slope_type=2.0, riemann=5, time_integrator=1)
    U2, B2, dts = orc.run(orc.Mesh.from_block_mesh(m), st, U, B, 3)
    np.testing.assert_array_equal(U2[: m.n_owned], U[: m.n_owned])
    np.testing.assert_array_equal(B2[: m.n_owned], B[: m.n_owned])


@pytest.mark.parametrize("dim", [2, 3])
def test_rk2_conservation_div_b_and_difference_from_hancock(dim):
    m = amr_mesh(dim)
    U, B = wl.random_smooth(m, seed=4)
    om = orc.Mesh.from_block_mesh(m)
    rk = orc.settings(gamma0=1.4, cfl=0.4, slope_type=2.0, riemann=5, time_integrator=1)
    hc = orc.settings(gamma0=1.4, cfl=0.4, slope_type=2.0, riemann=5, time_integrator=0)
    U2, B2, _ = orc.run(om, rk, U, B, 6)
    U3, _, _ = orc.run(om, hc, U, B, 6)
    t0, t1 = totals(m, U), totals(m, U2)
    assert abs(t1[0] - t0[0]) <= 1e-13 * abs(t0[0])
    assert abs(t1[1] - t0[1]) <= 1e-13 * abs(t0[1])
    assert div_b(m, B2) < 1e-11
    # same order of accuracy, different scheme: close but not equal
    diff = np.abs(U2[: m.n_owned] - U3[: m.n_owned]).max()
    assert 0.0 < diff < 0.1

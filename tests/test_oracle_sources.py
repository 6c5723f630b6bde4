"""Oracle gravity and viscosity source terms (CPU): the properties the reference's formulas give by
construction.

* uniform gravity on a uniform state at rest: the hydro and CT updates vanish exactly and
  AddGravitySourceTerm (scheme/AddGravitySourceTerm.cpp:47-99) leaves rho u = dt g rho and
  E + (rho u)^2 / (2 rho);
* the gravity CFL (scheme/ComputeDtMHDFunctor.cpp:155-249) and the viscous bound 4 nu / dx^2;
* viscous fluxes (scheme/ComputeViscousFluxesAndStoreFunctor.cpp:168-344) on a shear layer
  u = U0 sin(2 pi y) with B = 0 (no hydro change): the x momentum gets dt mu times the discrete
  Laplacian; mass, momentum and energy totals are conserved; a uniform velocity feels nothing.
"""
import math

import numpy as np
import pytest

from godunov_mhd_ct_gb300 import workloads as wl
from godunov_mhd_ct_gb300.mesh import BlockMesh

orc = pytest.importorskip("oracle.oracle")


def _mesh(dim):
    if dim == 2:
        return BlockMesh.uniform(2, level=1, block=(8, 8, 1))
    return BlockMesh.uniform(3, level=1, block=(4, 4, 4))


@pytest.mark.parametrize("dim", [2, 3])
def test_gravity_kick_on_uniform_state(dim):
    m = _mesh(dim)
    g = (0.3, -0.7, 0.2)
    U, B = wl.uniform_state(m, rho=1.3, p=0.9, v=(0.0, 0.0, 0.0), b=(0.0, 0.0, 0.0))
    st = orc.settings(gamma0=1.4, cfl=0.5, slope_type=2.0, riemann=5, gravity=g[:dim])
    dt = 1.7e-3
    U2, B2 = orc.step(orc.Mesh.from_block_mesh(m), st, U, B, dt)
    n = m.n_owned
    rho = U[:n, 0]
    for c in range(dim):
        want = 0.0 + dt * g[c] * (rho + rho) / 2
        np.testing.assert_array_equal(U2[:n, 2 + c], want)
    ru = [U2[:n, 2 + c] for c in range(dim)]
    ek = 0.5 * (ru[0] * ru[0] + ru[1] * ru[1]) / rho
    if dim == 3:
        ek = ek + 0.5 * (ru[2] * ru[2]) / rho
    np.testing.assert_array_equal(U2[:n, 1], U[:n, 1] + (ek - 0.0))
    np.testing.assert_array_equal(U2[:n, 0], rho)
    np.testing.assert_array_equal(B2[:n], B[:n])


@pytest.mark.parametrize("dim", [2, 3])
def test_gravity_and_viscous_cfl(dim):
    m = _mesh(dim)
    U, B = wl.random_smooth(m, seed=4)
    om = orc.Mesh.from_block_mesh(m)
    base = orc.inv_dt(om, orc.settings(gamma0=1.4, riemann=5), U, B)
    g = (0.5, -2.0, 1.0)[:dim]
    with_g = orc.inv_dt(om, orc.settings(gamma0=1.4, riemann=5, gravity=g), U, B)
    # the correction k / (sqrt(1 + 2k) - 1) is >= 1 and grows with |g|
    assert with_g > base
    stronger = orc.inv_dt(om, orc.settings(gamma0=1.4, riemann=5, gravity=tuple(10 * v for v in g)), U, B)
    assert stronger > with_g
    # a negligible field is floored at k = 1e-4: factor (sqrt(1.0002) - 1)^-1 * 1e-4 ~ 1.00005
    tiny = orc.inv_dt(om, orc.settings(gamma0=1.4, riemann=5, gravity=(1e-30,) * dim), U, B)
    k = 1e-4
    assert tiny == pytest.approx(base * k / (math.sqrt(1 + 2 * k) - 1), rel=1e-12)
    # viscosity: at least 4 mu / (rho dx^2) with the smallest density
    dx = m.cell_length()
    mu = 50.0
    visc = orc.inv_dt(om, orc.settings(gamma0=1.4, riemann=5, viscosity_mu=mu), U, B)
    want = 4 * (mu / U[: m.n_owned, 0]) / (dx * dx)
    assert visc == pytest.approx(max(base, float(want.max())), rel=1e-15)


def _shear(m, u0=0.05):
    """rho = 1, p = 1, B = 0, u = u0 sin(2 pi y)."""
    U, B = m.alloc_state()
    n = m.n_owned
    _, gj, _ = m.global_cell_index()
    y = (gj[:n] + 0.5) * m.cell_length()
    u = u0 * np.sin(2 * math.pi * y)
    U[:n, 0] = 1.0
    U[:n, 2] = u
    U[:n, 1] = 1.0 / (1.4 - 1.0) + 0.5 * u * u
    return U, B


@pytest.mark.parametrize("predictor", [False, True])
def test_viscous_shear_decay(predictor):
    m = BlockMesh.uniform(2, level=2, block=(8, 8, 1))
    U, B = _shear(m)
    mu = 2e-3
    dt = 1e-3
    st = orc.settings(gamma0=1.4, slope_type=2.0, riemann=5, viscosity_mu=mu, viscous_predictor=predictor)
    om = orc.Mesh.from_block_mesh(m)
    U2, B2 = orc.step(om, st, U, B, dt)
    U2h, _ = orc.step(om, orc.settings(gamma0=1.4, slope_type=2.0, riemann=5), U, B, dt)
    n = m.n_owned
    dx = m.cell_length()
    # the inviscid step leaves the shear layer alone (to round-off)
    assert np.abs(U2h[:n, 2] - U[:n, 2]).max() < 1e-15
    # viscous change of rho u: dt mu (u_{j+1} - 2 u_j + u_{j-1}) / dx^2, on the global grid
    gi, gj, _ = m.global_cell_index()
    ny = m.grid[1] * m.block[1]
    ug = np.zeros(ny)
    ug[gj[:n].ravel()] = U[:n, 2].ravel()
    lap = np.roll(ug, -1) - 2 * ug + np.roll(ug, 1)
    want = dt * mu * lap[gj[:n]] / (dx * dx)
    np.testing.assert_allclose(U2[:n, 2] - U[:n, 2], want, rtol=1e-9, atol=1e-17)
    # conservation: mass, momentum and energy totals
    for v in (0, 1, 2, 3):
        assert abs(U2[:n, v].sum() - U[:n, v].sum()) <= 1e-13 * max(1.0, abs(U[:n, v]).sum())
    np.testing.assert_array_equal(U2[:n, 0], U[:n, 0])


@pytest.mark.parametrize("dim", [2, 3])
def test_uniform_velocity_feels_no_viscosity(dim):
    m = _mesh(dim)
    U, B = wl.uniform_state(m)
    st = orc.settings(gamma0=1.4, slope_type=2.0, riemann=5, viscosity_mu=0.3, viscous_predictor=True)
    U2, B2 = orc.step(orc.Mesh.from_block_mesh(m), st, U, B, 1e-3)
    n = m.n_owned
    np.testing.assert_array_equal(U2[:n], U[:n])
    np.testing.assert_array_equal(B2[:n], B[:n])


@pytest.mark.parametrize("dim", [2, 3])
def test_sources_with_rk2_and_amr_conserve_mass(dim):
    from .test_oracle_amr import amr_mesh

    m = amr_mesh(dim)
    U, B = wl.random_smooth(m, seed=9)
    st = orc.settings(gamma0=1.4, cfl=0.4, slope_type=2.0, riemann=5, time_integrator=1, gravity=(0.1, -0.2, 0.05)[:dim],
                      viscosity_mu=1e-3)
    om = orc.Mesh.from_block_mesh(m)
    U2, B2, dts = orc.run(om, st, U, B, 4)
    vol = (m.block_dx() ** m.dim)[: m.n_owned, None, None, None]
    t0 = float((U[: m.n_owned, 0] * vol).sum())
    t1 = float((U2[: m.n_owned, 0] * vol).sum())
    assert np.all(dts > 0)
    assert abs(t1 - t0) <= 1e-13 * abs(t0)

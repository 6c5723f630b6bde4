"""CPU-only checks: the C-ABI library loads and exports what include/gmhd.h declares, host-side
mesh tables, settings parsing and the oracle's scheme invariants. No GPU calls here."""
import ctypes
import os
import re

import numpy as np
import pytest

from godunov_mhd_ct_gb300 import workloads as wl
from godunov_mhd_ct_gb300.mesh import BlockMesh, nb_slot
from godunov_mhd_ct_gb300.settings import MHDSettings

from .helpers import div_b, oracle_mesh, oracle_settings, settings, shared_face_mismatch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def native():
    from godunov_mhd_ct_gb300 import _native as nat
    from godunov_mhd_ct_gb300.csrc import build

    build.build()
    return nat


def test_library_exports_every_declared_symbol(native):
    header = open(os.path.join(ROOT, "include", "gmhd.h")).read()
    declared = set(re.findall(r"\b(gmhd_[a-z_]+)\s*\(", header))
    assert declared == set(native.exported_symbols())
    lib = native.lib()
    for name in declared:
        assert hasattr(lib, name), name
    assert lib.gmhd_error_string(0) == b"ok"


def test_layout_check_host_only(native):
    mesh = BlockMesh.uniform(3, level=1, block=(8, 8, 8))
    t = native.MeshTables(mesh)
    L = native.lib()
    assert L.gmhd_layout_check(ctypes.byref(t.c), mesh.ncell, 5 * mesh.ncell, mesh.nface) == 0
    assert L.gmhd_layout_check(ctypes.byref(t.c), mesh.ncell + 1, 5 * mesh.ncell, mesh.nface) != 0


def test_null_arguments_rejected_without_gpu(native):
    L = native.lib()
    assert not L.gmhd_create(None)
    assert L.gmhd_step(None, None, None, None, None, 0.0, None) == -1
    assert L.gmhd_set_mesh(None, None) == -1


@pytest.mark.parametrize("dim,bricks,level", [(2, (1, 1, 1), 3), (3, (1, 1, 1), 2), (2, (2, 1, 1), 2)])
def test_mesh_neighbour_tables_periodic(dim, bricks, level):
    m = BlockMesh.uniform(dim, bricks=bricks, level=level, block=(8, 8, 8))
    n = m.n_owned
    assert n == np.prod([b * (1 << level) for b in bricks[:dim]])
    # every neighbour relation is symmetric and points to the block at the shifted coordinate
    for ox in (-1, 0, 1):
        for oy in (-1, 0, 1):
            for oz in ((-1, 0, 1) if dim == 3 else (0,)):
                nb = m.neighbor[:n, nb_slot(ox, oy, oz)]
                assert np.all(nb >= 0)
                back = m.neighbor[nb, nb_slot(-ox, -oy, -oz)]
                assert np.array_equal(back, np.arange(n))
                exp = (m.coords[:n] + np.array([ox, oy, oz])) % np.array(m.grid)
                assert np.array_equal(m.coords[nb], exp)


def test_mesh_morton_order():
    m = BlockMesh.uniform(2, level=2, block=(8, 8, 1))
    assert [tuple(c[:2]) for c in m.coords[:4]] == [(0, 0), (1, 0), (0, 1), (1, 1)]


def test_mesh_outside_blocks():
    m = BlockMesh.uniform(3, level=1, block=(4, 4, 4), periodic=(True, False, True))
    n_out = m.n_blocks - m.n_owned
    assert n_out == 2 * 2 * 2  # y = -1 and y = 2 layers of a 2x2 (x, z) grid
    assert np.all(m.outside_normal[:, [0, 2]] == 0)
    assert set(m.outside_normal[:, 1].tolist()) == {1, -1}
    # inside blocks at the y border point to outside blocks, not to -1
    nb = m.neighbor[: m.n_owned, nb_slot(0, -1, 0)]
    assert np.all(nb >= 0)


def test_settings_from_ini_defaults_and_overrides():
    text = """
[hydro]
gamma0=1.666
cfl=0.8
slope_type=2.0
riemann=HLLD
implementation_version=0
[mhd]
small_beta=1e-3
"""
    s = MHDSettings.from_ini(text)
    assert s.gamma0 == 1.666 and s.cfl == 0.8 and s.slope_type == 2.0 and s.riemann_id == 5
    assert s.smallr == 1e-10 and s.smallc == 1e-10 and s.smallp == 1e-10 * 1e-10 / 1.666
    d = MHDSettings.from_ini("[hydro]\nriemann=LLF\n")
    assert d.gamma0 == 1.4 and d.cfl == 0.5 and d.slope_type == 1.0 and d.riemann_id == 2


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_invariants(oracle_lib, dim):
    mesh = BlockMesh.uniform(dim, level=2 if dim == 2 else 1, block=(16, 16, 1) if dim == 2 else (8, 8, 8))
    st = settings()
    om, os_ = oracle_mesh(oracle_lib, mesh), oracle_settings(oracle_lib, st)
    U, B = wl.orszag_tang(mesh, gamma=st.gamma0, rho_perturbation=1e-3, seed=5)
    U1, B1, dts = oracle_lib.run(om, os_, U, B, 10)
    assert np.all(dts > 0)
    n = mesh.n_owned
    for v in (0, 1):  # mass and total energy are conserved on a periodic mesh
        assert abs(U1[:n, v].sum() - U[:n, v].sum()) / abs(U[:n, v].sum()) < 1e-13
    assert np.max(np.abs(div_b(mesh, B1))) < 1e-12
    assert shared_face_mismatch(mesh, B1) == 0.0
    Uu, Bu = wl.uniform_state(mesh)
    Uu1, Bu1, _ = oracle_lib.run(om, os_, Uu, Bu, 3)
    assert np.array_equal(Uu1, Uu) and np.array_equal(Bu1, Bu)


def test_workload_divergence_free_and_reproducible():
    mesh = BlockMesh.uniform(3, level=1, block=(8, 8, 8))
    U, B = wl.orszag_tang(mesh, rho_perturbation=1e-3, seed=42)
    U2, B2 = wl.orszag_tang(mesh, rho_perturbation=1e-3, seed=42)
    assert np.array_equal(U, U2) and np.array_equal(B, B2)
    assert np.max(np.abs(div_b(mesh, B))) < 1e-12
    assert shared_face_mismatch(mesh, B) == 0.0
    rho0 = 25.0 / (36.0 * np.pi)
    r = U[:, 0] / rho0 - 1.0
    assert np.all(np.abs(r) <= 1e-3 + 1e-15) and np.std(r) > 2e-4


@pytest.mark.parametrize("dim,periodic", [(2, (True, True, True)), (3, (True, True, True)), (2, (False, True, True)),
                                          (3, (True, False, True))])
def test_native_forest_matches_uniform_builder(native, dim, periodic):
    """gmhd_forest_build on a uniform leaf set gives the uniform builder's tables (order, neighbours,
    outside blocks)."""
    block = (8, 8, 8 if dim == 3 else 1)
    u = BlockMesh.uniform(dim, level=2, block=block, periodic=periodic)
    t = native.forest_build(dim, u.bricks, u.periodic, u.block, 2, 2, np.array(u.leaf_keys(), np.int32))
    n = u.n_owned
    assert t["n_owned"] == n and len(t["level"]) == u.n_blocks
    np.testing.assert_array_equal(t["coord"][:n], u.coords[:n])
    np.testing.assert_array_equal(t["level"], u.level)
    # owned neighbours by id; outside blocks (numbered differently) by their coordinates, source, normal
    a, b = t["neighbor"][:n], u.neighbor[:n]
    inside = b < n
    np.testing.assert_array_equal(a[inside], b[inside])
    ca = {tuple(t["coord"][x]) + (int(t["outside_src"][x - n]),) + tuple(t["outside_normal"][x - n]) for x in a[~inside]}
    cb = {tuple(u.coords[x]) + (int(u.outside_src[x - n]),) + tuple(u.outside_normal[x - n]) for x in b[~inside]}
    assert ca == cb
    assert t["fine_neighbor"] is None
    np.testing.assert_array_equal(t["remap"][:, 0], 0)


def test_native_forest_adapt_balances(native):
    """Refining one leaf twice forces its neighbours to refine (2:1 across faces, edges, corners)."""
    u = BlockMesh.uniform(2, level=2, block=(8, 8, 1))
    m, _ = u.adapt(np.where(np.arange(u.n_owned) == 5, 1, 0), 2, 4)
    m2, table = m.adapt(np.where(m.level[: m.n_owned] == 3, 1, 0), 2, 4)
    for b in range(m2.n_owned):
        for s in range(27):
            n = m2.neighbor[b, s]
            if n >= 0:
                assert abs(int(m2.level[n]) - int(m2.level[b])) <= 1
    assert set(np.unique(table[:, 0])) <= {0, 1}
    assert np.bincount(m2.level[: m2.n_owned]).tolist()[2:] == [np.count_nonzero(m2.level == 2),
                                                                np.count_nonzero(m2.level == 3), 16]

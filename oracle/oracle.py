"""ctypes front-end of the FP64 CPU oracle (test infrastructure only; see ``oracle/__init__.py``).

Parity is pinned per call against golden vectors recorded from the reference's own model headers
(``tests/golden/``); the stage orchestration follows scheme/GodunovImplemV0.cpp:101-207.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_REF_PATH = os.path.join(_HERE, "_ref", "libref_models.so")
_lib = None


class OracleMesh(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32), ("bx", ctypes.c_int32), ("by", ctypes.c_int32),
        ("bz", ctypes.c_int32), ("n_blocks", ctypes.c_int32), ("n_owned", ctypes.c_int32),
        ("level", ctypes.POINTER(ctypes.c_int32)), ("neighbor", ctypes.POINTER(ctypes.c_int32)),
        ("scaling_factor", ctypes.c_double), ("outside_src", ctypes.POINTER(ctypes.c_int32)),
        ("outside_normal", ctypes.POINTER(ctypes.c_int32)), ("bc", ctypes.c_int32 * 6),
        ("coord", ctypes.POINTER(ctypes.c_int32)), ("fine_neighbor", ctypes.POINTER(ctypes.c_int32)),
        ("prolongation", ctypes.c_int32),
    ]


class OracleSettings(ctypes.Structure):
    _fields_ = [
        ("gamma0", ctypes.c_double), ("cfl", ctypes.c_double), ("slope_type", ctypes.c_double),
        ("smallr", ctypes.c_double), ("smallc", ctypes.c_double), ("riemann", ctypes.c_int32),
        ("time_integrator", ctypes.c_int32), ("gravity_enabled", ctypes.c_int32), ("gravity", ctypes.c_double * 3),
        ("viscosity_enabled", ctypes.c_int32), ("viscosity_mu", ctypes.c_double), ("viscous_predictor", ctypes.c_int32),
    ]


def build() -> None:
    """Compile liboracle.so with the committed Makefile (no-op when up to date)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def build_refkat() -> bool:
    """Compile the reference-header bridge when the reference tree is mounted. Returns success."""
    ref = os.environ.get("GMHD_REFERENCE_TREE", "/root/reference")
    if not os.path.isdir(os.path.join(ref, "models")):
        return False
    subprocess.run(["make", "-s", "-C", os.path.join(_HERE, "refkat"), f"REF={ref}"], check=True)
    return os.path.exists(_REF_PATH)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        L.oracle_step.restype = ctypes.c_int
        L.oracle_step.argtypes = [ctypes.POINTER(OracleMesh), ctypes.POINTER(OracleSettings), dp, dp, dp, dp,
                                  ctypes.c_double]
        L.oracle_inv_dt.restype = ctypes.c_double
        L.oracle_inv_dt.argtypes = [ctypes.POINTER(OracleMesh), ctypes.POINTER(OracleSettings), dp, dp]
        L.oracle_run.restype = ctypes.c_int
        L.oracle_run.argtypes = [ctypes.POINTER(OracleMesh), ctypes.POINTER(OracleSettings), dp, dp, ctypes.c_int,
                                 dp]
        L.oracle_run_to.restype = ctypes.c_int
        L.oracle_run_to.argtypes = [ctypes.POINTER(OracleMesh), ctypes.POINTER(OracleSettings), dp, dp, ctypes.c_int,
                                    dp, dp, ctypes.c_double]
        L.oracle_riemann.argtypes = [ctypes.POINTER(OracleSettings), dp, dp, dp]
        L.oracle_compute_emf.restype = ctypes.c_double
        L.oracle_compute_emf.argtypes = [ctypes.POINTER(OracleSettings), dp, ctypes.c_int]
        L.oracle_compute_primitives.argtypes = [ctypes.POINTER(OracleSettings), dp, dp, dp]
        L.oracle_find_speed_info.argtypes = [ctypes.POINTER(OracleSettings), dp, ctypes.c_int, dp]
        L.oracle_find_speed_fast.restype = ctypes.c_double
        L.oracle_find_speed_fast.argtypes = [ctypes.POINTER(OracleSettings), dp, ctypes.c_int]
        L.oracle_fill_outside.argtypes = [ctypes.POINTER(OracleMesh), dp, dp]
        L.oracle_ct_update.restype = ctypes.c_int
        L.oracle_ct_update.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int, dp, dp]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def settings(gamma0=1.4, cfl=0.5, slope_type=1.0, smallr=1e-10, smallc=1e-10, riemann=5,
             time_integrator=0, gravity=None, viscosity_mu=None, viscous_predictor=False) -> OracleSettings:
    """time_integrator: 0 HANCOCK, 1 RK2_SSP ([amr] time_integrator). gravity: (gx, gy, gz) of a uniform
    field ([gravity] enabled + uniform_g*) or None; viscosity_mu: [viscosity] mu or None (disabled);
    viscous_predictor: the viscous Hancock predictor term."""
    g = (0.0, 0.0, 0.0) if gravity is None else tuple(float(v) for v in gravity) + (0.0,) * (3 - len(gravity))
    return OracleSettings(gamma0, cfl, slope_type, smallr, smallc, riemann, time_integrator,
                          int(gravity is not None), (ctypes.c_double * 3)(*g[:3]), int(viscosity_mu is not None),
                          0.0 if viscosity_mu is None else float(viscosity_mu), int(bool(viscous_predictor)))


class Mesh:
    """Holds the ctypes mesh plus the numpy arrays it points into."""

    def __init__(self, dim, bx, by, bz, level, neighbor, n_owned, scaling_factor=1.0, outside_src=None,
                 outside_normal=None, bc=(1, 1, 1, 1, 1, 1), coord=None, fine_neighbor=None, prolongation=0):
        ip = ctypes.POINTER(ctypes.c_int32)
        self.level = np.ascontiguousarray(level, dtype=np.int32)
        self.neighbor = np.ascontiguousarray(neighbor, dtype=np.int32)
        self.out_src = np.ascontiguousarray(outside_src if outside_src is not None else np.zeros(1), dtype=np.int32)
        self.out_normal = np.ascontiguousarray(outside_normal if outside_normal is not None else np.zeros(3),
                                               dtype=np.int32).reshape(-1)
        self.coord = None if coord is None else np.ascontiguousarray(coord, dtype=np.int32).reshape(-1)
        self.fine = None if fine_neighbor is None else np.ascontiguousarray(fine_neighbor, dtype=np.int32).reshape(-1)
        self.c = OracleMesh(dim, bx, by, bz if dim == 3 else 1, len(self.level), n_owned,
                            self.level.ctypes.data_as(ip), self.neighbor.ctypes.data_as(ip), scaling_factor,
                            self.out_src.ctypes.data_as(ip), self.out_normal.ctypes.data_as(ip),
                            (ctypes.c_int32 * 6)(*[int(b) for b in bc]),
                            self.coord.ctypes.data_as(ip) if self.coord is not None else ctypes.cast(None, ip),
                            self.fine.ctypes.data_as(ip) if self.fine is not None else ctypes.cast(None, ip),
                            int(prolongation))

    @staticmethod
    def from_block_mesh(mesh, bc=None, prolongation=0):
        """Oracle view of a godunov_mhd_ct_gb300 BlockMesh (uniform or AMR)."""
        if bc is None:
            bc = [1 if mesh.periodic[d // 2] else 2 for d in range(6)]
        bx, by, bz = mesh.block
        return Mesh(mesh.dim, bx, by, bz, mesh.level, mesh.neighbor.reshape(-1), mesh.n_owned,
                    scaling_factor=mesh.scaling_factor,
                    outside_src=mesh.outside_src if mesh.outside_src.size else None,
                    outside_normal=mesh.outside_normal if mesh.outside_normal.size else None, bc=bc,
                    coord=mesh.coords, fine_neighbor=mesh.fine_neighbor, prolongation=prolongation)


def step(mesh: Mesh, st: OracleSettings, U, B, dt):
    """One do_time_step from (U, B); returns (U2, B2)."""
    U2 = np.array(U, dtype=np.float64, copy=True, order="C")
    B2 = np.array(B, dtype=np.float64, copy=True, order="C")
    rc = lib().oracle_step(ctypes.byref(mesh.c), ctypes.byref(st), _dp(U), _dp(U2), _dp(B), _dp(B2), dt)
    if rc != 0:
        raise RuntimeError(f"oracle_step failed: {rc}")
    return U2, B2


def fill_outside(mesh: Mesh, U, B):
    """FillOutsideCellFunctor on copies of U, B; returns (U, B)."""
    U = np.array(U, dtype=np.float64, copy=True, order="C")
    B = np.array(B, dtype=np.float64, copy=True, order="C")
    lib().oracle_fill_outside(ctypes.byref(mesh.c), _dp(U), _dp(B))
    return U, B


def inv_dt(mesh: Mesh, st: OracleSettings, U, B) -> float:
    return lib().oracle_inv_dt(ctypes.byref(mesh.c), ctypes.byref(st), _dp(U), _dp(B))


def block_stages(mesh: Mesh, st: OracleSettings, U, B, dt, blk):
    """Stage arrays of one block (oracle_block_stages): ghosted primitives q, slopes, predictor q2,
    edge field e and face source sf, flat, variable-major, x fastest."""
    c = mesh.c
    dim = c.dim
    b = (c.bx, c.by, c.bz if dim == 3 else 1)
    n2 = int(np.prod([v + 4 for v in b[:dim]]))
    n1 = int(np.prod([v + 2 for v in b[:dim]]))
    out = {"q": np.zeros(11 * n2), "slopes": np.zeros(dim * 8 * n1), "q2": np.zeros(8 * n1),
           "e": np.zeros((3 if dim == 3 else 1) * n2), "sf": np.zeros((3 if dim == 3 else 2) * n1)}
    U = np.ascontiguousarray(U, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    rc = lib().oracle_block_stages(ctypes.byref(c), ctypes.byref(st), _dp(U), _dp(B), ctypes.c_double(dt), int(blk),
                                   *(_dp(out[k]) for k in ("q", "slopes", "q2", "e", "sf")))
    if rc != 0:
        raise RuntimeError(f"oracle_block_stages failed: {rc}")
    return out


def block_fluxes_emf(mesh: Mesh, st: OracleSettings, U, B, dt, blk):
    """Face fluxes (per direction [8][faces], concatenated) and raw edge EMFs ([1|3][(b+1)^d]) of one
    block (oracle_block_fluxes_emf), both times dt/dx."""
    c = mesh.c
    dim = c.dim
    b = (c.bx, c.by, c.bz if dim == 3 else 1)
    nf = sum(int(np.prod([b[d] + (d == dr) for d in range(dim)])) for dr in range(dim))
    ne = int(np.prod([v + 1 for v in b[:dim]]))
    fl = np.zeros(8 * nf)
    emf = np.zeros((3 if dim == 3 else 1) * ne)
    U = np.ascontiguousarray(U, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    rc = lib().oracle_block_fluxes_emf(ctypes.byref(c), ctypes.byref(st), _dp(U), _dp(B), ctypes.c_double(dt),
                                       int(blk), _dp(fl), _dp(emf))
    if rc != 0:
        raise RuntimeError(f"oracle_block_fluxes_emf failed: {rc}")
    return fl, emf


def block_viscous_fluxes(mesh: Mesh, st: OracleSettings, U, B, dt, blk):
    """Viscous face fluxes of one block (oracle_block_viscous_fluxes), times dt/dx, per direction
    [8][faces] concatenated."""
    c = mesh.c
    dim = c.dim
    b = (c.bx, c.by, c.bz if dim == 3 else 1)
    nf = sum(int(np.prod([b[d] + (d == dr) for d in range(dim)])) for dr in range(dim))
    fl = np.zeros(8 * nf)
    U = np.ascontiguousarray(U, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    rc = lib().oracle_block_viscous_fluxes(ctypes.byref(c), ctypes.byref(st), _dp(U), _dp(B), ctypes.c_double(dt),
                                           int(blk), _dp(fl))
    if rc != 0:
        raise RuntimeError(f"oracle_block_viscous_fluxes failed: {rc}")
    return fl


def gravity_source(dim, block, gravity, dt, Uold, Unew):
    """AddGravitySourceTerm alone (oracle_gravity_source) on a copy of Unew [n][5][cells]."""
    Unew = np.array(Unew, dtype=np.float64, copy=True, order="C")
    Uold = np.ascontiguousarray(Uold, dtype=np.float64)
    b = (ctypes.c_int * 3)(*(tuple(block) + (1, 1))[:3])
    g = (ctypes.c_double * 3)(*(tuple(float(v) for v in gravity) + (0.0, 0.0, 0.0))[:3])
    rc = lib().oracle_gravity_source(int(dim), b, int(Unew.shape[0]), g, ctypes.c_double(dt), _dp(Uold), _dp(Unew))
    if rc != 0:
        raise RuntimeError(f"oracle_gravity_source failed: {rc}")
    return Unew


def block_update(mesh: Mesh, blk, fluxes, U2blk, B2blk):
    """Conservative update alone (oracle_block_update) of block blk by its face fluxes, on copies of
    the block's U2 [5][cells] and faces B2; returns (U2blk, B2blk)."""
    U2blk = np.array(U2blk, dtype=np.float64, copy=True, order="C")
    B2blk = np.array(B2blk, dtype=np.float64, copy=True, order="C")
    fluxes = np.ascontiguousarray(fluxes, dtype=np.float64)
    rc = lib().oracle_block_update(ctypes.byref(mesh.c), int(blk), _dp(fluxes), _dp(U2blk), _dp(B2blk))
    if rc != 0:
        raise RuntimeError(f"oracle_block_update failed: {rc}")
    return U2blk, B2blk


def ct_update(dim, block, emf, B):
    """The CT update alone (oracle_ct_update) on copies: B [n][faces] += curl of emf
    [n][1|3][(b+1)^d] (already times dt/dx). Returns the updated B."""
    B = np.array(B, dtype=np.float64, copy=True, order="C")
    emf = np.ascontiguousarray(emf, dtype=np.float64)
    n = int(B.shape[0]) if B.ndim > 1 else 1
    b = (ctypes.c_int * 3)(*(tuple(block) + (1, 1))[:3])
    rc = lib().oracle_ct_update(int(dim), b, n, _dp(emf), _dp(B))
    if rc != 0:
        raise RuntimeError(f"oracle_ct_update failed: {rc}")
    return B


def step_fluxes(mesh: Mesh, st: OracleSettings, U, B, dt):
    """One do_time_step from (U, B) that also returns the per-block face fluxes (flux * dt/dx,
    [n_owned][dir][var][face] flattened per block). Returns (U2, B2, fluxes)."""
    U2 = np.array(U, dtype=np.float64, copy=True, order="C")
    B2 = np.array(B, dtype=np.float64, copy=True, order="C")
    c = mesh.c
    dim = c.dim
    b = (c.bx, c.by, c.bz if dim == 3 else 1)
    nf = sum(int(np.prod([b[d] + (d == dr) for d in range(dim)])) for dr in range(dim))
    fl = np.zeros(c.n_owned * 8 * nf)
    L = lib()
    L.oracle_step_fluxes.restype = ctypes.c_int
    L.oracle_step_fluxes.argtypes = [ctypes.POINTER(OracleMesh), ctypes.POINTER(OracleSettings)] + \
        [ctypes.POINTER(ctypes.c_double)] * 4 + [ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
    rc = L.oracle_step_fluxes(ctypes.byref(c), ctypes.byref(st), _dp(np.ascontiguousarray(U, dtype=np.float64)), _dp(U2),
                              _dp(np.ascontiguousarray(B, dtype=np.float64)), _dp(B2), dt, _dp(fl))
    if rc != 0:
        raise RuntimeError(f"oracle_step_fluxes failed: {rc}")
    return U2, B2, fl.reshape(c.n_owned, -1)


def block_ghost_faces(mesh: Mesh, U, B, blk):
    """The ghosted face field of owned block blk (oracle_block_ghost_faces): Bx, By, Bz of a (b+4)^d cell
    box whose first face has index -2 (2D: the cell-centred Bz), x fastest, concatenated."""
    c = mesh.c
    dim = c.dim
    b = (c.bx, c.by, c.bz if dim == 3 else 1)
    g = [v + 4 for v in b[:dim]]
    n = 0
    for comp in range(3):
        n += int(np.prod([g[d] + (1 if d == comp else 0) for d in range(dim)]))
    out = np.zeros(n)
    L = lib()
    L.oracle_block_ghost_faces.restype = ctypes.c_int
    L.oracle_block_ghost_faces.argtypes = [ctypes.POINTER(OracleMesh), ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_double)]
    rc = L.oracle_block_ghost_faces(ctypes.byref(c), _dp(np.ascontiguousarray(U, dtype=np.float64)),
                                    _dp(np.ascontiguousarray(B, dtype=np.float64)), int(blk), _dp(out))
    if rc != 0:
        raise RuntimeError(f"oracle_block_ghost_faces failed: {rc}")
    return out


def correct_emf(mesh: Mesh, emf):
    """The border EMF correction alone (oracle_correct_emf) over the owned blocks: emf [n_owned][1|3][(b+1)^d]
    raw EMFs (as block_fluxes_emf returns them). Returns the corrected copy."""
    emf = np.ascontiguousarray(emf, dtype=np.float64)
    out = np.zeros_like(emf)
    L = lib()
    L.oracle_correct_emf.restype = ctypes.c_int
    L.oracle_correct_emf.argtypes = [ctypes.POINTER(OracleMesh), ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_double)]
    rc = L.oracle_correct_emf(ctypes.byref(mesh.c), _dp(emf), _dp(out))
    if rc != 0:
        raise RuntimeError(f"oracle_correct_emf failed: {rc}")
    return out


def update_all(mesh: Mesh, fluxes, U2, B2):
    """The conservative update alone (oracle_update_all) over the owned blocks, coarse/fine flux sums
    included, on copies of U2 [n_owned][5][cells] and B2 [n_owned][faces]. Returns (U2, B2)."""
    U2 = np.array(U2, dtype=np.float64, copy=True, order="C")
    B2 = np.array(B2, dtype=np.float64, copy=True, order="C")
    fl = np.ascontiguousarray(fluxes, dtype=np.float64)
    L = lib()
    L.oracle_update_all.restype = ctypes.c_int
    L.oracle_update_all.argtypes = [ctypes.POINTER(OracleMesh)] + [ctypes.POINTER(ctypes.c_double)] * 3
    rc = L.oracle_update_all(ctypes.byref(mesh.c), _dp(fl), _dp(U2), _dp(B2))
    if rc != 0:
        raise RuntimeError(f"oracle_update_all failed: {rc}")
    return U2, B2


def run(mesh: Mesh, st: OracleSettings, U, B, nsteps):
    """nsteps of CFL + step, in place on copies; returns (U, B, dts)."""
    U = np.array(U, dtype=np.float64, copy=True, order="C")
    B = np.array(B, dtype=np.float64, copy=True, order="C")
    dts = np.zeros(max(nsteps, 1), dtype=np.float64)
    rc = lib().oracle_run(ctypes.byref(mesh.c), ctypes.byref(st), _dp(U), _dp(B), nsteps, _dp(dts))
    if rc != 0:
        raise RuntimeError(f"oracle_run failed: {rc}")
    return U, B, dts[:nsteps]


def run_to(mesh: Mesh, st: OracleSettings, U, B, nsteps, t0, t_end):
    """nsteps with dt capped so that t does not pass t_end; returns (U, B, dts, t)."""
    U = np.array(U, dtype=np.float64, copy=True, order="C")
    B = np.array(B, dtype=np.float64, copy=True, order="C")
    dts = np.zeros(max(nsteps, 1), dtype=np.float64)
    t = ctypes.c_double(t0)
    rc = lib().oracle_run_to(ctypes.byref(mesh.c), ctypes.byref(st), _dp(U), _dp(B), nsteps, _dp(dts),
                             ctypes.byref(t), t_end)
    if rc != 0:
        raise RuntimeError(f"oracle_run_to failed: {rc}")
    return U, B, dts[:nsteps], t.value


# ---- per-call math (known-answer tests) -------------------------------------------------------
def riemann(st, qL, qR):
    qL = np.ascontiguousarray(qL, dtype=np.float64)
    qR = np.ascontiguousarray(qR, dtype=np.float64)
    out = np.zeros_like(qL)
    for i in range(qL.shape[0]):
        lib().oracle_riemann(ctypes.byref(st), _dp(qL[i]), _dp(qR[i]), _dp(out[i]))
    return out


def compute_emf(st, q, emf_dir):
    q = np.ascontiguousarray(q, dtype=np.float64)
    return np.array([lib().oracle_compute_emf(ctypes.byref(st), _dp(q[i]), emf_dir) for i in range(q.shape[0])])


def compute_primitives(st, u):
    u = np.ascontiguousarray(u, dtype=np.float64)
    q = np.zeros_like(u)
    c = np.zeros(u.shape[0])
    cc = ctypes.c_double()
    for i in range(u.shape[0]):
        lib().oracle_compute_primitives(ctypes.byref(st), _dp(u[i]), _dp(q[i]), ctypes.byref(cc))
        c[i] = cc.value
    return q, c


def find_speed_info(st, q, dim):
    q = np.ascontiguousarray(q, dtype=np.float64)
    out = np.zeros((q.shape[0], 3))
    for i in range(q.shape[0]):
        lib().oracle_find_speed_info(ctypes.byref(st), _dp(q[i]), dim, _dp(out[i]))
    return out


def find_speed_fast(st, q, d):
    q = np.ascontiguousarray(q, dtype=np.float64)
    return np.array([lib().oracle_find_speed_fast(ctypes.byref(st), _dp(q[i]), d) for i in range(q.shape[0])])


REFINE_CRITERIA = {"SIMPLE_GRADIENT": 0, "LOHNER_UNSPLIT": 1}


def refine_flags(mesh: Mesh, st: OracleSettings, U, B, criterion="LOHNER_UNSPLIT", level_min=0, level_max=30,
                 eps_refine=0.16, eps_coarsen=0.02, eps_lohner=0.02, use_rho=True, use_pressure=False):
    """Refinement flags (-1, 0, +1) of the owned blocks."""
    L = lib()
    L.oracle_refine_flags.argtypes = [ctypes.POINTER(OracleMesh), ctypes.POINTER(OracleSettings),
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p]
    pi = np.array([REFINE_CRITERIA[criterion], level_min, level_max, int(use_rho), int(use_pressure)], np.int32)
    pd = np.array([eps_refine, eps_coarsen, eps_lohner], np.float64)
    U = np.ascontiguousarray(U, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    flags = np.zeros(mesh.c.n_owned, np.int8)
    L.oracle_refine_flags(ctypes.byref(mesh.c), ctypes.byref(st), U.ctypes.data, B.ctypes.data, pi.ctypes.data,
                          pd.ctypes.data, flags.ctypes.data)
    return flags


def remap(old: Mesh, new: Mesh, table, U, B, new_shapes):
    """U, B of the new mesh from the old one (table: BlockMesh.adapt's remap)."""
    L = lib()
    L.oracle_remap.restype = ctypes.c_int
    L.oracle_remap.argtypes = [ctypes.POINTER(OracleMesh), ctypes.POINTER(OracleMesh), ctypes.c_void_p,
                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    t = np.ascontiguousarray(table, dtype=np.int32)
    U = np.ascontiguousarray(U, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    Un = np.zeros(new_shapes[0], np.float64)
    Bn = np.zeros(new_shapes[1], np.float64)
    rc = L.oracle_remap(ctypes.byref(old.c), ctypes.byref(new.c), t.ctypes.data, U.ctypes.data, B.ctypes.data,
                        Un.ctypes.data, Bn.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"oracle_remap failed: {rc}")
    return Un, Bn

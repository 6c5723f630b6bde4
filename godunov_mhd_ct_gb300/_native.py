"""ctypes binding of libgmhd.so (include/gmhd.h). There is no fallback: if the library is
missing or does not load, every entry point raises."""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgmhd.so")

GMHD_OK = 0
STATUS = {0: "ok", -1: "invalid argument", -2: "mesh not set or not supported", -3: "CUDA error",
          -4: "output aliases an input", -5: "non-physical state produced", -6: "exceeds a fixed capacity"}

PRECISION = {"fp64": 0, "mixed": 1}
PROLONGATION = {"SIMPLE_COPY": 0, "EXTRAPOLATE_LINEAR_MINMOD": 1}
TIME_INTEGRATOR = {"HANCOCK": 0, "RK2_SSP": 1}
RIEMANN = {"LLF": 2, "HLL": 3, "HLLC": 4, "HLLD": 5}
BC = {"NONE": 0, "PERIODIC": 1, "ZERO_GRADIENT": 2, "WALL": 3}
HEALTH = {1: "missing neighbour", 2: "level jump", 4: "density <= 0", 8: "non-finite value",
          16: "FP64 pressure recovery used"}


class GmhdParams(ctypes.Structure):
    _fields_ = [("gamma0", ctypes.c_double), ("cfl", ctypes.c_double), ("slope_type", ctypes.c_double),
                ("smallr", ctypes.c_double), ("smallc", ctypes.c_double), ("scaling_factor", ctypes.c_double),
                ("riemann", ctypes.c_int32), ("precision", ctypes.c_int32), ("prolongation", ctypes.c_int32),
                ("time_integrator", ctypes.c_int32), ("gravity_enabled", ctypes.c_int32),
                ("gravity", ctypes.c_double * 3), ("viscosity_enabled", ctypes.c_int32),
                ("viscosity_mu", ctypes.c_double), ("viscous_predictor", ctypes.c_int32)]


_ip = ctypes.POINTER(ctypes.c_int32)


class GmhdMesh(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int32), ("bx", ctypes.c_int32), ("by", ctypes.c_int32), ("bz", ctypes.c_int32),
                ("n_blocks", ctypes.c_int32), ("n_owned", ctypes.c_int32), ("level", _ip), ("neighbor", _ip),
                ("problem", _ip), ("n_problems", ctypes.c_int32), ("outside_src", _ip), ("outside_normal", _ip),
                ("bc", ctypes.c_int32 * 6), ("coord", _ip), ("fine_neighbor", _ip), ("n_fine", ctypes.c_int64),
                ("fine_at", ctypes.POINTER(ctypes.c_int64)), ("fine_id", _ip)]


class GmhdRefineParams(ctypes.Structure):
    _fields_ = [("criterion", ctypes.c_int32), ("level_min", ctypes.c_int32), ("level_max", ctypes.c_int32),
                ("use_rho", ctypes.c_int32), ("use_pressure", ctypes.c_int32), ("eps_refine", ctypes.c_double),
                ("eps_coarsen", ctypes.c_double), ("eps_lohner", ctypes.c_double)]


REFINE_CRITERIA = {"SIMPLE_GRADIENT": 0, "LOHNER_UNSPLIT": 1}


class NativeError(RuntimeError):
    pass


_lib = None


def lib():
    """Load libgmhd.so (built by godunov_mhd_ct_gb300.csrc.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise NativeError(f"{LIB_PATH} is missing: build it with python -m godunov_mhd_ct_gb300.csrc.build "
                          "(or __graft_entry__.build()); there is no CPU fallback")
    L = ctypes.CDLL(LIB_PATH)
    vp, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)
    L.gmhd_create.restype = vp
    L.gmhd_create.argtypes = [ctypes.POINTER(GmhdParams)]
    L.gmhd_destroy.argtypes = [vp]
    L.gmhd_set_mesh.argtypes = [vp, ctypes.POINTER(GmhdMesh)]
    L.gmhd_mem_bytes.restype = ctypes.c_uint64
    L.gmhd_mem_bytes.argtypes = [vp]
    L.gmhd_step.argtypes = [vp, vp, vp, vp, vp, ctypes.c_double, vp]
    L.gmhd_inv_dt.argtypes = [vp, vp, vp, dp, vp]
    L.gmhd_fill_outside.argtypes = [vp, vp, vp, vp]
    L.gmhd_advance.argtypes = [vp, vp, vp, vp, vp, ctypes.c_int32, dp, dp, dp, ctypes.c_int32, vp]
    L.gmhd_step_host.argtypes = [vp, vp, vp, vp, vp, ctypes.c_double, vp]
    L.gmhd_step_host_async.argtypes = [vp, vp, vp, vp, vp, ctypes.c_double, vp]
    L.gmhd_autotune.argtypes = [vp, vp, vp, vp, vp, ctypes.c_double, ctypes.POINTER(ctypes.c_int32),
                                ctypes.POINTER(ctypes.c_double), vp]
    L.gmhd_set_tile.argtypes = [vp, ctypes.c_int32]
    L.gmhd_refine_flags.argtypes = [vp, vp, vp, ctypes.POINTER(GmhdRefineParams), vp, vp]
    L.gmhd_remap.argtypes = [ctypes.c_int32] * 6 + [vp] * 5 + [vp]
    L.gmhd_forest_build.restype = vp
    L.gmhd_forest_build.argtypes = [ctypes.c_int32, vp, vp] + [ctypes.c_int32] * 6 + [vp, vp]
    L.gmhd_forest_sizes.argtypes = [vp] + [ctypes.POINTER(ctypes.c_int32)] * 3
    L.gmhd_forest_tables.argtypes = [vp] * 8
    L.gmhd_forest_fine.argtypes = [vp, ctypes.POINTER(ctypes.c_int64), vp, vp]
    L.gmhd_forest_destroy.argtypes = [vp]
    L.gmhd_last_status.argtypes = [vp, ctypes.POINTER(ctypes.c_uint32)]
    L.gmhd_last_cuda_error.argtypes = [vp]
    L.gmhd_error_string.restype = ctypes.c_char_p
    L.gmhd_error_string.argtypes = [ctypes.c_int]
    L.gmhd_layout_check.argtypes = [ctypes.POINTER(GmhdMesh), ctypes.c_int64, ctypes.c_int64, ctypes.c_int64]
    L.gmhd_inv_dt_noalloc.argtypes = [ctypes.POINTER(GmhdParams)] + [ctypes.c_int32] * 6 + [vp, ctypes.c_int32, vp, vp,
                                                                                          vp, vp]
    _lib = L
    return L


def check(rc: int, what: str, ctx=None) -> None:
    if rc != GMHD_OK:
        extra = ""
        if ctx is not None and rc == -3:
            extra = f" (cudaError {lib().gmhd_last_cuda_error(ctx)})"
        raise NativeError(f"{what} failed: {STATUS.get(rc, rc)}{extra}")


def exported_symbols():
    """Names declared in include/gmhd.h, for the ABI tests."""
    return ["gmhd_create", "gmhd_destroy", "gmhd_set_mesh", "gmhd_mem_bytes", "gmhd_step", "gmhd_inv_dt",
            "gmhd_fill_outside", "gmhd_advance", "gmhd_step_host", "gmhd_last_status", "gmhd_last_cuda_error",
            "gmhd_error_string", "gmhd_layout_check", "gmhd_inv_dt_noalloc", "gmhd_step_host_async",
            "gmhd_refine_flags", "gmhd_remap", "gmhd_forest_build", "gmhd_forest_sizes", "gmhd_forest_tables", "gmhd_forest_fine",
            "gmhd_forest_destroy", "gmhd_autotune", "gmhd_set_tile"]


class MeshTables:
    """Keeps the int32 arrays a GmhdMesh points into alive."""

    def __init__(self, mesh, problem=None, n_problems=1, bc=None):
        self.level = np.ascontiguousarray(mesh.level, dtype=np.int32)
        self.neighbor = np.ascontiguousarray(mesh.neighbor, dtype=np.int32).reshape(-1)
        self.problem = None if problem is None else np.ascontiguousarray(problem, dtype=np.int32)
        self.out_src = np.ascontiguousarray(mesh.outside_src, dtype=np.int32)
        self.out_normal = np.ascontiguousarray(mesh.outside_normal, dtype=np.int32).reshape(-1)
        if bc is None:
            bc = [BC["PERIODIC"] if mesh.periodic[d // 2] else BC["ZERO_GRADIENT"] for d in range(6)]
        c = GmhdMesh()
        c.dim = mesh.dim
        c.bx, c.by, c.bz = mesh.block
        c.n_blocks = mesh.n_blocks
        c.n_owned = mesh.n_owned
        c.level = self.level.ctypes.data_as(_ip)
        c.neighbor = self.neighbor.ctypes.data_as(_ip)
        c.problem = self.problem.ctypes.data_as(_ip) if self.problem is not None else ctypes.cast(None, _ip)
        c.n_problems = n_problems
        c.outside_src = self.out_src.ctypes.data_as(_ip) if self.out_src.size else ctypes.cast(None, _ip)
        c.outside_normal = self.out_normal.ctypes.data_as(_ip) if self.out_normal.size else ctypes.cast(None, _ip)
        for i in range(6):
            c.bc[i] = int(bc[i])
        # coarse/fine meshes: block coordinates and the children of refined neighbour regions
        self.coord = np.ascontiguousarray(mesh.coords, dtype=np.int32).reshape(-1)
        c.coord = self.coord.ctypes.data_as(_ip)
        # the children list when the mesh has one (no dense table built), else the dense table
        fl = getattr(mesh, "fine_list", None)
        self.fine = None
        c.fine_neighbor = ctypes.cast(None, _ip)
        c.n_fine = 0
        c.fine_at = ctypes.cast(None, ctypes.POINTER(ctypes.c_int64))
        c.fine_id = ctypes.cast(None, _ip)
        if fl is not None and fl[0].size:
            self.fine_at = np.ascontiguousarray(fl[0], dtype=np.int64)
            self.fine_id = np.ascontiguousarray(fl[1], dtype=np.int32)
            c.n_fine = int(self.fine_at.size)
            c.fine_at = self.fine_at.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
            c.fine_id = self.fine_id.ctypes.data_as(_ip)
        else:
            fine = getattr(mesh, "fine_neighbor", None)
            self.fine = None if fine is None else np.ascontiguousarray(fine, dtype=np.int32).reshape(-1)
            if self.fine is not None:
                c.fine_neighbor = self.fine.ctypes.data_as(_ip)
        self.c = c


def forest_build(dim, bricks, periodic, block, level_min, level_max, keys, flags=None):
    """Native leaf forest (gmhd_forest_build): returns a dict of numpy tables (level, coord, neighbor,
    fine_list = (at, id), the entries of the [n_blocks, 27, 8] children table that are not -1, or None on a
    single-level leaf set, outside_src, outside_normal, remap [n_owned, 15], n_owned)."""
    L = lib()
    keys = np.ascontiguousarray(np.asarray(keys, dtype=np.int32).reshape(-1, 4))
    br = np.ascontiguousarray(np.asarray(bricks, dtype=np.int32)[:3])
    pe = np.ascontiguousarray(np.asarray([int(bool(p)) for p in periodic[:3]], dtype=np.int32))
    fl = None if flags is None else np.ascontiguousarray(np.asarray(flags, dtype=np.int8).reshape(-1))
    h = L.gmhd_forest_build(int(dim), br.ctypes.data, pe.ctypes.data, int(block[0]), int(block[1]), int(block[2]),
                            int(level_min), int(level_max), keys.shape[0], keys.ctypes.data,
                            fl.ctypes.data if fl is not None else None)
    if not h:
        raise ValueError("gmhd_forest_build failed (invalid keys, or an outside block without a same-level inside "
                         "block: keep the level uniform along non-periodic borders)")
    try:
        no, nb, fine = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        check(L.gmhd_forest_sizes(h, ctypes.byref(no), ctypes.byref(nb), ctypes.byref(fine)), "gmhd_forest_sizes")
        no, nb = no.value, nb.value
        t = {"level": np.empty(nb, np.int32), "coord": np.empty((nb, 3), np.int32),
             "neighbor": np.empty((nb, 27), np.int32), "fine_neighbor": None,
             "outside_src": np.empty(nb - no, np.int32), "outside_normal": np.empty((nb - no, 3), np.int32),
             "remap": np.empty((no, 15), np.int32)}
        keys = ("level", "coord", "neighbor", "fine_neighbor", "outside_src", "outside_normal", "remap")
        check(L.gmhd_forest_tables(h, *(t[k].ctypes.data if t[k] is not None and t[k].size else None
                                        for k in keys)), "gmhd_forest_tables")
        t["fine_list"] = None
        if fine.value:
            n = ctypes.c_int64()
            check(L.gmhd_forest_fine(h, ctypes.byref(n), None, None), "gmhd_forest_fine")
            at, ids = np.empty(n.value, np.int64), np.empty(n.value, np.int32)
            check(L.gmhd_forest_fine(h, ctypes.byref(n), at.ctypes.data, ids.ctypes.data), "gmhd_forest_fine")
            t["fine_list"] = (at, ids)
        t["n_owned"] = no
        return t
    finally:
        L.gmhd_forest_destroy(h)

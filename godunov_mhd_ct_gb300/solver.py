"""Host-side mirror of the reference's interface for this path.

``GodunovImplemGB300`` plays the role of a ``GodunovImplemBase`` implementation
(scheme/GodunovImplemBase.h:45-90): ``resize_auxiliary_data``, ``total_mem_size_in_bytes`` and
``do_time_step(U, U2, Bface, Bface2, dt)``. ``compute_inv_dt`` is ComputeDtMHDFunctor::apply
(scheme/ComputeDtMHDFunctor.cpp:44-82) and ``fill_outside`` FillOutsideCellFunctor::apply
(border_conditions/FillOutside.cpp:47-93). All work goes through libgmhd.so (include/gmhd.h);
arrays are CUDA tensors (torch) in the C-ABI layout, or raw device pointers.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as nat
from .mesh import BlockMesh
from .settings import MHDSettings


def _ptr(x) -> int:
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if not x.is_cuda:
            raise ValueError("expected a CUDA tensor")
        if not x.is_contiguous():
            raise ValueError("expected a contiguous tensor")
        return x.data_ptr()
    raise TypeError(f"unsupported array type {type(x)}")


def _stream_ptr(stream) -> int | None:
    if stream is None:
        try:
            import torch

            return torch.cuda.current_stream().cuda_stream
        except Exception:  # noqa: BLE001
            return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class GodunovImplemGB300:
    """GB300 implementation of the MUSCL-Hancock + CT stage (create_godunov_implem's product)."""

    def __init__(self, settings: MHDSettings, mesh: BlockMesh, precision: str = "fp64", problem=None,
                 n_problems: int = 1, bc=None):
        if settings.riemann_id not in (2, 3, 4, 5):
            raise ValueError(f"unknown Riemann solver {settings.riemann!r} (the reference aborts here)")
        if settings.implementation_version != 0:
            # SolverGodunovMHD.cpp:91-97 accepts only version 0; this path implements it
            raise ValueError("only implementation_version=0 exists in the reference")
        self.settings = settings
        self.precision = precision
        prol = settings.prolongation.upper()
        if prol not in nat.PROLONGATION:
            raise ValueError(f"unsupported [amr] cell_centered_prolongation_type {settings.prolongation!r}")
        integ = settings.time_integrator.upper()
        if integ not in nat.TIME_INTEGRATOR:
            # RK3_SSP aborts in the reference (SolverGodunovMHD.cpp:174-177)
            raise ValueError(f"unsupported [amr] time_integrator {settings.time_integrator!r}")
        p = nat.GmhdParams(settings.gamma0, settings.cfl, settings.slope_type, settings.smallr, settings.smallc,
                           settings.scaling_factor if mesh is None else mesh.scaling_factor,
                           settings.riemann_id, nat.PRECISION[precision], nat.PROLONGATION[prol],
                           nat.TIME_INTEGRATOR[integ])
        if settings.gravity is not None:
            g = tuple(float(v) for v in settings.gravity) + (0.0,) * (3 - len(settings.gravity))
            p.gravity_enabled = 1
            p.gravity = (ctypes.c_double * 3)(*g[:3])
        if settings.viscosity_mu is not None:
            p.viscosity_enabled = 1
            p.viscosity_mu = float(settings.viscosity_mu)
            p.viscous_predictor = int(bool(settings.viscous_predictor))
        self._lib = nat.lib()
        self._ctx = self._lib.gmhd_create(ctypes.byref(p))
        if not self._ctx:
            raise nat.NativeError("gmhd_create failed (bad settings or no CUDA device)")
        self.mesh = None
        self._tables = None
        self.resize_auxiliary_data(mesh, problem=problem, n_problems=n_problems, bc=bc)

    # --- GodunovImplemBase -----------------------------------------------------------------------
    def resize_auxiliary_data(self, mesh: BlockMesh | None = None, problem=None, n_problems: int = 1, bc=None):
        if mesh is not None:
            self.mesh = mesh
            self._tables = nat.MeshTables(mesh, problem=problem, n_problems=n_problems, bc=bc)
            self.n_problems = n_problems
            self._bc = bc
        nat.check(self._lib.gmhd_set_mesh(self._ctx, ctypes.byref(self._tables.c)), "gmhd_set_mesh", self._ctx)

    def total_mem_size_in_bytes(self) -> int:
        return int(self._lib.gmhd_mem_bytes(self._ctx))

    def do_time_step(self, U, U2, Bface, Bface2, dt: float, stream=None) -> None:
        nat.check(self._lib.gmhd_step(self._ctx, _ptr(U), _ptr(U2), _ptr(Bface), _ptr(Bface2), float(dt),
                                      _stream_ptr(stream)), "gmhd_step", self._ctx)

    def autotune(self, U, U2, B, B2, dt: float, stream=None):
        """Pick the fastest shared-memory tile for this mesh's block size (gmhd_autotune): U2, B2 are
        scratch. Returns (tile x extent, ms per step)."""
        tile = ctypes.c_int32(0)
        ms = ctypes.c_double(0.0)
        nat.check(self._lib.gmhd_autotune(self._ctx, _ptr(U), _ptr(U2), _ptr(B), _ptr(B2), float(dt), ctypes.byref(tile),
                                          ctypes.byref(ms), _stream_ptr(stream)), "gmhd_autotune", self._ctx)
        return int(tile.value), float(ms.value)

    def set_tile(self, tile: int) -> None:
        """Tile request by hand (gmhd_set_tile): an x extent the step has for this block size, or 0."""
        nat.check(self._lib.gmhd_set_tile(self._ctx, int(tile)), "gmhd_set_tile", self._ctx)

    # --- solver-side device calls of the path ------------------------------------------------------
    def compute_inv_dt(self, U, Bface, stream=None):
        out = np.zeros(self.n_problems, dtype=np.float64)
        nat.check(self._lib.gmhd_inv_dt(self._ctx, _ptr(U), _ptr(Bface), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                        _stream_ptr(stream)), "gmhd_inv_dt", self._ctx)
        return out if self.n_problems > 1 else float(out[0])

    def compute_dt(self, U, Bface, stream=None):
        """dt = cfl / invDt (SolverGodunovMHD.cpp:375-403)."""
        return self.settings.cfl / self.compute_inv_dt(U, Bface, stream)

    def fill_outside(self, U, Bface, stream=None) -> None:
        nat.check(self._lib.gmhd_fill_outside(self._ctx, _ptr(U), _ptr(Bface), _stream_ptr(stream)),
                  "gmhd_fill_outside", self._ctx)

    def advance(self, U, U2, B, B2, nsteps: int, t=None, t_end=None, use_graph: bool = True, stream=None):
        """nsteps solver iterations on device; U/B hold the result. Returns (dt_log, t)."""
        npb = self.n_problems
        dtlog = np.zeros(max(nsteps, 1) * npb, dtype=np.float64)
        tt = np.zeros(npb) if t is None else np.ascontiguousarray(np.broadcast_to(t, (npb,)), dtype=np.float64).copy()
        te = None if t_end is None else np.ascontiguousarray(np.broadcast_to(t_end, (npb,)), dtype=np.float64)
        dp = ctypes.POINTER(ctypes.c_double)
        rc = self._lib.gmhd_advance(self._ctx, _ptr(U), _ptr(U2), _ptr(B), _ptr(B2), int(nsteps), tt.ctypes.data_as(dp),
                                    te.ctypes.data_as(dp) if te is not None else None, dtlog.ctypes.data_as(dp),
                                    int(bool(use_graph)), _stream_ptr(stream))
        nat.check(rc, "gmhd_advance", self._ctx)
        return dtlog[: nsteps * npb].reshape(nsteps, npb), tt

    def step_host(self, U: np.ndarray, B: np.ndarray, dt: float, U2: np.ndarray | None = None,
                  B2: np.ndarray | None = None):
        """do_time_step on host arrays (copies in and out inside the call)."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        B = np.ascontiguousarray(B, dtype=np.float64)
        U2 = U.copy() if U2 is None else U2
        B2 = B.copy() if B2 is None else B2
        nat.check(self._lib.gmhd_step_host(self._ctx, U.ctypes.data, U2.ctypes.data, B.ctypes.data, B2.ctypes.data,
                                           float(dt), None), "gmhd_step_host", self._ctx)
        return U2, B2

    # --- AMR cycle (SolverGodunovMHD::do_amr_cycle, SolverGodunovMHD.cpp:263-319) -------------------
    def refine_flags(self, U, B, criterion="LOHNER_UNSPLIT", level_min=0, level_max=30, eps_refine=0.16,
                     eps_coarsen=0.02, eps_lohner=0.02, variables=("rho",), stream=None):
        """Flags (-1 coarsen, 0 keep, +1 refine) of the owned blocks (compute_refine_flags)."""
        vs = {v.lower() for v in variables}
        p = nat.GmhdRefineParams(nat.REFINE_CRITERIA[criterion.upper()], level_min, level_max, int("rho" in vs),
                                 int("pressure" in vs), eps_refine, eps_coarsen, eps_lohner)
        flags = np.zeros(self.mesh.n_owned, dtype=np.int8)
        nat.check(self._lib.gmhd_refine_flags(self._ctx, _ptr(U), _ptr(B), ctypes.byref(p), flags.ctypes.data,
                                              _stream_ptr(stream)), "gmhd_refine_flags", self._ctx)
        return flags

    def regrid(self, U, B, level_min: int, level_max: int, stream=None, flags=None, **criterion):
        """One AMR cycle: refinement flags on the device, mesh adaptation + 2:1 balance on the host
        (BlockMesh.adapt, p4est's part), remap of U and B on the device, new mesh tables
        (resize_auxiliary_data). ``flags`` (one per owned block) replaces the flags of the criterion,
        e.g. to repeat another run's mesh sequence. Returns (new mesh, new U, new B); U, B stay valid
        until released. The flags used are kept in ``last_flags``."""
        import time

        import torch

        if self.n_problems != 1:
            raise ValueError("regrid works on single-problem meshes")
        t0 = time.perf_counter()
        if flags is None:
            flags = self.refine_flags(U, B, level_min=level_min, level_max=level_max, stream=stream, **criterion)
        else:
            flags = np.ascontiguousarray(flags, dtype=np.int8).reshape(-1)
            if flags.shape[0] != self.mesh.n_owned:
                raise ValueError("flags need one entry per owned block")
        self.last_flags = flags
        t1 = time.perf_counter()
        new_mesh, table = self.mesh.adapt(flags, level_min, level_max)
        t2 = time.perf_counter()
        us, bs = new_mesh.state_shapes()
        Un = torch.zeros(us, dtype=torch.float64, device=U.device)
        Bn = torch.zeros(bs, dtype=torch.float64, device=U.device)
        table = np.ascontiguousarray(table, dtype=np.int32)
        bx, by, bz = self.mesh.block
        nat.check(self._lib.gmhd_remap(self.mesh.dim, bx, by, bz, self.mesh.n_blocks, new_mesh.n_owned,
                                       table.ctypes.data, _ptr(U), _ptr(B), _ptr(Un), _ptr(Bn), _stream_ptr(stream)),
                  "gmhd_remap")
        t3 = time.perf_counter()
        self.resize_auxiliary_data(new_mesh, bc=self._bc)
        t4 = time.perf_counter()
        # host wall time per part of the cycle, accumulated: flags (incl. their device->host copy),
        # adapt + balance + tables, remap enqueue, new mesh tables (waits for the remap)
        self.regrid_seconds = [a + b for a, b in zip(getattr(self, "regrid_seconds", [0.0] * 4),
                                                     (t1 - t0, t2 - t1, t3 - t2, t4 - t3))]
        return new_mesh, Un, Bn

    def last_status(self) -> int:
        flags = ctypes.c_uint32(0)
        nat.check(self._lib.gmhd_last_status(self._ctx, ctypes.byref(flags)), "gmhd_last_status", self._ctx)
        return int(flags.value)

    def close(self) -> None:
        if getattr(self, "_ctx", None):
            self._lib.gmhd_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

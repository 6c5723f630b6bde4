"""Benchmark: cell-updates/s of the MUSCL-Hancock + CT stage on 3D Orszag-Tang 256^3
(512 leaf blocks of 32^3, periodic), mixed FP32/FP64 path vs the FP64 drop-in, with the HBM
roofline of the fused step kernel, an end-to-end host-buffer number and the CPU baseline; then one
leg per other benchmark configuration (2D Orszag-Tang 128^2, the 2D AMR blast with regrids, 1024
field loops, 3D Kelvin-Helmholtz shear layers on AMR) under "configs".

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gmhd|reference] [--legs 0,2,3,4]

A step is one solver iteration (CFL reduction + do_time_step) over the whole 256^3 mesh. Inputs
(U, B: 2.2 GB in FP64) are far larger than L2 (129 MB), so no L2 flush is needed between steps.
Under torchrun each rank runs an independent replica of the workload (replicas only): the timed
duration is the max over ranks and the value the cell-updates of all ranks over it. Prints one JSON
line on rank 0.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "cell-updates/s on 1 GB300, mixed vs FP64 at L1(rho)<=1e-6; % of HBM roofline"
UNIT = "cell-updates/s"
BYTES_PER_CELL_UPDATE = 128.0  # read U(5)+B(3), write U2(5)+B2(3), FP64
FALLBACK_HBM_GBS = 6800.0
# ncu counters of one mixed fused-step launch on a small case (key value lines: cells, dram bytes,
# warp instructions); per-cell figures scale to the full launch by the cell count
COUNTERS = os.path.join("profiles", "fused_step_mixed_ot3d_counters.txt")


def read_counters(path=COUNTERS):
    """Per-cell DRAM bytes and warp instructions of the dominant kernel from a committed ncu capture,
    or None when the file is absent."""
    try:
        vals = {}
        with open(os.path.join(ROOT, path)) as f:
            for line in f:
                line = line.split("#", 1)[0].split()
                if len(line) == 2:
                    vals[line[0]] = float(line[1])
        cells = vals["cells"]
        return {"dram_bytes_per_cell": (vals["dram_read_bytes"] + vals["dram_write_bytes"]) / cells,
                "warp_inst_per_cell": vals["warp_instructions"] / cells, "source": path}
    except (OSError, KeyError, ValueError):
        return None


def hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:  # noqa: BLE001
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms while running. start() returns once
    the first sample has arrived and drops it, so that the kept samples fall inside the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active," \
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:  # noqa: BLE001
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        t0 = time.perf_counter()
        while not self.rows and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            time.sleep(0.01)
        self.rows.clear()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:  # noqa: BLE001
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                for n, v in zip(names, r[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(ms, dist, device):
    """The timed duration of the slowest rank, on every rank (ms itself without a process group)."""
    if dist is None:
        return ms
    import torch

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(cells_per_rank, steps, world, ms):
    """Cell-updates per second of all ranks together over the max-over-ranks duration ms."""
    return world * cells_per_rank * steps / (ms * 1e-3)


def make_workload(side_blocks=8, block=32, seed=12345):
    from godunov_mhd_ct_gb300 import workloads as wl
    from godunov_mhd_ct_gb300.mesh import BlockMesh

    level = int(np.log2(side_blocks))
    mesh = BlockMesh.uniform(3, level=level, block=(block, block, block))
    U, B = wl.orszag_tang(mesh, gamma=5.0 / 3.0, rho_perturbation=1e-3, seed=seed)
    return mesh, U, B


def settings():
    from godunov_mhd_ct_gb300.settings import MHDSettings

    return MHDSettings(gamma0=5.0 / 3.0, cfl=0.5, slope_type=2.0, riemann="HLLD")


def cpu_baseline_run(steps, warmup, seconds_cap=25.0, side_blocks=8):
    """Time the FP64 oracle (the CPU restatement of the reference stage, OpenMP over blocks) on all host
    cores on the same Orszag-Tang workload (256^3: 512 blocks of 32^3 by default): warm-up iterations,
    then solver iterations (CFL + step) in one call, as many as fit in seconds_cap (at least one)."""
    from oracle import oracle as orc

    orc.build()
    mesh, U, B = make_workload(side_blocks=side_blocks, block=32)
    st = settings()
    om = orc.Mesh(3, 32, 32, 32, mesh.level, mesh.neighbor, mesh.n_owned)
    os_ = orc.settings(gamma0=st.gamma0, cfl=st.cfl, slope_type=st.slope_type, riemann=st.riemann_id)
    # warm-up iterations, the last of them timed to size the sample
    if warmup > 1:
        U, B, _ = orc.run(om, os_, U, B, warmup - 1)
    t0 = time.perf_counter()
    U, B, _ = orc.run(om, os_, U, B, 1)
    one = time.perf_counter() - t0
    done = max(1, min(steps, int(seconds_cap / max(one, 1e-6))))
    t0 = time.perf_counter()
    orc.run(om, os_, U, B, done)
    el = time.perf_counter() - t0
    cells = mesh.n_owned * mesh.ncell
    side = side_blocks * 32
    return {"value": cells * done / el, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": f"3D Orszag-Tang {side}^3 ({mesh.n_owned} blocks of 32^3), {done} oracle solver iterations "
                      f"in one call after {max(warmup, 1)} warm-up, FP64, OpenMP over blocks",
            "ms_per_step": 1e3 * el / done, "steps": done, "workload": f"3d_orszag_tang_{side}^3"}


# ---- the other benchmark configurations (one leg each, after the headline) -----------------------
def _accuracy(mesh0, U0, mesh, U, B, Uref, Bref):
    """L1 relative error of rho, E and face B against (Uref, Bref), max|div B| (per block cell size) and
    the drift of the rho and E volume integrals from (mesh0, U0)."""
    n = mesh.n_owned

    def l1(a, b):
        return float(np.abs(a - b).sum() / np.abs(b).sum())

    def totals(m, X):
        k = m.n_owned
        vol = m.block_dx()[:k] ** m.dim
        return (X[:k, 0].reshape(k, -1).sum(axis=1) * vol).sum(), (X[:k, 1].reshape(k, -1).sum(axis=1) * vol).sum()

    Bx, By, Bz = mesh.split_faces(B)
    d = (Bx[:n, ..., 1:] - Bx[:n, ..., :-1]) + (By[:n, :, 1:, :] - By[:n, :, :-1, :])
    if mesh.dim == 3:
        d = d + (Bz[:n, 1:] - Bz[:n, :-1])
    d = d / mesh.block_dx()[:n, None, None, None]
    m0, e0 = totals(mesh0, U0)
    m1, e1 = totals(mesh, U)
    return {"l1_rho": l1(U[:n, 0], Uref[:n, 0]), "l1_E": l1(U[:n, 1], Uref[:n, 1]), "l1_B": l1(B[:n], Bref[:n]),
            "max_divB": float(np.max(np.abs(d))), "mass_drift": float(abs(m1 - m0) / abs(m0)),
            "energy_drift": float(abs(e1 - e0) / abs(e0))}


def _run(st, mesh, U, B, nsteps, precision, bc=None, t_end=None, problem=None, n_problems=1, tile=None):
    """nsteps graph-replayed solver iterations on the GPU; returns (U, B, dt_log, ms per step)."""
    import torch

    from godunov_mhd_ct_gb300.solver import GodunovImplemGB300

    impl = GodunovImplemGB300(st, mesh, precision=precision, bc=bc, problem=problem, n_problems=n_problems)
    if tile:
        impl.set_tile(tile)
    dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    dU2, dB2 = torch.empty_like(dU), torch.empty_like(dB)
    t0 = None if t_end is None else 0.0
    impl.advance(dU.clone(), dU2, dB.clone(), dB2, 2, t=t0, t_end=t_end)  # warm-up and graph capture
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    dtlog, _ = impl.advance(dU, dU2, dB, dB2, nsteps, t=t0, t_end=t_end)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / nsteps
    out = dU.cpu().numpy(), dB.cpu().numpy(), dtlog, ms
    impl.close()
    del dU, dB, dU2, dB2
    torch.cuda.empty_cache()
    return out


def leg_config0(steps=200):
    """2D Orszag-Tang 128^2 (64 blocks of 16^2), 200 steps: mixed and FP64 on the GPU (accuracy of the
    mixed path against the FP64 one) and, as this configuration's CPU baseline, the FP64 oracle on all
    host cores."""
    from godunov_mhd_ct_gb300 import workloads as wl
    from godunov_mhd_ct_gb300.mesh import BlockMesh
    from oracle import oracle as orc

    mesh = BlockMesh.uniform(2, level=3, block=(16, 16, 1))
    st = settings()
    U, B = wl.orszag_tang(mesh, gamma=st.gamma0)
    cells = mesh.n_owned * mesh.ncell
    Um, Bm, _, ms_m = _run(st, mesh, U, B, steps, "mixed")
    Uf, Bf, _, ms_f = _run(st, mesh, U, B, steps, "fp64")
    # CPU baseline of this configuration
    orc.build()
    om = orc.Mesh(2, 16, 16, 1, mesh.level, mesh.neighbor, mesh.n_owned)
    os_ = orc.settings(gamma0=st.gamma0, cfl=st.cfl, slope_type=st.slope_type, riemann=st.riemann_id)
    t0 = time.perf_counter()
    orc.run(om, os_, U, B, steps)
    cpu_s = (time.perf_counter() - t0) / steps
    return {"workload": f"2d_orszag_tang_128^2 (64 blocks of 16^2), {steps} steps", "cells": cells,
            "value": cells / (ms_m * 1e-3), "ms_per_step": ms_m, "fp64_value": cells / (ms_f * 1e-3),
            "cpu_baseline": {"value": cells / cpu_s, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                             "sample": f"the whole configuration, {steps} oracle solver iterations in one call"},
            "accuracy": dict(_accuracy(mesh, U, mesh, Um, Bm, Uf, Bf), against="FP64 GPU path")}


def leg_config1(side_blocks=4, steps=10, precision="mixed", tile=None):
    """3D Orszag-Tang on (32 side_blocks)^3 cells (blocks of 32^3) at one precision and tile: the
    headline workload's solver loop alone, at a size chosen for profiling single launches."""
    mesh, U, B = make_workload(side_blocks=side_blocks)
    cells = mesh.n_owned * mesh.ncell
    _, _, _, ms = _run(settings(), mesh, U, B, steps, precision, tile=tile)
    return {"workload": f"3d_orszag_tang_{32 * side_blocks}^3 ({mesh.n_owned} blocks of 32^3), {precision}, "
                        f"tile {tile or 'default'}, {steps} steps", "cells": cells, "value": cells / (ms * 1e-3),
            "ms_per_step": ms}


def leg_config2(levels=(5, 10), steps=500, every=10):
    """2D MHD blast, levels 5-10 of 16^2 blocks, an AMR cycle every 10 steps (SIMPLE_GRADIENT > 0.1 on rho
    and p), 500 steps: the mixed solver loop with its regrids timed; accuracy against the FP64 GPU path
    over the same mesh sequence (the FP64 path equals the oracle bit for bit in the tests)."""
    import torch

    from godunov_mhd_ct_gb300 import workloads as wl
    from godunov_mhd_ct_gb300.mesh import BlockMesh
    from godunov_mhd_ct_gb300.solver import GodunovImplemGB300

    lmin, lmax = levels
    cycles = max(1, steps // every)
    crit = dict(criterion="SIMPLE_GRADIENT", eps_refine=0.1, eps_coarsen=0.02, eps_lohner=0.02)
    st = settings()
    mesh = BlockMesh.uniform(2, level=lmin, block=(16, 16, 1))
    U, B = wl.blast(mesh, gamma=st.gamma0)
    for _ in range(lmax - lmin):  # init-time refinement on the analytic state
        impl = GodunovImplemGB300(st, mesh, precision="fp64")
        fl = impl.refine_flags(torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda(), level_min=lmin,
                               level_max=lmax, variables=("rho", "pressure"), **crit)
        impl.close()
        mesh, _ = mesh.adapt(fl, lmin, lmax)
        U, B = wl.blast(mesh, gamma=st.gamma0)
    mesh0, U0, B0 = mesh, U, B

    def loop(precision, flags=None):
        impl = GodunovImplemGB300(st, mesh0, precision=precision)
        dU, dB = torch.from_numpy(U0).cuda(), torch.from_numpy(B0).cuda()
        log, updates = [], 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m = mesh0
        for c in range(cycles):
            impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), every)
            updates += every * m.n_owned * m.ncell
            if c < cycles - 1:
                m, dU, dB = impl.regrid(dU, dB, lmin, lmax, flags=None if flags is None else flags[c],
                                        variables=("rho", "pressure"), **crit)
                log.append(impl.last_flags)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        out = m, dU.cpu().numpy(), dB.cpu().numpy(), updates / el, el, impl.regrid_seconds
        impl.close()
        return out, log

    (mf, Uf, Bf, rate_f, _, _), flags = loop("fp64")
    (mm, Um, Bm, rate_m, el_m, rs), _ = loop("mixed", flags)
    return {"workload": f"2d_blast_amr levels {lmin}-{lmax} (16^2 blocks), regrid every {every} steps, "
                        f"{cycles * every} steps",
            "leaves_initial": mesh0.n_owned, "leaves_final": mm.n_owned, "value": rate_m,
            "ms_per_step": 1e3 * el_m / (cycles * every), "regrid_share": float(sum(rs) / el_m),
            "regrid_ms_per_cycle": {k: 1e3 * v / max(1, cycles - 1) for k, v in
                                    zip(("flags", "adapt_and_tables", "remap", "set_mesh"), rs)},
            "fp64_value": rate_f, "accuracy": dict(_accuracy(mesh0, U0, mm, Um, Bm, Uf, Bf),
                                                   against="FP64 GPU path, same mesh sequence")}


def _run_to_end(st, mesh, U, B, cells, t_end, problem, chunk=200):
    """The mixed batch from t = 0 until every problem reaches t_end, in calls of `chunk` graph-replayed
    iterations; returns (cell-updates of the active problems, seconds, launches)."""
    import torch

    from godunov_mhd_ct_gb300.solver import GodunovImplemGB300

    impl = GodunovImplemGB300(st, mesh, precision="mixed", problem=problem, n_problems=len(cells))
    dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    dU2, dB2 = torch.empty_like(dU), torch.empty_like(dB)
    t = np.zeros(len(cells))
    updates, launches = 0.0, 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    while (t < t_end).any():
        dtlog, t = impl.advance(dU, dU2, dB, dB2, chunk, t=t, t_end=t_end)
        updates += float(((dtlog > 0) * cells[None, :]).sum())
        launches += chunk
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    impl.close()
    return updates, el, launches


def leg_config3(steps=200, acc_steps=5, problems=1024, to_end=False):
    """1024 independent 2D field loops ((2N) x N cells, N = 32..512 log-uniform in cell count; 110 M
    cells) in one launch per step with per-problem dt and end time t = 0.5: `steps` graph-replayed
    iterations timed (the whole run to t = 0.5 is about 2e11 cell-updates; with to_end it is run and
    timed too); accuracy of the mixed path against the FP64 GPU path after acc_steps."""
    from godunov_mhd_ct_gb300 import workloads as wl
    from godunov_mhd_ct_gb300.mesh import BlockMesh

    st = settings()
    meshes, states, _ = wl.field_loop_batch(problems, seed=12345, sizes=(32, 64, 128, 256, 512))
    mesh, problem = BlockMesh.batch(meshes)
    U = np.concatenate([s_[0] for s_ in states])
    B = np.concatenate([s_[1] for s_ in states])
    del states
    cells = np.array([m.n_owned * m.ncell for m in meshes], dtype=np.float64)
    kw = dict(t_end=np.full(len(meshes), 0.5), problem=problem, n_problems=len(meshes))
    _, _, dtlog, ms = _run(st, mesh, U, B, steps, "mixed", **kw)
    updates = float(((dtlog > 0) * cells[None, :]).sum())
    Um, Bm, _, _ = _run(st, mesh, U, B, acc_steps, "mixed", **kw)
    Uf, Bf, _, ms_f = _run(st, mesh, U, B, acc_steps, "fp64", **kw)
    out = {"workload": f"{problems} field loops ({cells.sum() / 1e6:.0f} M cells, 16^2 blocks), {steps} steps of "
                       "the batch",
           "cells": int(cells.sum()), "value": updates / (steps * ms * 1e-3), "ms_per_step": ms,
           "fp64_value": float(cells.sum()) / (ms_f * 1e-3),
           "accuracy": dict(_accuracy(mesh, U, mesh, Um, Bm, Uf, Bf), steps=acc_steps, against="FP64 GPU path")}
    if to_end:
        upd, el, launches = _run_to_end(st, mesh, U, B, cells, kw["t_end"], problem)
        out["to_end"] = {"value": upd / el, "seconds": el, "cell_updates": upd, "launches": launches,
                         "path": "the whole run to t = 0.5, wall time of chunks of 200 graph-replayed steps"}
    return out


def leg_config4(levels=(4, 6), steps=100, acc_steps=2):
    """3D magnetised shear layers (Kelvin-Helmholtz), periodic in x and z, reflecting walls in y, levels
    4-6 of 16^3 blocks (1.64e8 cells), `steps` steps timed; accuracy of the mixed path against the FP64
    GPU path after acc_steps (FP64 runs at about 4 s per step here)."""
    from godunov_mhd_ct_gb300 import workloads as wl
    from godunov_mhd_ct_gb300.settings import MHDSettings

    st = MHDSettings(gamma0=1.4, cfl=0.5, slope_type=2.0, riemann="HLLD")
    mesh = wl.kh_amr_mesh(levels[0], levels[1], block=16)
    U, B = wl.kelvin_helmholtz(mesh, gamma=st.gamma0, seed=12345)
    bc = (1, 1, 3, 3, 1, 1)
    cells = mesh.n_owned * mesh.ncell
    _, _, _, ms = _run(st, mesh, U, B, steps, "mixed", bc=bc)
    Um, Bm, _, _ = _run(st, mesh, U, B, acc_steps, "mixed", bc=bc)
    Uf, Bf, _, ms_f = _run(st, mesh, U, B, acc_steps, "fp64", bc=bc)
    return {"workload": f"3d_kelvin_helmholtz_amr levels {levels[0]}-{levels[1]} (16^3 blocks, walls in y), "
                        f"{steps} steps",
            "cells": cells, "leaves": mesh.n_owned, "value": cells / (ms * 1e-3), "ms_per_step": ms,
            "fp64_value": cells / (ms_f * 1e-3),
            "accuracy": dict(_accuracy(mesh, U, mesh, Um, Bm, Uf, Bf), steps=acc_steps, against="FP64 GPU path")}


LEGS = {"0": leg_config0, "1": leg_config1, "2": leg_config2, "3": leg_config3, "4": leg_config4}


def run_legs(which, **kw):
    out = {}
    for k in [w for w in which.split(",") if w]:
        t0 = time.perf_counter()
        try:
            # the batched field loops also run to their end time (about 40 s), where finished problems
            # are skipped
            out[f"config{k}"] = LEGS[k](**(dict(kw, to_end=True) if k == "3" else kw))
        except Exception as e:  # noqa: BLE001 - a failing leg is reported, the headline line still prints
            out[f"config{k}"] = {"error": f"{type(e).__name__}: {e}"}
        out[f"config{k}"]["leg_seconds"] = time.perf_counter() - t0
    return out


def run_one_leg(args, rank):
    """--config N: one configuration leg alone (stated sizes unless --levels / --leg-steps say otherwise)."""
    if rank != 0:
        return
    from godunov_mhd_ct_gb300.csrc import build as cbuild

    if not os.path.exists(cbuild.LIB):
        cbuild.build()
    kw = {}
    if args.levels and args.config in ("2", "4"):
        kw["levels"] = tuple(int(v) for v in args.levels.split(":"))
    if args.config == "1":
        kw.update(side_blocks=args.side_blocks, precision=args.precision, tile=args.tile)
    if args.config == "3" and args.to_end:
        kw["to_end"] = True
    if args.leg_steps:
        kw["steps"] = args.leg_steps
    t0 = time.perf_counter()
    leg = LEGS[args.config](**kw)
    line = {"metric": METRIC, "value": leg["value"], "unit": UNIT, "impl": "gmhd", "n_gpus": 1,
            "higher_is_better": True, "dtype": "f32/f64 (mixed)", "data": "synthetic",
            "config": {"workload": leg["workload"], "leg": f"config{args.config}"}, "leg": leg,
            "leg_seconds": time.perf_counter() - t0}
    print(json.dumps(line), flush=True)


def run_reference(args, rank, world):
    if rank != 0:
        return
    cb = cpu_baseline_run(args.steps, min(args.warmup, 2), seconds_cap=120.0, side_blocks=args.side_blocks)
    line = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": cb["steps"], "warmup": args.warmup, "ms_per_step": cb["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": cb["workload"],
                       "note": "the reference's Kokkos build needs kalypsso-core/Kokkos/p4est (absent); this arm "
                               "times the FP64 CPU restatement of its stage on the same workload"},
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gmhd", choices=["gmhd", "reference"])
    ap.add_argument("--side-blocks", type=int, default=8, help="blocks per side (8 -> 256^3 with 32^3 blocks)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--accuracy-steps", type=int, default=50,
                    help="solver iterations of the mixed-vs-FP64 comparison (the workload's 50 steps)")
    ap.add_argument("--legs", default="0,2,3,4",
                    help="the other configurations to run after the headline (comma list of 0, 2, 3, 4; empty: none)")
    ap.add_argument("--config", default=None, choices=sorted(LEGS),
                    help="run one configuration leg alone and print its line (e.g. a small case under ncu)")
    ap.add_argument("--levels", default=None, help="--config 2 or 4: lo:hi refinement levels instead of the stated ones")
    ap.add_argument("--leg-steps", type=int, default=None, help="--config: solver iterations instead of the stated ones")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"], help="--config 1: the path to run")
    ap.add_argument("--tile", type=int, default=None, help="--config 1: tile request instead of the default")
    ap.add_argument("--to-end", action="store_true", help="--config 3: also run and time the batch to t = 0.5")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.config is not None:
        return run_one_leg(args, rank)

    import torch

    from godunov_mhd_ct_gb300.csrc import build as cbuild

    if not os.path.exists(cbuild.LIB):
        cbuild.build()
    from godunov_mhd_ct_gb300.solver import GodunovImplemGB300

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    mesh, U, B = make_workload(side_blocks=args.side_blocks)
    st = settings()
    cells = mesh.n_owned * mesh.ncell
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        dU0 = torch.from_numpy(U).cuda()
        dB0 = torch.from_numpy(B).cuda()
        dU, dB = dU0.clone(), dB0.clone()
        dU2, dB2 = torch.empty_like(dU), torch.empty_like(dB)
    stream.synchronize()

    # ---- headline: mixed-precision solver iterations (graph-captured, dt on device) -----------
    mixed = GodunovImplemGB300(st, mesh, precision="mixed")
    # the tile autotuner picks the shared-memory tile for these 32^3 blocks (U2, B2 are scratch here)
    tile, _ = mixed.autotune(dU, dU2, dB, dB2, mixed.compute_dt(dU, dB, stream=stream), stream=stream)
    mixed.advance(dU, dU2, dB, dB2, args.warmup, stream=stream)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    dtlog, _ = mixed.advance(dU, dU2, dB, dB2, args.steps, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), dist, "cuda")
    value = whole_job_rate(cells, args.steps, world, ms)

    # ---- dominant kernel: the fused step, timed alone with CUDA events on its stream ----------
    nk = 20
    dt_fixed = float(dtlog[0, 0])
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        for _ in range(3):
            mixed.do_time_step(dU0, dU2, dB0, dB2, dt_fixed, stream=stream)
        k0.record(stream)
        for _ in range(nk):
            mixed.do_time_step(dU0, dU2, dB0, dB2, dt_fixed, stream=stream)
        k1.record(stream)
    torch.cuda.synchronize()
    kern_ms = k0.elapsed_time(k1) / nk
    peak, peak_src = hbm_peak()
    achieved = BYTES_PER_CELL_UPDATE * cells / (kern_ms * 1e-3) / 1e9
    n_sm = torch.cuda.get_device_properties(local_rank).multi_processor_count

    out = {}
    if rank == 0:
        # ---- FP64 drop-in path on the same workload, and accuracy of mixed vs FP64 -----------
        n_acc = max(1, args.accuracy_steps)
        fp64 = GodunovImplemGB300(st, mesh, precision="fp64")
        with torch.cuda.stream(stream):
            aU, aB = dU0.clone(), dB0.clone()
            bU, bB = dU0.clone(), dB0.clone()
        fp64.advance(aU, dU2, aB, dB2, 1, stream=stream)  # warm-up (graph capture excluded)
        with torch.cuda.stream(stream):
            aU.copy_(dU0)
            aB.copy_(dB0)
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        fp64.advance(aU, dU2, aB, dB2, n_acc, stream=stream)
        f1.record(stream)
        torch.cuda.synchronize()
        fp64_ms = f0.elapsed_time(f1) / n_acc
        mixed.advance(bU, dU2, bB, dB2, n_acc, stream=stream)
        torch.cuda.synchronize()
        n = mesh.n_owned
        Ua, Ba, Ub, Bb = aU.cpu().numpy()[:n], aB.cpu().numpy()[:n], bU.cpu().numpy()[:n], bB.cpu().numpy()[:n]

        def l1(a, b):
            return float(np.abs(a - b).sum() / np.abs(b).sum())

        Bx, By, Bz = mesh.split_faces(Bb)
        divb = float(np.max(np.abs((Bx[..., 1:] - Bx[..., :-1]) + (By[:, :, 1:] - By[:, :, :-1]) +
                                   (Bz[:, 1:] - Bz[:, :-1])))) / mesh.cell_length()
        out["accuracy"] = {"steps": n_acc, "l1_rho": l1(Ub[:, 0], Ua[:, 0]), "l1_E": l1(Ub[:, 1], Ua[:, 1]),
                           "l1_B": l1(Bb, Ba), "max_divB_mixed": divb,
                           "mass_drift_mixed": float(abs(Ub[:, 0].sum() - U[:n, 0].sum()) / U[:n, 0].sum()),
                           "energy_drift_mixed": float(abs(Ub[:, 1].sum() - U[:n, 1].sum()) / U[:n, 1].sum())}
        out["fp64"] = {"value": cells / (fp64_ms * 1e-3), "ms_per_step": fp64_ms,
                       "mixed_over_fp64": (cells * args.steps / (ms * 1e-3 * world)) / (cells / (fp64_ms * 1e-3))}

        # ---- end to end through the C ABI with host buffers (copies inside the timed region) ---
        hU = torch.from_numpy(U).pin_memory()
        hB = torch.from_numpy(B).pin_memory()
        hU2 = torch.empty_like(hU).pin_memory()
        hB2 = torch.empty_like(hB).pin_memory()
        import ctypes

        from godunov_mhd_ct_gb300 import _native as nat

        L = nat.lib()
        cstream = torch.cuda.current_stream()
        sp = ctypes.c_void_p(cstream.cuda_stream)

        def host_step(a_u, a_b, b_u, b_b, asynchronous):
            fn = L.gmhd_step_host_async if asynchronous else L.gmhd_step_host
            nat.check(fn(mixed._ctx, a_u.data_ptr(), b_u.data_ptr(), a_b.data_ptr(), b_b.data_ptr(),
                         ctypes.c_double(dt_fixed), sp), "gmhd_step_host")

        # dependent chain: every step's input is the previous step's host output (a solver that keeps its
        # state in host memory); the call copies U, B in, steps and copies U2, B2 out before returning
        ne = 6
        host_step(hU, hB, hU2, hB2, False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bufs = [(hU, hB), (hU2, hB2)]
        for k in range(ne):
            (a_u, a_b), (b_u, b_b) = bufs[k % 2], bufs[(k + 1) % 2]
            host_step(a_u, a_b, b_u, b_b, False)
        e2e_dep_s = (time.perf_counter() - t0) / ne
        # independent steps (each step copies the same host input in and its result out), stream-ordered:
        # the copy-in, the step and the copy-out of consecutive steps overlap
        hU.copy_(torch.from_numpy(U))
        hB.copy_(torch.from_numpy(B))
        ne_async = 10
        for _ in range(2):
            host_step(hU, hB, hU2, hB2, True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(ne_async):
            host_step(hU, hB, hU2, hB2, True)
        torch.cuda.synchronize()
        e2e_ind_s = (time.perf_counter() - t0) / ne_async
        out["e2e"] = {"value": cells / e2e_dep_s, "unit": UNIT, "h2d_bytes_per_step": int(U.nbytes + B.nbytes),
                      "d2h_bytes_per_step": int(U[:n].nbytes + B[:n].nbytes),
                      "path": "gmhd_step_host (C ABI, pinned host buffers): copy in, step, copy out, return, the "
                              "copies overlapped with the step slab by slab; a dependent chain, each step's input "
                              "the previous step's host output; mixed, dt fixed",
                      "independent_value": cells / e2e_ind_s,
                      "independent_path": "gmhd_step_host_async: independent steps on the same host input, copy-in, "
                                          "step and copy-out of consecutive steps overlapped"}
        if not args.no_cpu_baseline and world == 1:
            cb = cpu_baseline_run(steps=1000, warmup=1, seconds_cap=15.0, side_blocks=args.side_blocks)
            out["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}

        ctr = read_counters()
        kern_name = ("column_step_kernel<float> (mixed, 16x8 columns through the block)" if tile == 16 else
                     f"fused_step_kernel<float,3,{tile},{tile},{tile}> (mixed, persistent)")
        issue = None
        if ctr and clk.get("sm_mhz"):
            # warp instructions per cell (ncu) x cells / launch time, against 4 issue slots per SM per clock
            inst = ctr["warp_inst_per_cell"] * cells
            peak_issue = n_sm * 4 * clk["sm_mhz"] * 1e6
            issue = {"bound": "issue", "achieved": inst / (kern_ms * 1e-3), "peak": peak_issue,
                     "unit": "warp-instructions/s", "frac": inst / (kern_ms * 1e-3) / peak_issue,
                     "warp_inst_per_cell": ctr["warp_inst_per_cell"], "sms": n_sm, "sm_mhz": clk["sm_mhz"],
                     "source": ctr["source"]}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32/f64 (mixed)", "data": "synthetic",
            "config": {"workload": "3d_orszag_tang_256^3", "cells": cells, "blocks": mesh.n_owned, "tile": tile,
                       "block": list(mesh.block), "ghost": 2, "precision": "mixed", "riemann": "HLLD",
                       "slope": "MC", "cfl": st.cfl, "l2": "inputs (2.2 GB) larger than L2 (129 MB); no flush"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": ctr["dram_bytes_per_cell"] * cells if ctr else None,
                         "traffic_source": (ctr["source"] + " (ncu dram__bytes_read.sum + dram__bytes_write.sum of "
                                            "a small case, per cell, times the cells of this launch)") if ctr else None,
                         "peak_source": peak_src, "kernel": kern_name, "kernel_ms": kern_ms,
                         "bytes_per_launch": BYTES_PER_CELL_UPDATE * cells,
                         "limiter": "instruction issue (see issue_roofline), not HBM"},
            "issue_roofline": issue,
            "gpu_launches": 2 * args.steps,
            "clocks": clk,
        }
        line.update(out)
        if args.legs and world == 1:
            del dU, dB, dU2, dB2, dU0, dB0
            torch.cuda.empty_cache()
            line["configs"] = run_legs(args.legs)
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

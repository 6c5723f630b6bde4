"""Run W warm-up steps and measured do_time_steps of the fused step on a uniform 3D Orszag-Tang
mesh or an AMR workload, for timing and for profiling single launches (e.g. under
ncu -k regex:fused_step -s W -c 1).

    python -m godunov_mhd_ct_gb300.profile_step --precision mixed --side-blocks 4 --block 32
    python -m godunov_mhd_ct_gb300.profile_step --workload blast --levels 5:9 --block 16
"""
from __future__ import annotations

import argparse
import time


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--side-blocks", type=int, default=4)
    ap.add_argument("--block", type=int, default=32)
    ap.add_argument("--dim", type=int, default=3, choices=[2, 3])
    ap.add_argument("--problems", type=int, default=1024, help="fieldloops: number of independent problems")
    ap.add_argument("--t-end", type=float, default=0.5, help="fieldloops: end time of every problem")
    ap.add_argument("--workload", default="ot", choices=["ot", "blast", "kh", "fieldloops"],
                    help="ot: uniform Orszag-Tang; blast: 2D AMR blast; kh: 3D AMR shear layers with walls")
    ap.add_argument("--levels", default="5:8", help="base:max level of the AMR workloads")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--regrid", type=int, default=0,
                    help="AMR workloads: run --repeat solver iterations with an AMR cycle every REGRID steps")
    ap.add_argument("--repeat", type=int, default=1)
    args = ap.parse_args()

    import numpy as np
    import torch

    from . import workloads as wl
    from .mesh import BlockMesh
    from .settings import MHDSettings
    from .solver import GodunovImplemGB300

    st = MHDSettings(gamma0=5.0 / 3.0, cfl=0.5, slope_type=2.0, riemann="HLLD")
    bc = None
    if args.workload == "fieldloops":
        # independent 2D field loops of log-uniform sizes (2N x N cells, N = 32..512) batched in one
        # launch per step, each with its own dt, run until every problem reaches t_end
        t0 = time.perf_counter()
        meshes, states, _ = wl.field_loop_batch(args.problems, seed=12345, sizes=(32, 64, 128, 256, 512))
        mesh, problem = BlockMesh.batch(meshes)
        U = np.concatenate([s_[0] for s_ in states])
        B = np.concatenate([s_[1] for s_ in states])
        del states
        cells = np.array([m.n_owned * m.ncell for m in meshes], dtype=np.float64)
        print(f"fieldloops: {len(meshes)} problems, {cells.sum() / 1e6:.1f} M cells, {mesh.n_owned} blocks "
              f"(setup {time.perf_counter() - t0:.1f} s)")
        impl = GodunovImplemGB300(st, mesh, precision=args.precision, problem=problem, n_problems=len(meshes))
        dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
        dU2, dB2 = torch.empty_like(dU), torch.empty_like(dB)
        t = np.zeros(len(meshes))
        updates, steps = 0.0, 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        while (t < args.t_end).any():
            dtlog, t = impl.advance(dU, dU2, dB, dB2, 100, t=t, t_end=args.t_end)
            updates += float(((dtlog > 0) * cells[None, :]).sum())
            steps += 100
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        print(f"{args.precision} field loops to t={args.t_end}: {steps} launches of the batch, "
              f"{updates / 1e9:.2f} G cell-updates in {el:.2f} s: {updates / el / 1e9:.3f} G cell-updates/s, "
              f"health flags {impl.last_status()}")
        return
    if args.workload == "ot":
        level = int(np.log2(args.side_blocks))
        blk = (args.block, args.block, args.block if args.dim == 3 else 1)
        mesh = BlockMesh.uniform(args.dim, level=level, block=blk)
        U, B = wl.orszag_tang(mesh, gamma=st.gamma0, rho_perturbation=1e-3, seed=12345)
    else:
        lo, hi = (int(v) for v in args.levels.split(":"))
        if args.workload == "blast":
            mesh = wl.blast_mesh(lo, hi, block=args.block)
            U, B = wl.blast(mesh, gamma=st.gamma0)
        else:
            st = MHDSettings(gamma0=1.4, cfl=0.5, slope_type=2.0, riemann="HLLD")
            mesh = wl.kh_amr_mesh(lo, hi, block=args.block)
            U, B = wl.kelvin_helmholtz(mesh, gamma=st.gamma0, seed=12345)
            bc = (1, 1, 3, 3, 1, 1)
        print(f"{args.workload}: {mesh.n_owned} leaves, levels {np.bincount(mesh.level[: mesh.n_owned])[lo:]}")
    impl = GodunovImplemGB300(st, mesh, precision=args.precision, bc=bc)
    dU, dB = torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda()
    dU2, dB2 = torch.empty_like(dU), torch.empty_like(dB)
    if bc is not None:
        impl.fill_outside(dU, dB)
    dt = impl.compute_dt(dU, dB)
    for _ in range(args.warmup):
        impl.do_time_step(dU, dU2, dB, dB2, dt)
    torch.cuda.synchronize()
    if args.regrid > 0 and args.workload != "ot":
        # solver loop with AMR cycles (SolverGodunovMHD::next_iteration_impl): cell-updates over wall time
        lo, hi = (int(v) for v in args.levels.split(":"))
        crit = dict(criterion="LOHNER_UNSPLIT", eps_refine=0.16, eps_coarsen=0.02, eps_lohner=0.02,
                    variables=("rho", "pressure"))
        # warm-up: one AMR cycle outside the timed region (first use of the allocator and fill kernels)
        mesh, dU, dB = impl.regrid(dU, dB, lo, hi, **crit)
        torch.cuda.synchronize()
        impl.regrid_seconds = [0.0] * 4
        updates, done, t_regrid, cycles = 0, 0, 0.0, 0
        t0 = time.perf_counter()
        while done < args.repeat:
            n = min(args.regrid, args.repeat - done)
            impl.advance(dU, torch.empty_like(dU), dB, torch.empty_like(dB), n)
            updates += n * mesh.n_owned * mesh.ncell
            done += n
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            mesh, dU, dB = impl.regrid(dU, dB, lo, hi, **crit)
            t_regrid += time.perf_counter() - t1
            cycles += 1
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        parts = ", ".join(f"{k} {1e3 * v / cycles:.3f} ms" for k, v in
                          zip(("flags", "adapt", "remap", "set_mesh"), impl.regrid_seconds))
        print(f"per cycle ({cycles}): {parts}; steps {1e3 * (el - t_regrid) / cycles:.3f} ms per {args.regrid} steps")
        print(f"{args.precision} {mesh.dim}D with an AMR cycle every {args.regrid} steps: {args.repeat} steps, "
              f"{updates / el / 1e9:.3f} G cell-updates/s, regrid {t_regrid / el * 100:.1f} % of the time, "
              f"final {mesh.n_owned} leaves, levels {np.bincount(mesh.level[: mesh.n_owned])[lo:]}")
        return
    t0 = time.perf_counter()
    for _ in range(args.repeat):
        impl.do_time_step(dU, dU2, dB, dB2, dt)
    torch.cuda.synchronize()
    el = (time.perf_counter() - t0) / args.repeat
    cells = mesh.n_owned * mesh.ncell
    flags = impl.last_status()
    print(f"{args.precision} {mesh.dim}D {cells} cells: {el * 1e3:.3f} ms/step, {cells / el / 1e9:.3f} Gcell/s, "
          f"health flags {flags}")


if __name__ == "__main__":
    main()

"""Record golden vectors from the reference's own per-cell MHD math.

Runs the known-answer bridge (oracle/refkat: the reference's models/mhd_utils.h,
models/RiemannSolvers_MHD.h and models/HydroSettings.cpp compiled unmodified against stub
headers) on seeded inputs and writes ``kat_models.npz`` next to this script. Needs the reference
tree (default /root/reference, or $GMHD_REFERENCE_TREE); the committed npz is what tests use.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as orc  # noqa: E402

GAMMAS = (5.0 / 3.0, 1.4)
SMALLR, SMALLC = 1e-10, 1e-10


def dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def random_prims(rng, n):
    """Primitive states (rho, p, u, v, w, Bx, By, Bz) spanning low/high beta and fast flows."""
    q = np.empty((n, 8))
    q[:, 0] = 10.0 ** rng.uniform(-2, 1, n)
    q[:, 1] = 10.0 ** rng.uniform(-3, 1.5, n)
    q[:, 2:5] = rng.uniform(-3, 3, (n, 3))
    q[:, 5:8] = rng.uniform(-2, 2, (n, 3))
    return q


def special_pairs():
    """Hand-picked Riemann problems: degenerate, symmetric, supersonic and shock-tube states."""
    bw_l = [1.0, 1.0, 0.0, 0.0, 0.0, 0.75, 1.0, 0.0]
    bw_r = [0.125, 0.1, 0.0, 0.0, 0.0, 0.75, -1.0, 0.0]
    same = [1.0, 1.0, 0.3, -0.2, 0.1, 0.5, 0.4, -0.3]
    zero_bn_l = [1.0, 1.0, 0.1, 0.2, 0.3, 0.0, 0.5, 0.2]
    zero_bn_r = [0.5, 0.3, -0.1, 0.0, 0.1, 0.0, -0.5, 0.1]
    super_r = [1.0, 0.01, 20.0, 0.0, 0.0, 0.1, 0.1, 0.0]
    super_l = [1.0, 0.01, -20.0, 0.0, 0.0, 0.1, 0.1, 0.0]
    low_beta_l = [1.0, 1e-3, 0.0, 0.0, 0.0, 1.0, 1.0, 0.5]
    low_beta_r = [1.0, 1e-3, 0.0, 0.0, 0.0, 1.0, -1.0, 0.5]
    l = [bw_l, same, zero_bn_l, super_r, super_l, low_beta_l, bw_r]
    r = [bw_r, same, zero_bn_r, super_r, super_l, low_beta_r, bw_l]
    return np.array(l), np.array(r)


def main():
    if not orc.build_refkat():
        raise SystemExit("reference tree not found: cannot record golden vectors")
    R = ctypes.CDLL(orc._REF_PATH)
    R.ref_settings.argtypes = [ctypes.c_double] * 4 + [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    i64 = ctypes.c_int64
    R.ref_riemann_batch.argtypes = [ctypes.c_double] * 3 + [ctypes.c_int, i64] + [ctypes.POINTER(ctypes.c_double)] * 3
    R.ref_compute_emf_batch.argtypes = [ctypes.c_double] * 3 + [i64, ctypes.c_int] + [ctypes.POINTER(ctypes.c_double)] * 2
    R.ref_compute_primitives_batch.argtypes = [ctypes.c_double] * 3 + [i64] + [ctypes.POINTER(ctypes.c_double)] * 3
    R.ref_find_speed_info_batch.argtypes = [ctypes.c_double, i64, ctypes.c_int] + [ctypes.POINTER(ctypes.c_double)] * 2
    R.ref_find_speed_fast_batch.argtypes = [ctypes.c_double, i64, ctypes.c_int] + [ctypes.POINTER(ctypes.c_double)] * 2

    rng = np.random.default_rng(20261203)
    out = {}
    # settings derivation (HydroSettings.cpp:18-31)
    rows = []
    for g in GAMMAS:
        for st in (1.0, 2.0):
            o = np.zeros(9)
            R.ref_settings(g, st, SMALLR, SMALLC, 5, dp(o))
            rows.append(np.concatenate([[g, st, SMALLR, SMALLC, 5], o]))
    out["settings"] = np.array(rows)

    n = 128
    for g in GAMMAS:
        gt = f"g{int(round(g * 1000))}"
        ql = random_prims(rng, n)
        qr = random_prims(rng, n)
        sl, sr = special_pairs()
        ql = np.ascontiguousarray(np.concatenate([ql, sl]))
        qr = np.ascontiguousarray(np.concatenate([qr, sr]))
        for rid, name in ((2, "llf"), (3, "hll"), (4, "hllc"), (5, "hlld")):
            f = np.zeros_like(ql)
            R.ref_riemann_batch(g, SMALLR, SMALLC, rid, ql.shape[0], dp(ql), dp(qr), dp(f))
            out[f"riemann_{name}_{gt}_qL"] = ql
            out[f"riemann_{name}_{gt}_qR"] = qr
            out[f"riemann_{name}_{gt}_flux"] = f
        qe = np.ascontiguousarray(random_prims(rng, 4 * n).reshape(n, 4, 8))
        # a few edges with all four states equal (uniform flow)
        qe[:8] = qe[:8, :1, :]
        for d in range(3):
            e = np.zeros(n)
            R.ref_compute_emf_batch(g, SMALLR, SMALLC, n, d, dp(qe), dp(e))
            out[f"emf{d}_{gt}_q"] = qe
            out[f"emf{d}_{gt}_out"] = e
        u = np.empty((n, 8))
        u[:, 0] = 10.0 ** rng.uniform(-2, 1, n)
        u[:, 2:5] = rng.uniform(-3, 3, (n, 3)) * u[:, :1]
        u[:, 5:8] = rng.uniform(-2, 2, (n, 3))
        ek = 0.5 * (u[:, 2] ** 2 + u[:, 3] ** 2 + u[:, 4] ** 2) / u[:, 0]
        em = 0.5 * (u[:, 5] ** 2 + u[:, 6] ** 2 + u[:, 7] ** 2)
        u[:, 1] = ek + em + 10.0 ** rng.uniform(-3, 1, n) / (g - 1)
        u[:16, 1] = ek[:16] + em[:16] - 0.1  # negative internal energy -> pressure floor
        u[16:24, 0] = -1.0  # density below smallr -> density floor
        u = np.ascontiguousarray(u)
        q = np.zeros_like(u)
        c = np.zeros(n)
        R.ref_compute_primitives_batch(g, SMALLR, SMALLC, n, dp(u), dp(q), dp(c))
        out[f"prim_{gt}_u"] = u
        out[f"prim_{gt}_q"] = q
        out[f"prim_{gt}_c"] = c
        qs = np.ascontiguousarray(random_prims(rng, n))
        for dim in (2, 3):
            v = np.zeros((n, 3))
            R.ref_find_speed_info_batch(g, n, dim, dp(qs), dp(v))
            out[f"speedinfo{dim}_{gt}_q"] = qs
            out[f"speedinfo{dim}_{gt}_out"] = v
        for d in range(3):
            v = np.zeros(n)
            R.ref_find_speed_fast_batch(g, n, d, dp(qs), dp(v))
            out[f"speedfast{d}_{gt}_out"] = v
        out[f"speedfast_{gt}_q"] = qs
    path = os.path.join(HERE, "kat_models.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path)} bytes, {len(out)} arrays)")


if __name__ == "__main__":
    main()

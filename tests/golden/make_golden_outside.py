"""Record golden digests of the reference's fill of the blocks beyond non-periodic domain borders.

Runs the functor bridge (oracle/refkat/functor_bridge.cpp: the reference's FillOutsideCellFunctor,
border_conditions/FillOutside.cpp, compiled unmodified against the stub headers) on 2D and 3D meshes
(uniform and two-level) whose non-periodic faces carry ZERO_GRADIENT and WALL border conditions, mixed
per face, so that edge and corner outside blocks see two or three conditions. The state is seeded
(``case_inputs``), the outside blocks start from noise so that a value the fill leaves untouched
shows. Writes ``functor_outside.npz`` next to this script: per case the SHA-256 digests of the
outside blocks' U and B after the reference's fill (``sha_U``, ``sha_B``) and, for the smallest case,
the arrays in full. Needs the reference tree (default /root/reference, or $GMHD_REFERENCE_TREE); the
committed npz is what tests use.

    python tests/golden/make_golden_outside.py
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from godunov_mhd_ct_gb300 import workloads as wl  # noqa: E402
from godunov_mhd_ct_gb300.mesh import BlockMesh  # noqa: E402
from oracle import oracle as orc  # noqa: E402

BRIDGE = os.path.join(ROOT, "oracle", "_ref", "libref_functors.so")
ZG, WALL, PER = 2, 3, 1

# name: dim, block, level(s) (base, refined band or None), border conditions per face, seed
CASES = {
    "2d_walls": (2, (8, 8, 1), (2, None), (WALL, WALL, WALL, WALL, PER, PER), 11),
    "2d_zero_gradient": (2, (8, 8, 1), (2, None), (ZG, ZG, ZG, ZG, PER, PER), 12),
    "2d_mixed": (2, (8, 4, 1), (2, None), (ZG, WALL, WALL, ZG, PER, PER), 13),
    "2d_mixed_amr": (2, (8, 8, 1), (2, ((0.5, 0.5, 0.5), 0.0, 0.15)), (WALL, ZG, ZG, WALL, PER, PER), 14),
    "3d_mixed": (3, (4, 4, 4), (1, None), (ZG, WALL, WALL, ZG, ZG, WALL), 15),
    "3d_yz_amr": (3, (4, 4, 4), (2, ((0.5, 0.5, 0.5), 0.0, 0.1)), (PER, PER, WALL, ZG, WALL, WALL), 16),
}
GAMMA = 5.0 / 3.0


def case_mesh(name):
    dim, block, (base, band), bc, _ = CASES[name]
    periodic = tuple(bc[2 * a] == PER for a in range(3))
    if band is None:
        return BlockMesh.uniform(dim, level=base, block=block, periodic=periodic)
    c, lo, hi = band
    return BlockMesh.amr(dim, wl.refine_band(c, lo, hi, axes=dim), base_level=base, max_level=base + 1, block=block,
                         periodic=periodic)


def case_inputs(name):
    """Mesh, oracle mesh, border conditions and the seeded U, B of every block (outside ones noise)."""
    dim, block, _, bc, seed = CASES[name]
    mesh = case_mesh(name)
    U, B = wl.random_smooth(mesh, gamma=GAMMA, seed=seed, amp=0.3)
    rng = np.random.default_rng(seed + 1000)
    n = mesh.n_owned
    U[n:] = rng.uniform(-1.0, 1.0, U[n:].shape)
    B[n:] = rng.uniform(-1.0, 1.0, B[n:].shape)
    om = orc.Mesh.from_block_mesh(mesh, bc=list(bc))
    return mesh, om, list(bc), U, B


def reference_fill_outside(mesh, bc, U, B):
    """The reference's FillOutsideCellFunctor on copies of U, B (all blocks). Returns (U, B)."""
    L = ctypes.CDLL(BRIDGE)
    ip = ctypes.POINTER(ctypes.c_int)
    dp = ctypes.POINTER(ctypes.c_double)
    Uo = np.array(U, dtype=np.float64, copy=True, order="C")
    Bo = np.array(B, dtype=np.float64, copy=True, order="C")
    lev = np.ascontiguousarray(mesh.level, dtype=np.int32)
    nbr = np.ascontiguousarray(mesh.neighbor, dtype=np.int32).reshape(-1)
    coord = np.ascontiguousarray(mesh.coords, dtype=np.int32).reshape(-1)
    b = (ctypes.c_int * 3)(*mesh.block)
    bcs = (ctypes.c_int * 6)(*bc)
    rc = L.ref_fill_outside(mesh.dim, b, mesh.n_blocks, mesh.n_owned, lev.ctypes.data_as(ip), nbr.ctypes.data_as(ip),
                            coord.ctypes.data_as(ip), bcs, Uo.ctypes.data_as(dp), Bo.ctypes.data_as(dp))
    if rc != 0:
        raise RuntimeError(f"ref_fill_outside failed: {rc}")
    return Uo, Bo


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def main():
    if not orc.build_refkat() or not os.path.exists(BRIDGE):
        sys.exit("the reference tree is needed to record the golden outside fill")
    out = {}
    for name in CASES:
        mesh, om, bc, U, B = case_inputs(name)
        Ur, Br = reference_fill_outside(mesh, bc, U, B)
        n = mesh.n_owned
        assert np.array_equal(Ur[:n], U[:n]) and np.array_equal(Br[:n], B[:n])
        out[f"{name}_n_outside"] = np.int64(mesh.n_blocks - n)
        out[f"{name}_sha_U"] = np.array(digest(Ur[n:]))
        out[f"{name}_sha_B"] = np.array(digest(Br[n:]))
        if name == "2d_mixed":
            out[f"{name}_U"], out[f"{name}_B"] = Ur[n:], Br[n:]
    path = os.path.join(HERE, "functor_outside.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({len(CASES)} cases)")


if __name__ == "__main__":
    main()

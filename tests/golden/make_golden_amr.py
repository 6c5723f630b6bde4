"""Record golden arrays of the reference's coarse/fine stage code.

Runs the functor bridge (oracle/refkat/functor_bridge.cpp: the reference's
CorrectEmfAtBlockBorderFunctor and ReadFluxesAndConservativeUpdateFunctor compiled unmodified
against stub headers whose StencilHelper reads the mesh's neighbour tables) on two-level 2D and 3D
meshes, with inputs made by the oracle: the raw edge EMFs of every owned block (``emf_raw``,
oracle_block_fluxes_emf) and the face fluxes of one step (``fluxes``, oracle_step_fluxes). Writes
``functor_amr.npz`` next to this script: per case dt and the reference's results on the blocks next
to a level change (``blocks``: owned blocks with a neighbour at another level), the corrected EMFs
(``emf_ref``) and their U and faces after the conservative update from U, B (``upd_U``, ``upd_B``);
the inputs are rebuilt from the seeded state (``case_inputs``). The reference's ghosted primitive
variables (ConvertToPrimitivesVariablesFunctor, SIMPLE_COPY and EXTRAPOLATE_LINEAR_MINMOD) of the
blocks in ``prim_blocks`` (the level-change blocks, and on walled meshes also those next to outside
blocks) are kept as SHA-256 digests of their bytes (``prim_sha_<prolongation>``), the first two
of them in full (``prim_q_<prolongation>``). Needs the reference tree
(default /root/reference, or $GMHD_REFERENCE_TREE); the committed npz is what tests use.

    python tests/golden/make_golden_amr.py
"""
from __future__ import annotations

import ctypes
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

# name: dim, block, refined shell (centre, r_lo, r_hi), base level, periodic, state seed
CASES = {
    "2d_b8": (2, (8, 8, 1), ((0.5, 0.5, 0.5), 0.1, 0.2), 2, (True, True, True), 3),
    "2d_b8_walls": (2, (8, 8, 1), ((0.5, 0.5, 0.5), 0.0, 0.1), 2, (True, False, True), 4),
    "3d_b4": (3, (4, 4, 4), ((0.375, 0.375, 0.375), 0.0, 0.04), 2, (True, True, True), 5),
    "3d_b4_corner": (3, (4, 4, 4), ((0.25, 0.25, 0.25), 0.0, 0.05), 1, (True, True, True), 6),
}
GAMMA, SLOPE = 5.0 / 3.0, 2.0


def case_mesh(name):
    dim, block, (c, lo, hi), base, periodic, _ = CASES[name]
    return BlockMesh.amr(dim, wl.refine_band(c, lo, hi, axes=dim), base_level=base, max_level=base + 1, block=block,
                         periodic=periodic)


def case_inputs(name):
    """Mesh, oracle mesh and settings, state, dt, raw EMFs [n_owned][1|3][(b+1)^d] and fluxes."""
    dim, block, _, _, periodic, seed = CASES[name]
    mesh = case_mesh(name)
    U, B = wl.random_smooth(mesh, gamma=GAMMA, seed=seed, amp=0.3)
    bc = [1 if periodic[d // 2] else 3 for d in range(6)]
    om = orc.Mesh.from_block_mesh(mesh, bc=bc)
    st = orc.settings(gamma0=GAMMA, cfl=0.4, slope_type=SLOPE, riemann=5)
    U, B = orc.fill_outside(om, U, B)
    dt = 0.4 / orc.inv_dt(om, st, U, B)
    ne = int(np.prod([v + 1 for v in block[:dim]])) * (3 if dim == 3 else 1)
    emf = np.zeros((mesh.n_owned, ne))
    for blk in range(mesh.n_owned):
        _, emf[blk] = orc.block_fluxes_emf(om, st, U, B, dt, blk)
    _, _, fluxes = orc.step_fluxes(om, st, U, B, dt)
    return mesh, om, st, U, B, dt, emf, fluxes


def _tables(mesh):
    ip = ctypes.POINTER(ctypes.c_int)
    keep = [np.ascontiguousarray(mesh.level, dtype=np.int32),
            np.ascontiguousarray(mesh.neighbor, dtype=np.int32).reshape(-1),
            None if mesh.fine_neighbor is None else np.ascontiguousarray(mesh.fine_neighbor, dtype=np.int32).reshape(-1),
            np.ascontiguousarray(mesh.coords, dtype=np.int32).reshape(-1)]
    ptrs = [a.ctypes.data_as(ip) if a is not None else ctypes.cast(None, ip) for a in keep]
    return keep, ptrs


def reference_correct_emf(mesh, emf):
    """The reference's CorrectEmfAtBlockBorderFunctor on the raw EMFs of the owned blocks (the bridge's
    [n_blocks][3][(b+1)^d] array, 2D: component 2). Returns the corrected owned-block EMFs in the
    oracle's layout ([n_owned][1|3][(b+1)^d])."""
    L = ctypes.CDLL(BRIDGE)
    dp = ctypes.POINTER(ctypes.c_double)
    dim = mesh.dim
    ne = int(np.prod([v + 1 for v in mesh.block[:dim]]))
    full = np.zeros((mesh.n_blocks, 3, ne))
    if dim == 3:
        full[: mesh.n_owned] = emf.reshape(mesh.n_owned, 3, ne)
    else:
        full[: mesh.n_owned, 2] = emf
    out = np.zeros_like(full)
    keep, (lev, nbr, fine, coord) = _tables(mesh)
    b = (ctypes.c_int * 3)(*mesh.block)
    rc = L.ref_correct_emf(dim, b, mesh.n_blocks, mesh.n_owned, lev, nbr, fine, coord, full.ctypes.data_as(dp),
                           out.ctypes.data_as(dp))
    if rc != 0:
        raise RuntimeError(f"ref_correct_emf failed: {rc}")
    out = out[: mesh.n_owned]
    return out.reshape(mesh.n_owned, -1) if dim == 3 else out[:, 2].copy()


def reference_update(mesh, dt, fluxes, U, B):
    """The reference's ReadFluxesAndConservativeUpdateFunctor (all directions) on the owned blocks of a
    copy of U, B by the per-block face fluxes. Returns (U, B) of the owned blocks."""
    L = ctypes.CDLL(BRIDGE)
    dp = ctypes.POINTER(ctypes.c_double)
    n = mesh.n_owned
    Uo = np.array(U[:n], dtype=np.float64, copy=True, order="C")
    Bo = np.array(B[:n], dtype=np.float64, copy=True, order="C")
    fl = np.ascontiguousarray(fluxes, dtype=np.float64)
    keep, (lev, nbr, fine, coord) = _tables(mesh)
    b = (ctypes.c_int * 3)(*mesh.block)
    prm = (ctypes.c_double * 6)(GAMMA, SLOPE, 1e-10, 1e-10, 1.0, 0.0)
    flags = (ctypes.c_int * 5)(5, 0, 0, 0, 0)
    g = (ctypes.c_double * 3)(0.0, 0.0, 0.0)
    rc = L.ref_update_mesh(mesh.dim, b, mesh.n_blocks, n, lev, nbr, fine, coord, prm, flags, g, ctypes.c_double(dt),
                           fl.ctypes.data_as(dp), Uo.ctypes.data_as(dp), Bo.ctypes.data_as(dp))
    if rc != 0:
        raise RuntimeError(f"ref_update_mesh failed: {rc}")
    return Uo, Bo


def reference_primitives(mesh, U, B, blk, prolongation, om):
    """The reference's ConvertToPrimitivesVariablesFunctor on owned block blk: its primitive variables
    [11][(b+4)^d] with the ghost cells filled from the neighbour leaves. The ghosted face field it reads
    is the oracle's (block_ghost_faces) for owned blocks and the block's own faces for outside ones."""
    L = ctypes.CDLL(BRIDGE)
    dp = ctypes.POINTER(ctypes.c_double)
    dim = mesh.dim
    nbg = orc.block_ghost_faces(om, U, B, 0).size
    Bg = np.zeros((mesh.n_blocks, nbg))
    for k in range(mesh.n_owned):
        Bg[k] = orc.block_ghost_faces(om, U, B, k)
    # outside blocks: their own faces inside the ghosted box (the part the functor reads)
    g = [v + 4 for v in mesh.block[:dim]]
    faces = mesh.split_faces(B)
    for k in range(mesh.n_owned, mesh.n_blocks):
        off = 0
        for comp in range(3):
            shape = [g[d] + (1 if d == comp and not (dim == 2 and comp == 2) else 0) for d in range(dim)][::-1]
            box = np.zeros(shape)
            inner = faces[comp][k] if dim == 3 else faces[comp][k][0]
            sl = tuple(slice(2, 2 + n) for n in inner.shape)
            box[sl] = inner
            Bg[k, off:off + box.size] = box.reshape(-1)
            off += box.size
    n2 = int(np.prod(g))
    q = np.zeros(11 * n2)
    keep, (lev, nbr, fine, coord) = _tables(mesh)
    b = (ctypes.c_int * 3)(*mesh.block)
    prm = (ctypes.c_double * 6)(GAMMA, SLOPE, 1e-10, 1e-10, 1.0, 0.0)
    Uc = np.ascontiguousarray(U, dtype=np.float64)
    rc = L.ref_block_primitives(dim, b, mesh.n_blocks, mesh.n_owned, lev, nbr, fine, coord, prm, int(prolongation),
                                Uc.ctypes.data_as(dp), Bg.ctypes.data_as(dp), int(blk), q.ctypes.data_as(dp))
    if rc != 0:
        raise RuntimeError(f"ref_block_primitives failed: {rc}")
    return q


def level_change_blocks(mesh):
    """Owned blocks with a neighbour region at another level (coarser, or split into finer leaves)."""
    n = mesh.n_owned
    nb = mesh.neighbor[:n]
    other = np.zeros(n, bool)
    for b in range(n):
        for s_ in range(27):
            v = nb[b, s_]
            if v >= 0 and mesh.level[v] != mesh.level[b]:
                other[b] = True
            if v < 0 and mesh.fine_neighbor is not None and (mesh.fine_neighbor[b, s_] >= 0).any():
                other[b] = True
    return np.nonzero(other)[0].astype(np.int32)


def prim_blocks(mesh):
    """Blocks whose ghost cells come from another level or from outside blocks."""
    sel = set(level_change_blocks(mesh).tolist())
    n = mesh.n_owned
    for b in range(n):
        if np.any((mesh.neighbor[b] >= n)):
            sel.add(b)
    return np.array(sorted(sel), dtype=np.int32)


def digest(a):
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def oracle_mesh_of(mesh, prolongation):
    bc = [1 if mesh.periodic[d // 2] else 3 for d in range(6)]
    return orc.Mesh.from_block_mesh(mesh, bc=bc, prolongation=prolongation)


def main():
    if not orc.build_refkat() or not os.path.exists(BRIDGE):
        sys.exit("the reference tree is needed to record the golden coarse/fine stages")
    out = {}
    for name in CASES:
        mesh, om, st, U, B, dt, emf, fluxes = case_inputs(name)
        sel = level_change_blocks(mesh)
        out[f"{name}_dt"] = np.float64(dt)
        out[f"{name}_blocks"] = sel
        out[f"{name}_emf_ref"] = reference_correct_emf(mesh, emf)[sel]
        Uu, Bu = reference_update(mesh, dt, fluxes, U, B)
        out[f"{name}_upd_U"], out[f"{name}_upd_B"] = Uu[sel], Bu[sel]
        pb = prim_blocks(mesh)
        out[f"{name}_prim_blocks"] = pb
        for prol in (0, 1):
            om2 = oracle_mesh_of(mesh, prol)
            qs = [reference_primitives(mesh, U, B, int(b), prol, om2) for b in pb]
            out[f"{name}_prim_sha_{prol}"] = np.array([digest(q) for q in qs])
            out[f"{name}_prim_q_{prol}"] = np.array(qs[:2])
    path = os.path.join(HERE, "functor_amr.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({len(CASES)} cases)")


if __name__ == "__main__":
    main()

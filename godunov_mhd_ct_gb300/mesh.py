"""Block mesh: leaf blocks of a p4est-style brick forest at one refinement level, with the
neighbour table the kernels use in place of kalypsso-core's hashmap + StencilHelper lookups.

Block order follows p4est: bricks (trees) in x-fastest order, then leaves along the Morton
(Z-order) curve inside each brick (SolverGodunovMHD.cpp:323-371 partitions along that curve).

Neighbour table: ``neighbor[b, (oz+1)*9 + (oy+1)*3 + (ox+1)]`` is the block sharing the face,
edge or corner of block ``b`` in direction (ox, oy, oz) in {-1,0,1}^3, or -1 across a domain
boundary that has no outside block.

Outside blocks (non-periodic directions) are appended after the owned blocks, as the reference
stores its "outside" quadrants after owned + ghost ones; ``border_conditions/FillOutside.cpp``
fills them before each step. ``outside_src[b - n_owned]`` is the inside block across the
outside normal (diagonal for edge/corner outside blocks) and ``outside_normal[b - n_owned]`` the
normal per axis: +1 when the block lies below the domain, -1 above it, 0 within its range.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


def _morton_key(ix: np.ndarray, iy: np.ndarray, iz: np.ndarray, bits: int) -> np.ndarray:
    key = np.zeros(ix.shape, dtype=np.int64)
    for b in range(bits):
        key |= ((ix >> b) & 1).astype(np.int64) << (3 * b)
        key |= ((iy >> b) & 1).astype(np.int64) << (3 * b + 1)
        key |= ((iz >> b) & 1).astype(np.int64) << (3 * b + 2)
    return key


def nb_slot(ox: int, oy: int, oz: int) -> int:
    return (oz + 1) * 9 + (oy + 1) * 3 + (ox + 1)


@dataclass
class BlockMesh:
    dim: int
    block: tuple            # (bx, by, bz); bz == 1 in 2D
    level: np.ndarray       # [n_blocks] int32
    neighbor: np.ndarray    # [n_blocks, 27] int32
    coords: np.ndarray      # [n_blocks, 3] int64 block coordinates (outside blocks: outside the grid)
    n_owned: int
    grid: tuple             # blocks per direction over the whole domain
    periodic: tuple
    scaling_factor: float = 1.0
    outside_src: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    outside_normal: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    bricks: tuple = (1, 1, 1)  # root trees per direction
    # children of neighbour regions one level finer, as a list: (flat indices into the [n_blocks, 27, 8]
    # table, leaf ids) of its entries that are not -1; None on meshes without level jumps
    fine_list: tuple | None = None
    _fine_dense: np.ndarray | None = field(default=None, repr=False)

    @property
    def fine_neighbor(self) -> np.ndarray | None:
        """[n_blocks, 27, 8] leaves covering a neighbour region one level finer (children x fastest, -1
        where absent), built from fine_list when first read; None on meshes without level jumps."""
        if self._fine_dense is None and self.fine_list is not None:
            dense = np.full(self.n_blocks * 27 * 8, -1, np.int32)
            dense[self.fine_list[0]] = self.fine_list[1]
            self._fine_dense = dense.reshape(self.n_blocks, 27, 8)
        return self._fine_dense

    @property
    def n_blocks(self) -> int:
        return int(self.level.shape[0])

    @property
    def ncell(self) -> int:
        bx, by, bz = self.block
        return bx * by * bz

    @property
    def face_counts(self):
        bx, by, bz = self.block
        nfx = (bx + 1) * by * bz
        nfy = bx * (by + 1) * bz
        nfz = bx * by * (bz + 1) if self.dim == 3 else bx * by
        return nfx, nfy, nfz

    @property
    def nface(self) -> int:
        return sum(self.face_counts)

    @property
    def is_amr(self) -> bool:
        if self.fine_list is not None:
            return True
        return self.n_owned > 0 and bool(np.any(self.level[: self.n_owned] != self.level[0]))

    def domain_length(self, d: int) -> float:
        """Extent of the domain along axis d (``grid`` counts blocks at the finest level)."""
        return self.grid[d] * self.block[d] * self.cell_length(int(self.level[: self.n_owned].max()))

    def block_dx(self) -> np.ndarray:
        """Cell length per block: (1 / (bx * 2^level)) * scaling_factor."""
        return (1.0 / (float(self.block[0]) * np.exp2(self.level.astype(np.float64)))) * self.scaling_factor

    def cell_length(self, level: int | None = None) -> float:
        """dx = (1 / (bx * 2^level)) * scaling_factor (core compute_cell_length, unit brick)."""
        lv = int(self.level[0]) if level is None else level
        return (1.0 / float(self.block[0] << lv)) * self.scaling_factor

    @staticmethod
    def uniform(dim: int, bricks=(1, 1, 1), level: int = 0, block=(16, 16, 16), periodic=(True, True, True),
                scaling_factor: float = 1.0) -> "BlockMesh":
        """All leaves of a brick forest refined uniformly to ``level``."""
        if dim not in (2, 3):
            raise ValueError("dim must be 2 or 3")
        bx, by, bz = block
        if dim == 2:
            bz = 1
            bricks = (bricks[0], bricks[1], 1)
        if min(bx, by) < 4 or (dim == 3 and bz < 4):
            raise ValueError("block sizes must be >= 2*ghost_width = 4 (SolverGodunovMHD.cpp:118-140)")
        n_side = 1 << level
        gx, gy = bricks[0] * n_side, bricks[1] * n_side
        gz = bricks[2] * n_side if dim == 3 else 1
        per = tuple(bool(p) for p in periodic[:dim]) + (True,) * (3 - dim)
        # enumerate blocks in p4est order
        tz, ty, tx = np.meshgrid(np.arange(bricks[2]), np.arange(bricks[1]), np.arange(bricks[0]), indexing="ij")
        trees = np.stack([tx.ravel(), ty.ravel(), tz.ravel()], axis=1)
        lz, ly, lx = np.meshgrid(np.arange(n_side if dim == 3 else 1), np.arange(n_side), np.arange(n_side),
                                 indexing="ij")
        lx, ly, lz = lx.ravel(), ly.ravel(), lz.ravel()
        order = np.argsort(_morton_key(lx, ly, lz, max(level, 1)), kind="stable")
        lx, ly, lz = lx[order], ly[order], lz[order]
        coords = []
        for t in trees:
            coords.append(np.stack([t[0] * n_side + lx, t[1] * n_side + ly,
                                    (t[2] * n_side if dim == 3 else 0) + lz], axis=1))
        coords = np.concatenate(coords).astype(np.int64)
        n_owned = coords.shape[0]
        lookup = -np.ones((gx, gy, gz), dtype=np.int64)
        lookup[coords[:, 0], coords[:, 1], coords[:, 2]] = np.arange(n_owned)

        # outside blocks across non-periodic boundaries: one layer, including edge/corner ones
        ext_lookup = {}
        out_coords, out_src, out_normal = [], [], []
        if not all(per[:dim]):
            rng = [range(-1, g + 1) if not per[d] else range(g) for d, g in enumerate((gx, gy, gz))]
            if dim == 2:
                rng[2] = range(1)
            for cz in rng[2]:
                for cy in rng[1]:
                    for cx in rng[0]:
                        c = (cx, cy, cz)
                        inside = 0 <= cx < gx and 0 <= cy < gy and 0 <= cz < gz
                        if inside:
                            continue
                        # source: clamp to the grid (the block across the inward normal)
                        src = (min(max(cx, 0), gx - 1), min(max(cy, 0), gy - 1), min(max(cz, 0), gz - 1))
                        normal = tuple(int(np.sign(src[d] - c[d])) for d in range(3))
                        ext_lookup[c] = n_owned + len(out_coords)
                        out_coords.append(c)
                        out_src.append(lookup[src])
                        out_normal.append(normal)
        n_blocks = n_owned + len(out_coords)
        all_coords = np.concatenate([coords, np.array(out_coords, dtype=np.int64).reshape(-1, 3)])
        gsz = (gx, gy, gz)

        def find(c):
            c = list(c)
            for d in range(3):
                if per[d]:
                    c[d] %= gsz[d]
            if all(0 <= c[d] < gsz[d] for d in range(3)):
                return int(lookup[c[0], c[1], c[2]])
            return ext_lookup.get(tuple(c), -1)

        neighbor = -np.ones((n_blocks, 27), dtype=np.int32)
        offs = [(ox, oy, oz) for oz in (-1, 0, 1) for oy in (-1, 0, 1) for ox in (-1, 0, 1)]
        if all(per[:dim]):
            # vectorised periodic case
            for ox, oy, oz in offs:
                if dim == 2 and oz != 0:
                    continue
                nc = (coords + np.array([ox, oy, oz])) % np.array(gsz)
                neighbor[:n_owned, nb_slot(ox, oy, oz)] = lookup[nc[:, 0], nc[:, 1], nc[:, 2]]
        else:
            for b in range(n_blocks):
                for ox, oy, oz in offs:
                    if dim == 2 and oz != 0:
                        continue
                    c = all_coords[b] + np.array([ox, oy, oz])
                    neighbor[b, nb_slot(ox, oy, oz)] = find(tuple(int(v) for v in c))
        return BlockMesh(dim=dim, block=(bx, by, bz), level=np.full(n_blocks, level, dtype=np.int32),
                         neighbor=neighbor, coords=all_coords, n_owned=n_owned, grid=gsz, periodic=per,
                         scaling_factor=scaling_factor,
                         outside_src=np.array(out_src, dtype=np.int32),
                         outside_normal=np.array(out_normal, dtype=np.int32).reshape(-1, 3),
                         bricks=tuple(bricks))

    @staticmethod
    def amr(dim: int, refine, bricks=(1, 1, 1), base_level: int = 1, max_level: int = 2, block=(16, 16, 16),
            periodic=(True, True, True), scaling_factor: float = 1.0) -> "BlockMesh":
        """Leaves of a brick forest refined from ``base_level`` up to ``max_level`` where
        ``refine(level, lo, hi)`` is true for the leaf's box [lo, hi) (unit-brick coordinates, 3
        components), then 2:1-balanced across faces, edges and corners (p4est's full balance).

        Neighbour region o of a leaf at level L is: a leaf at L (``neighbor``), part of a leaf at
        L-1 (``neighbor`` = that leaf), split into leaves at L+1 (``neighbor`` = -1 and
        ``fine_neighbor[b, slot]`` = the 2^d children, x fastest), or an outside block at L. Outside
        blocks need a same-level inside leaf across the border (FillOutside.cpp:134-145 looks the
        inside quadrant up at the outside quadrant's level)."""
        f = _Forest(dim, bricks, periodic, base_level, block)
        if not (0 <= base_level <= max_level):
            raise ValueError("need 0 <= base_level <= max_level")
        e0 = f.ext(base_level)
        leaves = {(base_level, cx, cy, cz) for cz in range(e0[2]) for cy in range(e0[1]) for cx in range(e0[0])}
        for L in range(base_level, max_level):
            h = 1.0 / (1 << L)
            for key in sorted(k for k in leaves if k[0] == L):
                lo = np.array([key[1] * h, key[2] * h, key[3] * h if dim == 3 else 0.0])
                hi = lo + np.array([h, h, h if dim == 3 else 1.0])
                if refine(L, lo, hi):
                    leaves.remove(key)
                    leaves.update(f.kids(key))
        return f.native(sorted(leaves), None, base_level, max(max_level, base_level), scaling_factor)[0]

    def leaf_keys(self):
        """int32 [n_owned, 4]: (level, cx, cy, cz) of the owned leaves, in block order."""
        n = self.n_owned
        return np.concatenate([self.level[:n, None].astype(np.int32), self.coords[:n].astype(np.int32)], axis=1)

    def adapt(self, flags, level_min: int, level_max: int):
        """Refine (flag > 0) and coarsen (flag < 0, whole families only) the owned leaves, then
        2:1-balance (refinement wins; a family is not coarsened if balance would refine its parent
        again). Returns (new mesh, remap) with remap[n] for new owned leaf n:
        [kind, s0, ..., s7, f0, ..., f5] where kind 0 keeps old leaf s0, kind 1 is child s1 (x fastest)
        of old leaf s0, kind 2 is the parent of old leaves s0..s(2^d - 1) (x fastest); f0..f5 (kinds 1
        and 2) are the kept old leaves of the same level across the faces -x, +x, -y, +y, -z, +z (-1
        otherwise). Plays p4est's adapt + balance and the reference's AMR cycle
        (SolverGodunovMHD.cpp:263-319)."""
        f = _Forest(self.dim, self.bricks, self.periodic, level_min, self.block)
        return f.native(self.leaf_keys(), np.asarray(flags).reshape(-1), level_min, level_max, self.scaling_factor)

    @staticmethod
    def batch(meshes) -> tuple["BlockMesh", np.ndarray]:
        """Concatenate independent single-problem meshes (same dim and block size) into one block
        list for a batched launch. Returns (mesh, problem id per block). Owned blocks of all problems
        come first, in problem order; outside blocks follow."""
        dims = {m.dim for m in meshes}
        blocks = {tuple(m.block) for m in meshes}
        if len(dims) != 1 or len(blocks) != 1:
            raise ValueError("batched problems must share dim and block size")
        n_owned = sum(m.n_owned for m in meshes)
        own_off, out_off = [], []
        o, q = 0, n_owned
        for m in meshes:
            own_off.append(o)
            out_off.append(q)
            o += m.n_owned
            q += m.n_blocks - m.n_owned
        n_blocks = q

        def remap(m, idx, p):
            idx = np.asarray(idx)
            return np.where(idx < 0, -1, np.where(idx < m.n_owned, idx + own_off[p], idx - m.n_owned + out_off[p]))

        level = np.zeros(n_blocks, np.int32)
        neighbor = -np.ones((n_blocks, 27), np.int32)
        coords = np.zeros((n_blocks, 3), np.int64)
        problem = np.zeros(n_blocks, np.int32)
        out_src, out_normal = [], []
        for p, m in enumerate(meshes):
            own = slice(own_off[p], own_off[p] + m.n_owned)
            out = slice(out_off[p], out_off[p] + m.n_blocks - m.n_owned)
            level[own], level[out] = m.level[: m.n_owned], m.level[m.n_owned:]
            neighbor[own] = remap(m, m.neighbor[: m.n_owned], p)
            neighbor[out] = remap(m, m.neighbor[m.n_owned:], p)
            coords[own], coords[out] = m.coords[: m.n_owned], m.coords[m.n_owned:]
            problem[own] = p
            problem[out] = p
            out_src.append(remap(m, m.outside_src, p))
            out_normal.append(m.outside_normal)
        first = meshes[0]
        bm = BlockMesh(dim=first.dim, block=first.block, level=level, neighbor=neighbor, coords=coords,
                       n_owned=n_owned, grid=first.grid, periodic=first.periodic,
                       scaling_factor=first.scaling_factor,
                       outside_src=np.concatenate(out_src).astype(np.int32) if out_src else np.zeros(0, np.int32),
                       outside_normal=np.concatenate(out_normal).astype(np.int32).reshape(-1, 3))
        return bm, problem

    # ---- layout helpers -------------------------------------------------------------------------
    def state_shapes(self):
        """Shapes of U [n_blocks, 5, bz, by, bx] and B [n_blocks, nface] (C-ABI layout)."""
        bx, by, bz = self.block
        return (self.n_blocks, 5, bz, by, bx), (self.n_blocks, self.nface)

    def alloc_state(self):
        """Zeroed U and B of state_shapes() (FP64)."""
        us, bs = self.state_shapes()
        return np.zeros(us, dtype=np.float64), np.zeros(bs, dtype=np.float64)

    def split_faces(self, B: np.ndarray):
        """Views (Bx, By, Bz) of a face array [n_blocks, nface] with shapes (z, y, x)."""
        bx, by, bz = self.block
        nfx, nfy, nfz = self.face_counts
        Bx = B[:, :nfx].reshape(-1, bz, by, bx + 1)
        By = B[:, nfx:nfx + nfy].reshape(-1, bz, by + 1, bx)
        if self.dim == 3:
            Bz = B[:, nfx + nfy:].reshape(-1, bz + 1, by, bx)
        else:
            Bz = B[:, nfx + nfy:].reshape(-1, bz, by, bx)
        return Bx, By, Bz

    def global_cell_index(self):
        """Global integer (x, y, z) cell coordinates per owned cell, arrays shaped like U[:, 0]."""
        bx, by, bz = self.block
        c = self.coords[: self.n_blocks]
        k, j, i = np.meshgrid(np.arange(bz), np.arange(by), np.arange(bx), indexing="ij")
        gi = c[:, 0, None, None, None] * bx + i[None]
        gj = c[:, 1, None, None, None] * by + j[None]
        gk = c[:, 2, None, None, None] * bz + k[None]
        return gi, gj, gk


class _Forest:
    """Leaf-set helpers of a brick forest (children, periodic wrap); balance and the mesh tables come
    from the native forest of libgmhd.so (gmhd_forest_build)."""

    def __init__(self, dim, bricks, periodic, base_level, block):
        if dim not in (2, 3):
            raise ValueError("dim must be 2 or 3")
        bx, by, bz = block
        if dim == 2:
            bz = 1
            bricks = (bricks[0], bricks[1], 1)
        if min(bx, by) < 4 or (dim == 3 and bz < 4) or bx % 2 or by % 2 or (dim == 3 and bz % 2):
            raise ValueError("block sizes must be even and >= 4 on AMR meshes")
        self.dim, self.bricks, self.base_level, self.block = dim, tuple(bricks), base_level, (bx, by, bz)
        self.per = tuple(bool(p) for p in periodic[:dim]) + (True,) * (3 - dim)
        self.offs = [(ox, oy, oz) for oz in ((-1, 0, 1) if dim == 3 else (0,)) for oy in (-1, 0, 1)
                     for ox in (-1, 0, 1) if (ox, oy, oz) != (0, 0, 0)]

    def ext(self, L):
        b = self.bricks
        return (b[0] << L, b[1] << L, (b[2] << L) if self.dim == 3 else 1)

    def kids(self, key):
        L, cx, cy, cz = key
        return [(L + 1, 2 * cx + ex, 2 * cy + ey, 2 * cz + ez) for ez in ((0, 1) if self.dim == 3 else (0,))
                for ey in (0, 1) for ex in (0, 1)]

    def wrap(self, L, c):
        e = self.ext(L)
        out = []
        for d in range(3):
            v = c[d]
            if self.per[d]:
                v %= e[d]
            elif not 0 <= v < e[d]:
                return None
            out.append(v)
        return tuple(out)

    def native(self, keys, flags, level_min, level_max, scaling_factor):
        """Adapt (flags) or just balance the leaf set with the native forest (gmhd_forest_build) and
        wrap its tables in a BlockMesh. Returns (mesh, remap rows)."""
        from . import _native

        t = _native.forest_build(self.dim, self.bricks, self.per, self.block, level_min, level_max,
                                 np.asarray(keys, dtype=np.int32).reshape(-1, 4), flags)
        no = t["n_owned"]
        lv = t["level"]
        # in a 2:1-balanced leaf set every coarser neighbour sees this leaf's region as finer, so the
        # fine table is present exactly when levels jump
        mesh = BlockMesh(dim=self.dim, block=self.block, level=lv, neighbor=t["neighbor"],
                         coords=t["coord"].astype(np.int64), n_owned=no, grid=self.ext(int(lv[:no].max())),
                         periodic=self.per, scaling_factor=scaling_factor, outside_src=t["outside_src"],
                         outside_normal=t["outside_normal"], fine_list=t["fine_list"],
                         bricks=self.bricks)
        return mesh, t["remap"]

"""Seeded synthetic initial states for the benchmark configurations (host side, numpy).

The reference has no shipped datasets; these generators stand in for its init/ problems with
the shapes, sizes and distributions of the benchmark configurations:

* Orszag-Tang 2D/3D (init/InitOrszagTang.cpp): rho = 25/(36 pi), p = 5/(12 pi),
  v = (-sin 2 pi y, sin 2 pi x, 0); face B is the discrete curl of
  A_z = B0 (cos 4 pi x / (4 pi) + cos 2 pi y / (2 pi)) sampled at edges, B0 = 1/sqrt(4 pi), so the
  discrete divergence is zero to round-off. Optional seeded density perturbation
  rho *= 1 + amp (2U - 1), U from splitmix64(seed, global cell id).
* field loop advection (init/InitFieldLoopAdvection.cpp), magnetic blast (init/InitBlast.cpp).

Every value is computed from global integer cell/face/edge indices, so the copies of a face that
two blocks share are bit-identical.
"""
from __future__ import annotations

import math

import numpy as np

from .mesh import BlockMesh

def splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser (Steele, Lea & Flood 2014) on uint64 arrays, wrapping arithmetic."""
    with np.errstate(over="ignore"):
        z = (x.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform01(seed: int, ids: np.ndarray) -> np.ndarray:
    """Counter-based U[0,1) from (seed, id)."""
    with np.errstate(over="ignore"):
        x = (np.uint64(seed) << np.uint64(40)) ^ ids.astype(np.uint64)
    return (splitmix64(x) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _faces_from_az(mesh: BlockMesh, B: np.ndarray, az, x0=0.0, y0=0.0):
    """Face B = curl(A_z e_z) on the faces of every block; az(x, y) evaluated at edges. Edge
    positions are wrapped on periodic axes, so the two copies of a face shared across a periodic
    border hold the same value (the shared-face agreement SolverGodunovMHD.cpp:506-513 checks)."""
    bx, by, bz = mesh.block
    dxb = mesh.block_dx()
    dx = dxb[:, None, None, None]  # per block (AMR meshes mix levels)
    Bx, By, Bz = mesh.split_faces(B)
    c = mesh.coords
    # cells per axis across the domain at each block's level
    n_x = np.rint(mesh.domain_length(0) / dxb).astype(np.int64)[:, None, None, None]
    n_y = np.rint(mesh.domain_length(1) / dxb).astype(np.int64)[:, None, None, None]

    def wx(g):
        return (np.mod(g, n_x) if mesh.periodic[0] else g).astype(np.float64)

    def wy(g):
        return (np.mod(g, n_y) if mesh.periodic[1] else g).astype(np.float64)

    # x faces: Bx(i, j) = (Az(x_i, y_{j+1}) - Az(x_i, y_j)) / dy
    k, j, i = np.meshgrid(np.arange(bz), np.arange(by), np.arange(bx + 1), indexing="ij")
    gi = c[:, 0, None, None, None] * bx + i[None]
    gj = c[:, 1, None, None, None] * by + j[None]
    Bx[...] = (az(x0 + wx(gi) * dx, y0 + wy(gj + 1) * dx) - az(x0 + wx(gi) * dx, y0 + wy(gj) * dx)) / dx
    # y faces: By(i, j) = -(Az(x_{i+1}, y_j) - Az(x_i, y_j)) / dx
    k, j, i = np.meshgrid(np.arange(bz), np.arange(by + 1), np.arange(bx), indexing="ij")
    gi = c[:, 0, None, None, None] * bx + i[None]
    gj = c[:, 1, None, None, None] * by + j[None]
    By[...] = -(az(x0 + wx(gi + 1) * dx, y0 + wy(gj) * dx) - az(x0 + wx(gi) * dx, y0 + wy(gj) * dx)) / dx
    Bz[...] = 0.0


def _cell_centred_b(mesh: BlockMesh, B: np.ndarray):
    Bx, By, Bz = mesh.split_faces(B)
    bcx = 0.5 * (Bx[..., :-1] + Bx[..., 1:])
    bcy = 0.5 * (By[..., :-1, :] + By[..., 1:, :])
    if mesh.dim == 3:
        bcz = 0.5 * (Bz[:, :-1] + Bz[:, 1:])
    else:
        bcz = Bz
    return bcx, bcy, bcz


def _fill_energy(mesh, U, B, rho, p, vx, vy, vz, gamma):
    bcx, bcy, bcz = _cell_centred_b(mesh, B)
    n = mesh.n_owned
    U[:n, 0] = rho
    U[:n, 2] = rho * vx
    U[:n, 3] = rho * vy
    U[:n, 4] = rho * vz
    U[:n, 1] = p / (gamma - 1.0) + 0.5 * rho * (vx * vx + vy * vy + vz * vz) + 0.5 * (
        bcx[:n] ** 2 + bcy[:n] ** 2 + bcz[:n] ** 2)


def orszag_tang(mesh: BlockMesh, gamma: float = 5.0 / 3.0, rho_perturbation: float = 0.0, seed: int = 0):
    """Orszag-Tang vortex on [0,1]^d (uniform in z in 3D). Returns (U, B)."""
    U, B = mesh.alloc_state()
    B0 = 1.0 / math.sqrt(4.0 * math.pi)
    twopi = 2.0 * math.pi

    def az(x, y):
        return B0 * (np.cos(2.0 * twopi * x) / (2.0 * twopi) + np.cos(twopi * y) / twopi)

    _faces_from_az(mesh, B, az)
    n = mesh.n_owned
    gi, gj, gk = mesh.global_cell_index()
    gi, gj, gk = gi[:n], gj[:n], gk[:n]
    dx = mesh.block_dx()[:n, None, None, None]
    x = (gi + 0.5) * dx
    y = (gj + 0.5) * dx
    rho = np.full(x.shape, 25.0 / (36.0 * math.pi))
    if rho_perturbation:
        if mesh.is_amr:
            raise ValueError("the density perturbation is defined on uniform meshes")
        gx = mesh.grid[0] * mesh.block[0]
        gy = mesh.grid[1] * mesh.block[1]
        ids = gi + gx * (gj + gy * gk)
        rho = rho * (1.0 + rho_perturbation * (2.0 * uniform01(seed, ids) - 1.0))
    p = np.full(x.shape, 5.0 / (12.0 * math.pi))
    vx = -np.sin(twopi * y)
    vy = np.sin(twopi * x)
    vz = np.zeros_like(x)
    _fill_energy(mesh, U, B, rho, p, vx, vy, vz, gamma)
    return U, B


def field_loop(mesh: BlockMesh, gamma=5.0 / 3.0, radius=0.3, speed=1.0, angle=0.0, A0=1e-3,
               x0=-1.0, y0=-0.5):
    """Field-loop advection: rho = 1, p = 1, v = speed (cos a, sin a), A_z = A0 (R - r) for r < R,
    on [x0, x0 + Lx] x [y0, y0 + Ly] (init/InitFieldLoopAdvection.cpp)."""
    U, B = mesh.alloc_state()

    def az(x, y):
        r = np.sqrt(x * x + y * y)
        return np.where(r < radius, A0 * (radius - r), 0.0)

    _faces_from_az(mesh, B, az, x0=x0, y0=y0)
    n = mesh.n_owned
    shape = U[:n, 0].shape
    vx = np.full(shape, speed * math.cos(angle))
    vy = np.full(shape, speed * math.sin(angle))
    _fill_energy(mesh, U, B, np.ones(shape), np.ones(shape), vx, vy, np.zeros(shape), gamma)
    return U, B


def uniform_state(mesh: BlockMesh, gamma=1.4, rho=1.3, p=0.7, v=(0.3, -0.2, 0.1), b=(0.4, -0.25, 0.15)):
    """Exactly uniform state (must be preserved exactly by the scheme)."""
    U, B = mesh.alloc_state()
    Bx, By, Bz = mesh.split_faces(B)
    Bx[...] = b[0]
    By[...] = b[1]
    Bz[...] = b[2]
    n = mesh.n_owned
    shape = U[:n, 0].shape
    vz = v[2]
    _fill_energy(mesh, U, B, np.full(shape, rho), np.full(shape, p), np.full(shape, v[0]),
                 np.full(shape, v[1]), np.full(shape, vz), gamma)
    return U, B


def random_smooth(mesh: BlockMesh, gamma=1.4, seed=0, amp=0.2):
    """Smooth random periodic state (few Fourier modes) with a divergence-free face B."""
    rng = np.random.default_rng(seed)
    U, B = mesh.alloc_state()
    kx, ky = rng.integers(1, 3, 2)
    ph = rng.uniform(0, 2 * math.pi, 6)
    Lx = mesh.domain_length(0)
    Ly = mesh.domain_length(1)

    def az(x, y):
        return 0.1 * (np.sin(2 * math.pi * kx * x / Lx + ph[0]) * np.cos(2 * math.pi * ky * y / Ly + ph[1]))

    _faces_from_az(mesh, B, az)
    Bx, By, Bz = mesh.split_faces(B)
    Bx += 0.3
    By -= 0.2
    n = mesh.n_owned
    gi, gj, gk = mesh.global_cell_index()
    dx = mesh.block_dx()[:n, None, None, None]
    x = (gi[:n] + 0.5) * dx
    y = (gj[:n] + 0.5) * dx
    z = (gk[:n] + 0.5) * dx
    Lz = mesh.domain_length(2)
    if mesh.dim == 3:
        # Bz face values: a constant keeps the field divergence-free
        Bz[...] = 0.15
    else:
        Bz[...] = 0.1
    s = np.sin(2 * math.pi * x / Lx + ph[2]) * np.cos(2 * math.pi * y / Ly + ph[3])
    if mesh.dim == 3:
        s = s * np.cos(2 * math.pi * z / Lz + ph[4])
    rho = 1.0 + amp * s
    p = 1.0 + amp * np.cos(2 * math.pi * x / Lx + ph[4])
    vx = 0.5 * amp * np.sin(2 * math.pi * y / Ly + ph[1])
    vy = 0.5 * amp * np.cos(2 * math.pi * x / Lx + ph[0])
    vz = 0.3 * amp * s if mesh.dim == 3 else 0.2 * amp * s
    _fill_energy(mesh, U, B, rho, p, vx, vy, vz, gamma)
    return U, B


def gaussian01(seed: int, ids: np.ndarray) -> np.ndarray:
    """Counter-based standard normal from (seed, id) (Box-Muller on two splitmix64 uniforms)."""
    u1 = uniform01(seed, 2 * ids)
    u2 = uniform01(seed, 2 * ids + 1)
    return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * math.pi * u2)


def kelvin_helmholtz(mesh: BlockMesh, gamma=1.4, p0=2.5, bx0=0.1, width=0.01, noise=1e-3, seed=0,
                     chunk_blocks: int = 2048):
    """Magnetised shear layer on [0,1]^d (init/InitKelvinHelmholtz.cpp): rho = 2, vx = +0.5 for
    |y - 0.5| < 0.25 and rho = 1, vx = -0.5 outside, tanh-smoothed with `width`; vy = 0.01 sin(4 pi x)
    plus seeded Gaussian noise of amplitude `noise`; p = p0; uniform Bx = bx0. The cells are filled
    `chunk_blocks` blocks at a time, so that the temporaries stay small next to U and B on large meshes."""
    U, B = mesh.alloc_state()
    Bx, By, Bz = mesh.split_faces(B)
    Bx[...] = bx0
    By[...] = 0.0
    Bz[...] = 0.0
    n = mesh.n_owned
    bx, by, bz = mesh.block
    k, j, i = np.meshgrid(np.arange(bz), np.arange(by), np.arange(bx), indexing="ij")
    top = int(mesh.level[:n].max())
    gx = mesh.grid[0] * mesh.block[0]
    gy = mesh.grid[1] * mesh.block[1]
    for b0 in range(0, n, chunk_blocks):
        b1 = min(n, b0 + chunk_blocks)
        c = mesh.coords[b0:b1]
        gi = c[:, 0, None, None, None] * bx + i[None]
        gj = c[:, 1, None, None, None] * by + j[None]
        gk = c[:, 2, None, None, None] * bz + k[None]
        dx = mesh.block_dx()[b0:b1, None, None, None]
        x = (gi + 0.5) * dx
        y = (gj + 0.5) * dx
        s = 0.5 * (1.0 + np.tanh((0.25 - np.abs(y - 0.5)) / width))
        rho = 1.0 + s
        vx = -0.5 + s
        # noise id: the cell's lower corner on the finest level's grid (unique across levels)
        sh = (top - mesh.level[b0:b1]).astype(np.int64)[:, None, None, None]
        ids = (gi << sh) + gx * ((gj << sh) + gy * (gk << sh))
        vy = 0.01 * np.sin(4.0 * math.pi * x) + noise * gaussian01(seed, ids)
        vz = np.zeros_like(x)
        bcx, bcy, bcz = _cell_centred_b(mesh, B[b0:b1])
        U[b0:b1, 0] = rho
        U[b0:b1, 2] = rho * vx
        U[b0:b1, 3] = rho * vy
        U[b0:b1, 4] = rho * vz
        U[b0:b1, 1] = np.full(x.shape, p0) / (gamma - 1.0) + 0.5 * rho * (vx * vx + vy * vy + vz * vz) + 0.5 * (
            bcx ** 2 + bcy ** 2 + bcz ** 2)
    return U, B


def field_loop_batch(n_problems: int, seed: int = 0, sizes=(32, 64, 128, 256), block: int = 16, gamma=5.0 / 3.0):
    """Independent 2D field-loop problems on [-1,1] x [-0.5,0.5] (periodic), each (2N) x N cells in
    block x block leaf blocks (2 x 1 bricks, level log2(N / block)). Per problem, from the seed:
    loop radius R ~ U[0.2, 0.35], speed |v| ~ U[1, 3], direction ~ U[0, 2 pi), and N drawn so that the
    cell count 2N^2 is log-uniform between the smallest and the largest allowed size.
    Returns (meshes, [(U, B)], params) per problem."""
    rng = np.random.default_rng(seed)
    sizes = sorted(sizes)
    lo, hi = np.log(2.0 * sizes[0] ** 2), np.log(2.0 * sizes[-1] ** 2)
    meshes, states, params = [], [], []
    for _ in range(n_problems):
        target = np.exp(rng.uniform(lo, hi))
        n = min(sizes, key=lambda s_: abs(np.log(2.0 * s_ * s_) - np.log(target)))
        level = int(round(np.log2(n // block)))
        radius = float(rng.uniform(0.2, 0.35))
        speed = float(rng.uniform(1.0, 3.0))
        angle = float(rng.uniform(0.0, 2.0 * math.pi))
        mesh = BlockMesh.uniform(2, bricks=(2, 1, 1), level=level, block=(block, block, 1))
        U, B = field_loop(mesh, gamma=gamma, radius=radius, speed=speed, angle=angle)
        meshes.append(mesh)
        states.append((U, B))
        params.append({"N": n, "radius": radius, "speed": speed, "angle": angle})
    return meshes, states, params


# ---- coarse/fine (AMR) workloads -------------------------------------------------------------
def refine_band(center, r_lo, r_hi, axes=2):
    """Refinement predicate for BlockMesh.amr: leaves whose box meets the shell r_lo <= |x - c| <= r_hi
    (distance over the first `axes` coordinates, unit-brick coordinates)."""
    c = np.asarray(center, dtype=np.float64)

    def f(level, lo, hi):
        p = np.clip(c, lo, hi)
        near = float(np.sqrt(((p - c)[:axes] ** 2).sum()))
        far = float(np.sqrt((np.maximum(np.abs(lo - c), np.abs(hi - c))[:axes] ** 2).sum()))
        return near <= r_hi and far >= r_lo

    return f


def blast_mesh(base_level: int = 5, max_level: int = 9, block: int = 16, radius: float = 0.1,
               band: float = 0.02) -> BlockMesh:
    """2D magnetised blast mesh on [-0.5, 0.5]^2 (periodic): leaves within `band` of the initial
    front r = radius refined to max_level, 2:1 balanced (the shape of app/test_mhd_blast_2d.ini with
    levels 5-10; the mesh is static here)."""
    return BlockMesh.amr(2, refine_band((0.5, 0.5, 0.5), radius - band, radius + band), base_level=base_level,
                         max_level=max_level, block=(block, block, 1))


def blast(mesh: BlockMesh, gamma=5.0 / 3.0, radius=0.1, p_in=10.0, p_out=0.1, x0=-0.5, y0=-0.5):
    """rho = 1, p = p_in for r < radius else p_out, v = 0, B = (1/sqrt 2, 1/sqrt 2, 0)
    (init/InitBlast, MHD variant with a uniform oblique field)."""
    U, B = mesh.alloc_state()
    Bx, By, Bz = mesh.split_faces(B)
    b0 = 1.0 / math.sqrt(2.0)
    Bx[...] = b0
    By[...] = b0
    Bz[...] = 0.0
    n = mesh.n_owned
    gi, gj, _ = mesh.global_cell_index()
    dx = mesh.block_dx()[:n, None, None, None]
    x = x0 + (gi[:n] + 0.5) * dx
    y = y0 + (gj[:n] + 0.5) * dx
    r = np.sqrt(x * x + y * y)
    p = np.where(r < radius, p_in, p_out)
    z = np.zeros_like(x)
    _fill_energy(mesh, U, B, np.ones_like(x), p, z, z, z, gamma)
    return U, B


def kh_amr_mesh(base_level: int = 5, max_level: int = 7, block: int = 16, band: float = 0.02) -> BlockMesh:
    """3D shear-layer mesh on [0,1]^3, periodic in x and z, reflecting in y: leaves within `band` of
    the layers |y - 0.5| = 0.25 refined to max_level (the shape of the 3D Kelvin-Helmholtz
    configuration with levels 6-9; the mesh is static here)."""
    def refine(level, lo, hi):
        return any(lo[1] - band <= yl <= hi[1] + band for yl in (0.25, 0.75))

    return BlockMesh.amr(3, refine, base_level=base_level, max_level=max_level, block=(block, block, block),
                         periodic=(True, False, True))

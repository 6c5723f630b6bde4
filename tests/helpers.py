"""Shared helpers for the parity tests: workloads on both paths, error metrics."""
from __future__ import annotations

import numpy as np

from godunov_mhd_ct_gb300.mesh import BlockMesh
from godunov_mhd_ct_gb300.settings import MHDSettings


def settings(gamma0=5.0 / 3.0, cfl=0.5, slope_type=2.0, riemann="HLLD"):
    return MHDSettings(gamma0=gamma0, cfl=cfl, slope_type=slope_type, riemann=riemann)


def oracle_mesh(orc, mesh: BlockMesh, bc=None):
    if bc is None:
        bc = [1 if mesh.periodic[f // 2] else 2 for f in range(6)]
    return orc.Mesh(mesh.dim, mesh.block[0], mesh.block[1], mesh.block[2], mesh.level, mesh.neighbor,
                    mesh.n_owned, mesh.scaling_factor, mesh.outside_src, mesh.outside_normal, bc)


def oracle_settings(orc, st: MHDSettings):
    return orc.settings(gamma0=st.gamma0, cfl=st.cfl, slope_type=st.slope_type, smallr=st.smallr,
                        smallc=st.smallc, riemann=st.riemann_id,
                        time_integrator=1 if st.time_integrator.upper() == "RK2_SSP" else 0,
                        gravity=st.gravity, viscosity_mu=st.viscosity_mu, viscous_predictor=st.viscous_predictor)


def max_rel_diff(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.maximum(np.abs(b), 1e-300)
    return float(np.max(np.abs(a - b) / np.maximum(scale, np.max(np.abs(b)) * 1e-12)))


def l1_rel(a, b):
    return float(np.sum(np.abs(np.asarray(a) - np.asarray(b))) / np.sum(np.abs(np.asarray(b))))


def div_b(mesh: BlockMesh, B):
    """Discrete divergence per owned cell, (sum of face differences) / dx."""
    Bx, By, Bz = mesh.split_faces(np.asarray(B))
    n = mesh.n_owned
    d = (Bx[:n, ..., 1:] - Bx[:n, ..., :-1]) + (By[:n, :, 1:, :] - By[:n, :, :-1, :])
    if mesh.dim == 3:
        d = d + (Bz[:n, 1:] - Bz[:n, :-1])
    return d / mesh.cell_length()


def shared_face_mismatch(mesh: BlockMesh, B):
    """Max |difference| between the two copies of every face shared by neighbouring blocks."""
    from godunov_mhd_ct_gb300.mesh import nb_slot

    Bx, By, Bz = mesh.split_faces(np.asarray(B))
    worst = 0.0
    n = mesh.n_owned
    right_x = mesh.neighbor[:n, nb_slot(1, 0, 0)]
    right_y = mesh.neighbor[:n, nb_slot(0, 1, 0)]
    ok = right_x >= 0
    worst = max(worst, float(np.max(np.abs(Bx[:n][ok, ..., -1] - Bx[right_x[ok], ..., 0]), initial=0.0)))
    ok = right_y >= 0
    worst = max(worst, float(np.max(np.abs(By[:n][ok, :, -1, :] - By[right_y[ok], :, 0, :]), initial=0.0)))
    if mesh.dim == 3:
        right_z = mesh.neighbor[:n, nb_slot(0, 0, 1)]
        ok = right_z >= 0
        worst = max(worst, float(np.max(np.abs(Bz[:n][ok, -1] - Bz[right_z[ok], 0]), initial=0.0)))
    return worst


def same_level_face_mismatch(mesh: BlockMesh, B):
    """Max |difference| between the two copies of faces shared by same-level neighbours (AMR meshes
    included; coarse/fine borders are skipped)."""
    from godunov_mhd_ct_gb300.mesh import nb_slot

    faces = mesh.split_faces(np.asarray(B))
    n = mesh.n_owned
    worst = 0.0
    for d in range(mesh.dim):
        o = [0, 0, 0]
        o[d] = 1
        right = mesh.neighbor[:n, nb_slot(*o)]
        ok = (right >= 0) & (right < n)
        ok[ok] &= mesh.level[right[ok]] == mesh.level[:n][ok]
        if not ok.any():
            continue
        F = faces[d]
        a = np.take(F[:n][ok], -1, axis=3 - d)
        b = np.take(F[right[ok]], 0, axis=3 - d)
        worst = max(worst, float(np.max(np.abs(a - b))))
    return worst


def div_b_per_block(mesh: BlockMesh, B):
    """Discrete divergence per owned cell with each block's own cell length (AMR meshes)."""
    Bx, By, Bz = mesh.split_faces(np.asarray(B))
    n = mesh.n_owned
    d = (Bx[:n, ..., 1:] - Bx[:n, ..., :-1]) + (By[:n, :, 1:, :] - By[:n, :, :-1, :])
    if mesh.dim == 3:
        d = d + (Bz[:n, 1:] - Bz[:n, :-1])
    return d / mesh.block_dx()[:n, None, None, None]


def totals(mesh: BlockMesh, U):
    """Volume integrals of rho and E over the owned blocks (cell volume dx^d per block)."""
    n = mesh.n_owned
    vol = mesh.block_dx()[:n] ** mesh.dim
    U = np.asarray(U)
    return float((U[:n, 0].reshape(n, -1).sum(axis=1) * vol).sum()), float((U[:n, 1].reshape(n, -1).sum(axis=1) * vol).sum())


def accuracy_block(mesh0: BlockMesh, U0, mesh: BlockMesh, U, B, Uref, Bref):
    """The per-result report: L1 relative error of rho, E and face B against (Uref, Bref) on the same
    mesh, max |div B| of (U, B), and the relative drift of the rho and E integrals from the initial
    state (mesh0, U0)."""
    n = mesh.n_owned
    U, B, Uref, Bref = (np.asarray(x) for x in (U, B, Uref, Bref))
    m0, e0 = totals(mesh0, U0)
    m1, e1 = totals(mesh, U)
    return {"l1_rho": l1_rel(U[:n, 0], Uref[:n, 0]), "l1_E": l1_rel(U[:n, 1], Uref[:n, 1]),
            "l1_B": l1_rel(B[:n], Bref[:n]), "max_divB": float(np.max(np.abs(div_b_per_block(mesh, B)))),
            "mass_drift": abs(m1 - m0) / abs(m0), "energy_drift": abs(e1 - e0) / abs(e0)}


def record(name, **values):
    """Append a result line (JSON) to the file named by GMHD_RESULTS_LOG, when set, and print it."""
    import json
    import os

    line = json.dumps({"case": name, **values}, default=float)
    print(line)
    path = os.environ.get("GMHD_RESULTS_LOG")
    if path:
        with open(path, "a") as f:
            f.write(line + "\n")

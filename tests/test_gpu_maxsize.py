"""Largest meshes: block offsets past 2^31 doubles.

1024^3 cells in 32768 blocks of 32^3 put the face array B (3.3e9 doubles) and the state U (5.4e9)
beyond 32-bit element offsets; U, B, U2, B2 take 139 GB of device memory. The state is built on the
device (exactly uniform), one step of the mixed path must keep it bit for bit, and the CFL
reduction must return the uniform state's value. The FP64 path is checked the same way on 768^3
(27 bricks of 8^3 blocks; U holds 2.3e9 doubles).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_mhd_ct_gb300.mesh import BlockMesh  # noqa: E402
from godunov_mhd_ct_gb300.solver import GodunovImplemGB300  # noqa: E402

from .helpers import settings  # noqa: E402

pytestmark = pytest.mark.gpu

RHO, P, V, BF = 1.3, 0.7, (0.3, -0.2, 0.1), (0.4, -0.25, 0.15)


def _uniform_device_state(mesh, gamma):
    """U [n][5][cells] and B [n][faces] of an exactly uniform state, filled on the device."""
    n, ncell = mesh.n_blocks, mesh.ncell
    nfx, nfy, _ = mesh.face_counts
    e = P / (gamma - 1.0) + 0.5 * RHO * sum(v * v for v in V) + 0.5 * sum(b * b for b in BF)
    U = torch.empty((n, 5, ncell), dtype=torch.float64, device="cuda")
    for var, val in enumerate((RHO, e, RHO * V[0], RHO * V[1], RHO * V[2])):
        U[:, var].fill_(val)
    B = torch.empty((n, mesh.nface), dtype=torch.float64, device="cuda")
    B[:, :nfx].fill_(BF[0])
    B[:, nfx:nfx + nfy].fill_(BF[1])
    B[:, nfx + nfy:].fill_(BF[2])
    return U, B


def _need(bytes_):
    free = torch.cuda.mem_get_info()[0]
    if free < bytes_:
        pytest.skip(f"needs {bytes_ / 1e9:.0f} GB of free device memory, {free / 1e9:.0f} GB free")


def _expected_inv_dt(mesh, gamma):
    """max over directions of (fast speed + |v|) / dx summed over axes, for the uniform state."""
    b2 = sum(b * b for b in BF)
    c2 = gamma * P / RHO
    d2 = 0.5 * (b2 / RHO + c2)
    dx = mesh.cell_length()
    return sum((np.sqrt(d2 + np.sqrt(d2 * d2 - c2 * bn * bn / RHO)) + abs(v)) / dx for bn, v in zip(BF, V))


@pytest.mark.parametrize("precision,bricks,level", [("mixed", (1, 1, 1), 5), ("fp64", (3, 3, 3), 3)])
def test_uniform_state_preserved_past_32bit_offsets(precision, bricks, level):
    mesh = BlockMesh.uniform(3, bricks=bricks, level=level, block=(32, 32, 32))
    words = mesh.n_blocks * (5 * mesh.ncell + mesh.nface)
    assert words > 2 ** 31
    _need(2 * 8 * words + 8e9)
    st = settings()
    U, B = _uniform_device_state(mesh, st.gamma0)
    U2, B2 = U.clone(), B.clone()
    impl = GodunovImplemGB300(st, mesh, precision=precision)
    inv_dt = impl.compute_inv_dt(U, B)
    assert inv_dt == pytest.approx(_expected_inv_dt(mesh, st.gamma0), rel=1e-5 if precision == "mixed" else 1e-12)
    impl.do_time_step(U, U2, B, B2, st.cfl / inv_dt)
    torch.cuda.synchronize()
    assert impl.last_status() & ~16 == 0
    assert torch.equal(U2, U)
    assert torch.equal(B2, B)
    impl.close()

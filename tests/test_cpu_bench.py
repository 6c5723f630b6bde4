"""bench.py host logic without a GPU: the committed counters parse, the configuration legs are
registered, a failing leg is reported without hiding the others, and the accuracy block of a leg
(L1, div B, drift) reads zero for identical states and sees a change."""
import importlib.util
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(__file__))
_spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
bench = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(bench)


def test_counters_parse():
    c = bench.read_counters()
    assert c is not None
    assert 50 < c["dram_bytes_per_cell"] < 400 and 50 < c["warp_inst_per_cell"] < 1000


def test_legs_registered():
    assert set(bench.LEGS) == {"0", "1", "2", "3", "4"}


def test_failing_leg_is_reported(monkeypatch):
    def boom(**_):
        raise RuntimeError("no device")

    monkeypatch.setitem(bench.LEGS, "0", boom)
    out = bench.run_legs("0")
    assert out["config0"]["error"].startswith("RuntimeError") and "leg_seconds" in out["config0"]


def test_accuracy_block():
    from godunov_mhd_ct_gb300 import workloads as wl
    from godunov_mhd_ct_gb300.mesh import BlockMesh

    mesh = BlockMesh.uniform(2, level=2, block=(8, 8, 1))
    U, B = wl.orszag_tang(mesh, gamma=5.0 / 3.0)
    acc = bench._accuracy(mesh, U, mesh, U, B, U, B)
    assert acc["l1_rho"] == 0.0 and acc["mass_drift"] == 0.0 and acc["max_divB"] < 1e-12
    U2 = U.copy()
    U2[:, 0] *= 1.0 + 1e-6
    acc = bench._accuracy(mesh, U, mesh, U2, B, U, B)
    assert np.isclose(acc["l1_rho"], 1e-6, rtol=1e-3) and np.isclose(acc["mass_drift"], 1e-6, rtol=1e-3)

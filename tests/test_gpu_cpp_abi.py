"""The C ABI from a C++ program (tests/cpp/abi_demo.cpp), without Python or torch in the caller: forest
tables, gmhd_set_mesh, gmhd_advance on the FP64 and the mixed path, health flags; the program checks mass
conservation, div B at round-off and the mixed path within 1e-6 (L1) of FP64."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_caller_through_the_c_abi(tmp_path):
    from godunov_mhd_ct_gb300.csrc import build as cbuild

    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    libdir = os.path.dirname(cbuild.LIB)
    exe = str(tmp_path / "abi_demo")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "abi_demo.cpp"), "-L", libdir, "-lgmhd",
                        "-Xlinker", f"-rpath,{libdir}", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "abi_demo:" in r.stdout

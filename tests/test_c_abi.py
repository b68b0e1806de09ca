"""The library through its C ABI from a plain C program (no Python between):
compiled with gcc against include/ffe.h and libffe_gb300.so.  The program's
three fused-exact steps on a 16x12x8 FP32 grid must equal the golden fixture
cabi_fp32_periodic (the oracle's output from the same inputs) bit for bit."""
import os
import subprocess

import numpy as np
import pytest

import ffe
from conftest import ROOT


def build_c(tmp_path):
    exe = str(tmp_path / "abi_roundtrip")
    libdir = os.path.dirname(ffe.LIB_PATH)
    cmd = ["gcc", "-O2", "-std=c11", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c", "abi_roundtrip.c"), "-o", exe, "-L", libdir, "-lffe_gb300",
           "-Wl,-rpath," + libdir, "-lm"]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def test_c_program_compiles_and_links(tmp_path):
    import build as ffe_build
    ffe_build.build()
    assert os.path.exists(build_c(tmp_path))


@pytest.mark.gpu
def test_c_program_runs(tmp_path):
    import build as ffe_build
    ffe_build.build()
    raw = str(tmp_path / "cabi_out.bin")
    r = subprocess.run([build_c(tmp_path), raw], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "c abi ok" in r.stdout
    z = np.load(os.path.join(ROOT, "tests", "golden", "cabi_fp32_periodic.npz"))
    shp = z["out_ex"].shape
    got = np.fromfile(raw, dtype=np.float32).reshape((6,) + shp)
    for c, n in enumerate(("ex", "ey", "ez", "bx", "by", "bz")):
        want = z["out_" + n]
        assert np.array_equal(got[c], want), (n, float(np.max(np.abs(got[c].astype(float) - want))))

"""The library through its C ABI from a plain C program (no Python between):
compiled with gcc against include/ffe.h and libffe_gb300.so."""
import os
import subprocess

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
    r = subprocess.run([build_c(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "c abi ok" in r.stdout

"""The C++ drop-in header: programs written against the reference's
ski-lls.h compile, link and (on a GPU) solve through libskills_gb300.so."""
import os
import re
import subprocess

import numpy as np
import pytest

import skills_gb300 as skl
from conftest import ROOT

# the reference's example programs, when its source tree is named
REF = os.environ.get("SKILLS_REF_DIR")
LIBDIR = os.path.dirname(skl.LIB_PATH)


def _build(src, out):
    if not os.path.exists(skl.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           "-I", "/usr/local/cuda/include", src, "-o", out, "-L", LIBDIR, "-lskills_gb300",
           "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return out


@pytest.mark.parametrize("name", ["ski-llsDenseExample.cpp", "ski-llsSparseExample.cpp"])
def test_reference_examples_compile_unchanged(tmp_path, name):
    if not REF:
        pytest.skip("SKILLS_REF_DIR (the reference source tree) is not set")
    src = os.path.join(REF, "test", name)
    if not os.path.exists(src):
        pytest.skip("reference example not found under SKILLS_REF_DIR")
    _build(src, str(tmp_path / "ex"))


@pytest.mark.parametrize("name", ["dense_drop_in.cpp", "sparse_drop_in.cpp"])
def test_drop_in_programs_compile(tmp_path, name):
    _build(os.path.join(ROOT, "tests", "cpp", name), str(tmp_path / "prog"))


@pytest.mark.gpu
def test_drop_in_programs_run(tmp_path, fixtures):
    exe = _build(os.path.join(ROOT, "tests", "cpp", "dense_drop_in.cpp"), str(tmp_path / "d"))
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    line = [ln for ln in out.stdout.splitlines() if ln.startswith("x ")][0]
    x = np.array([float(v) for v in line.split()[1:3]])
    np.testing.assert_allclose(x, fixtures["dense_example/x_expected"], atol=5e-5)
    line2 = [ln for ln in out.stdout.splitlines() if ln.startswith("x2 ")][0]
    np.testing.assert_allclose(np.array([float(v) for v in line2.split()[1:3]]),
                               fixtures["dense_example/x_expected"], atol=5e-5)
    line3 = [ln for ln in out.stdout.splitlines() if ln.startswith("x3 ")][0]
    np.testing.assert_allclose(np.array([float(v) for v in line3.split()[1:3]]),
                               fixtures["dense_example/x_expected"], atol=5e-5)
    assert line3.split()[4] == "2"   # rank = n
    exe = _build(os.path.join(ROOT, "tests", "cpp", "sparse_drop_in.cpp"), str(tmp_path / "s"))
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    line = [ln for ln in out.stdout.splitlines() if ln.startswith("x ")][0]
    x = np.array([float(v) for v in line.split()[1:4]])
    np.testing.assert_allclose(x, fixtures["sparse_example/x_expected"], atol=5e-5)
    assert "error-path: Matrix is not overdetermined." in out.stdout

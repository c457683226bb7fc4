"""Command-line drivers (ski-lls_gb300/cli): the equivalents of the
reference's test/ls_qr.cpp and test/ls_blendenpik_hashing.cpp, run the way
test/test_solvers.sh runs its solvers (MatrixMarket input, b = ones, the
"Residual of ... is:" line), with the script's expected residuals asserted."""
import os
import re
import subprocess

import numpy as np
import pytest
import scipy.io
import scipy.sparse as sp

from conftest import RANK_DEF_NAMES, FULL_RANK_TAGS, fixture_csc, residual_matches

import build_lib

HAVE_LIB = os.path.exists(build_lib.LIB)


@pytest.fixture(scope="module")
def tools():
    if not HAVE_LIB:
        pytest.skip("library not built")
    return dict(zip(build_lib.CLI_TOOLS, build_lib.build_cli()))


def _residual(out, solver):
    m = re.search(r"Residual of %s is: ([-+0-9.eE]+)" % solver, out)
    assert m, out[-500:]
    return float(m.group(1))


def test_cli_usage_and_bad_input(tools, tmp_path):
    r = subprocess.run([tools["ls_qr"]], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    bad = tmp_path / "bad.mtx"
    bad.write_text("%%MatrixMarket matrix coordinate real general\n3 2 4\n1 1 1.0\n")
    r = subprocess.run([tools["ls_qr"], str(bad)], capture_output=True, text=True)
    assert r.returncode == 1 and "truncated" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", RANK_DEF_NAMES)
def test_ls_qr_rank_deficient_residuals(tools, fixtures, tmp_path, name):
    n, d, p, i, x = fixture_csc(fixtures, name)
    path = tmp_path / (name + ".mtx")
    scipy.io.mmwrite(str(path), sp.csc_matrix((x, i, p), shape=(n, d)))
    r = subprocess.run([tools["ls_qr"], str(path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    res = _residual(r.stdout, "ls_sparse_spqr")
    assert residual_matches(res, float(fixtures[name + "/expected_residual"])), res


@pytest.mark.gpu
@pytest.mark.parametrize("tag", FULL_RANK_TAGS)
def test_ls_blendenpik_hashing_full_rank_dense(tools, fixtures, tmp_path, tag):
    A = np.asarray(fixtures[f"{tag}DenseFullRank/dense"], dtype=np.float64)
    n = A.shape[0]
    path = tmp_path / (tag + ".mtx")
    scipy.io.mmwrite(str(path), A)   # array format
    r = subprocess.run([tools["ls_blendenpik_hashing"], str(path)], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    res = _residual(r.stdout, "ls_blendenpik_hashing")
    b = np.ones(n)
    ref = np.linalg.norm(A @ np.linalg.lstsq(A, b, rcond=None)[0] - b)
    assert abs(res - ref) <= 1e-6 * ref, (res, ref)

"""Command-line drivers (ski-lls_gb300/cli): the equivalents of the
reference's test/ls_qr.cpp, test/ls_blendenpik_hashing.cpp and
test/ls_blendenpik.cpp, run the way
test/test_solvers.sh runs its solvers (MatrixMarket input, b = ones, the
"Residual of ... is:" line), with the script's expected residuals asserted."""
import os
import re
import subprocess
import warnings

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


@pytest.mark.gpu
@pytest.mark.parametrize("tag", FULL_RANK_TAGS)
def test_ls_blendenpik_full_rank_dense(tools, fixtures, tmp_path, tag):
    # test/test_solvers.sh runs ls_blendenpik on the same six dense fixtures
    A = np.asarray(fixtures[f"{tag}DenseFullRank/dense"], dtype=np.float64)
    n = A.shape[0]
    path = tmp_path / (tag + ".mtx")
    scipy.io.mmwrite(str(path), A)
    r = subprocess.run([tools["ls_blendenpik"], str(path)], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    res = _residual(r.stdout, "ls_blendenpik")
    b = np.ones(n)
    ref = np.linalg.norm(A @ np.linalg.lstsq(A, b, rcond=None)[0] - b)
    assert abs(res - ref) <= 1e-6 * ref, (res, ref)


_MM_HARNESS = r"""
#include <cstdio>
#include "mm_read.hpp"
int main(int argc, char** argv)
{
    try {
        MMMatrix A = mm_read(argv[1]);
        if (argc > 2) A = mm_transpose(A);
        std::printf("%lld %lld %d\n", (long long)A.m, (long long)A.n, A.dense ? 1 : 0);
        for (int64_t v : A.p) std::printf("%lld ", (long long)v);
        std::printf("\n");
        for (int64_t v : A.i) std::printf("%lld ", (long long)v);
        std::printf("\n");
        for (double v : A.x) std::printf("%.17g ", v);
        std::printf("\n");
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def mm_harness(tmp_path_factory):
    d = tmp_path_factory.mktemp("mm")
    src = d / "mm.cpp"
    src.write_text(_MM_HARNESS)
    exe = d / "mm"
    cli = os.path.join(os.path.dirname(build_lib.__file__), "cli")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", cli, str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(exe)


def _read_with(exe, path, transpose=False):
    r = subprocess.run([exe, str(path)] + (["t"] if transpose else []), capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    head, p, i, x = r.stdout.split("\n")[:4]
    m, n, dense = (int(v) for v in head.split())
    x = np.array([float(v) for v in x.split()])
    if dense:
        return np.asarray(x.reshape((n, m)).T)
    return sp.csc_matrix((x, [int(v) for v in i.split()], [int(v) for v in p.split()]),
                         shape=(m, n))


@pytest.mark.parametrize("header,body,shape", [
    ("coordinate real general", "4 3 5\n1 1 1.5\n3 1 -2\n2 3 4e-3\n4 2 7\n3 1 0.5\n", (4, 3)),
    ("coordinate integer general", "3 2 3\n1 2 5\n3 1 -1\n2 2 2\n", (3, 2)),
    ("coordinate pattern general", "3 3 4\n1 1\n2 3\n3 2\n1 3\n", (3, 3)),
    ("coordinate real symmetric", "3 3 4\n1 1 2.0\n2 1 -1.0\n3 2 0.25\n3 3 4.0\n", (3, 3)),
    ("coordinate real skew-symmetric", "3 3 2\n2 1 1.5\n3 1 -2.0\n", (3, 3)),
    ("array real general", "3 2\n1.0\n2.0\n3.0\n-4.0\n5.5\n6e-2\n", (3, 2)),
])
def test_matrix_market_reader_matches_scipy(mm_harness, tmp_path, header, body, shape):
    """ski-lls_gb300/cli/mm_read.hpp (the drivers' reader, standing in for the
    reference's cholmod_l_read_matrix) against scipy.io.mmread; duplicates summed."""
    path = tmp_path / "a.mtx"
    path.write_text("%%MatrixMarket matrix " + header + "\n% a comment\n" + body)
    with warnings.catch_warnings():   # scipy's changing sparse-return default
        warnings.simplefilter("ignore", DeprecationWarning)
        ref = scipy.io.mmread(str(path))
    ref = ref.toarray() if sp.issparse(ref) else np.asarray(ref)
    got = _read_with(mm_harness, path)
    got = got.toarray() if sp.issparse(got) else got
    assert got.shape == shape
    np.testing.assert_array_equal(got, ref)
    if "coordinate" in header:
        gt = _read_with(mm_harness, path, transpose=True)
        assert gt.has_sorted_indices
        np.testing.assert_array_equal(gt.toarray(), ref.T)


def test_matrix_market_reader_reads_the_reference_fixtures(mm_harness, fixtures, tmp_path):
    for name in ("lp_ship12l", "Franz1"):
        n, d, p, i, x = fixture_csc(fixtures, name)
        A = sp.csc_matrix((x, i, p), shape=(n, d))
        path = tmp_path / (name + ".mtx")
        scipy.io.mmwrite(str(path), A)
        got = _read_with(mm_harness, path)
        assert got.shape == A.shape and (got != A).nnz == 0

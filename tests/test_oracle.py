"""The CPU oracle pinned against the reference's golden data (no GPU)."""
import ctypes
import math

import numpy as np
import pytest
import scipy.sparse as sp

import ski_lls_oracle as orc
from conftest import RANK_DEF_NAMES, FULL_RANK_TAGS, fixture_csc, residual_matches, GOLDEN


def test_rng_matches_committed_glibc_stream():
    z = np.load(f"{GOLDEN}/rand_glibc.npz")
    for s in z["seeds"]:
        got = orc.Rng(int(s)).fill(1000)
        np.testing.assert_array_equal(got, z[f"seed_{int(s)}"])


def test_rng_matches_live_libc():
    try:
        libc = ctypes.CDLL("libc.so.6")
    except OSError:
        pytest.skip("no glibc")
    for s in (1, 7, 12, 123456789):
        libc.srand(ctypes.c_uint(s))
        want = [libc.rand() for _ in range(500)]
        assert list(orc.Rng(s).fill(500)) == want


def test_hashing_matches_golden():
    z = np.load(f"{GOLDEN}/hashing.npz")
    from make_golden import CASES  # noqa: E402  (tests/golden is on sys.path below)
    for (m, n, k) in CASES:
        rows, vals = orc.gen_hashing(orc.Rng(1), m, n, k)
        np.testing.assert_array_equal(rows, z[f"{m}_{n}_{k}/rows"])
        np.testing.assert_array_equal((vals > 0).astype(np.uint8), z[f"{m}_{n}_{k}/signs"])
        assert np.all(np.abs(np.abs(vals) - 1 / math.sqrt(k)) == 0)
        r = rows.reshape(n, k)
        assert all(len(set(row)) == k for row in r)   # distinct rows per column of S
        assert r.min() >= 0 and r.max() < m


def test_sparse_sketch_matches_dense_product():
    rng = np.random.default_rng(3)
    n, d, m, k = 300, 20, 34, 2
    A = sp.random(n, d, density=0.1, random_state=4, format="csc")
    A.sort_indices()
    b = rng.standard_normal(n)
    rows, vals = orc.gen_hashing(orc.Rng(1), m, n, k)
    S = sp.csc_matrix((vals, rows, np.arange(0, n * k + 1, k)), shape=(m, n))
    SA, Sb = orc.sparse_sketch(n, d, A.indptr, A.indices, A.data, b, m, k, rows, vals)
    np.testing.assert_allclose(SA, (S @ A).toarray(), rtol=1e-14, atol=1e-14)
    np.testing.assert_allclose(Sb, S @ b, rtol=1e-14, atol=1e-14)


def test_dht_is_orthonormal_and_involutive():
    rng = np.random.default_rng(0)
    for N in (7, 40, 125, 1000):
        x = rng.standard_normal((N, 3))
        D = np.ones(N)
        y = orc.unitary_dht(x, D)
        np.testing.assert_allclose(np.linalg.norm(y, axis=0), np.linalg.norm(x, axis=0), rtol=1e-12)
        np.testing.assert_allclose(orc.unitary_dht(y, D), x, atol=1e-12)


def test_dht_matches_the_cas_definition_with_signs_and_padding():
    """FFTW's DHT kind (src/fftw_r2r.cpp:45-51) is Y_k = sum_j X_j cas(2 pi j k / N),
    cas = cos + sin; the reference scales by 1/sqrt(N) and zero-pads to N
    (src/fast_unitary_transform.cpp:63-64, :79, :98-99)."""
    rng = np.random.default_rng(11)
    for n, N in ((6, 6), (7, 7), (10, 16), (30, 42)):
        x = rng.standard_normal((n, 2))
        D = rng.choice([-1.0, 1.0], size=n)
        jk = np.outer(np.arange(N), np.arange(n)) * (2 * np.pi / N)
        H = (np.cos(jk) + np.sin(jk)) / np.sqrt(N)
        np.testing.assert_allclose(orc.unitary_dht(x, D, N), H @ (D[:, None] * x), atol=1e-12)
        if N == n:
            np.testing.assert_allclose(orc.dht_unscaled(x), np.sqrt(N) * H @ x, atol=1e-12)


def test_dense_example_known_answer(fixtures):
    A = fixtures["dense_example/A"]
    b = fixtures["dense_example/b"]
    for seed in (1, 2, 3):
        out = orc.ls_dense_hashing_blendenpik(A, b, 1.1, 3, seed=seed)
        np.testing.assert_allclose(out["x"], fixtures["dense_example/x_expected"], atol=5e-5)


def test_sparse_example_known_answer(fixtures):
    p, i, x = (fixtures[f"sparse_example/{k}"] for k in ("indptr", "indices", "data"))
    out = orc.ls_sparse_spqr(4, 3, p, i, x, fixtures["sparse_example/b"], 1.1, 3)
    np.testing.assert_allclose(out["x"], fixtures["sparse_example/x_expected"], atol=5e-5)


@pytest.mark.parametrize("name", RANK_DEF_NAMES)
def test_rank_deficient_residuals(fixtures, name):
    n, d, p, i, x = fixture_csc(fixtures, name)
    b = np.ones(n)
    out = orc.ls_sparse_spqr(n, d, p, i, x, b, 1.4, 2)
    res = float(np.linalg.norm(orc.csc_residual(n, d, p, i, x, out["x"], b)))
    assert residual_matches(res, float(fixtures[name + "/expected_residual"])), res


@pytest.mark.parametrize("tag", FULL_RANK_TAGS)
def test_full_rank_fixtures_vs_lstsq(fixtures, tag):
    Ad = fixtures[f"{tag}DenseFullRank/dense"]
    b = np.ones(Ad.shape[0])
    xr = np.linalg.lstsq(Ad, b, rcond=None)[0]
    out = orc.ls_dense_hashing_blendenpik(Ad, b, 1.7, 1, it_tol=1e-12, seed=5)
    assert np.linalg.norm(out["x"] - xr) <= 1e-8 * np.linalg.norm(xr)
    n, d, p, i, x = fixture_csc(fixtures, f"{tag}SparseFullRank")
    As = sp.csc_matrix((x, i, p), shape=(n, d)).toarray()
    xr = np.linalg.lstsq(As, b, rcond=None)[0]
    out = orc.ls_sparse_spqr(n, d, p, i, x, b, 1.4, 2, it_tol=1e-12)
    assert np.linalg.norm(out["x"] - xr) <= 1e-8 * np.linalg.norm(xr)


@pytest.mark.parametrize("tag", FULL_RANK_TAGS)
def test_noCPQR_full_rank_fixtures_vs_lstsq(fixtures, tag):
    """The _noCPQR restatement (unpivoted QR of the sketch, LSQR from zero) on
    the reference's dense full-rank fixtures, against LAPACK least squares."""
    Ad = fixtures[f"{tag}DenseFullRank/dense"]
    b = np.ones(Ad.shape[0])
    xr = np.linalg.lstsq(Ad, b, rcond=None)[0]
    out = orc.ls_dense_hashing_blendenpik_noCPQR(Ad, b, 1.7, 1, it_tol=1e-12, seed=5)
    assert out["rank"] == Ad.shape[1] and out["flag"] == 0
    assert np.linalg.norm(out["x"] - xr) <= 1e-8 * np.linalg.norm(xr)


def test_noCPQR_rejects_underdetermined():
    with pytest.raises(RuntimeError, match="Matrix is not overdetermined."):
        orc.ls_dense_hashing_blendenpik_noCPQR(np.ones((3, 5)), np.ones(3), 1.7, 1)


def test_random_sample_rows_match_live_libc():
    """select_k_from_n over 0..N-1 (src/sparse_helpers.cpp:74-86) driven by the C
    library's own rand(), against the oracle's draw from its restated stream."""
    try:
        libc = ctypes.CDLL("libc.so.6")
    except OSError:
        pytest.skip("no glibc")
    for (N, m, s) in ((50, 33, 5), (1000, 250, 41)):
        libc.srand(ctypes.c_uint(s))
        idx = list(range(N))
        for i in range(m):
            j = libc.rand() % (N - i) + i
            idx[i], idx[j] = idx[j], idx[i]
        assert list(orc.random_sample_rows(orc.Rng(s), N, m)) == idx[:m]


@pytest.mark.parametrize("tag", FULL_RANK_TAGS)
def test_blendenpik_full_rank_fixtures_vs_lstsq(fixtures, tag):
    """The ls_dense_blendenpik restatement on the dense full-rank fixtures the
    reference's test/test_solvers.sh runs ls_blendenpik on, at its driver's
    gamma = 2.2 (test/ls_blendenpik.cpp:61), against LAPACK least squares; the
    sketch is exactly the sampled rows of the randomized DHT."""
    Ad = fixtures[f"{tag}DenseFullRank/dense"]
    n, d = Ad.shape
    b = np.ones(n)
    xr = np.linalg.lstsq(Ad, b, rcond=None)[0]
    out = orc.ls_dense_blendenpik(Ad, b, 2.2, it_tol=1e-12, seed=5)
    assert out["rank"] == d and out["flag"] == 0 and out["m"] == math.ceil(2.2 * d)
    assert np.linalg.norm(out["x"] - xr) <= 1e-8 * np.linalg.norm(xr)
    D = orc.rand_signs(orc.Rng(5), n)
    Y = orc.unitary_dht(Ad, D)
    np.testing.assert_array_equal(out["rows"], orc.random_sample_rows(orc.Rng(5), n, out["m"]))
    np.testing.assert_array_equal(out["SA"], Y[out["rows"]])


def test_blendenpik_rejects_underdetermined_and_oversized_sample():
    with pytest.raises(RuntimeError, match="Matrix is not overdetermined."):
        orc.ls_dense_blendenpik(np.ones((3, 5)), np.ones(3), 2.2)
    with pytest.raises(ValueError):
        orc.ls_dense_blendenpik(np.eye(10, 6), np.ones(10), 2.0)   # 12 rows of 10


def test_blendenpik_padded_transform_vs_lstsq():
    """The transform padded to a smooth even length (the reference pads in its
    wisdom mode, src/fast_unitary_transform.cpp:63-64): the sample is drawn from
    all N rows, including rows that come from the zero padding."""
    rng = np.random.default_rng(12)
    A = rng.standard_normal((1001, 40))
    b = rng.standard_normal(1001)
    N = 1050   # even, N / 2 = 525 = 3 * 5^2 * 7
    out = orc.ls_dense_blendenpik(A, b, 2.2, it_tol=1e-12, seed=3, N=N)
    xr = np.linalg.lstsq(A, b, rcond=None)[0]
    assert out["rank"] == 40 and out["flag"] == 0
    assert out["rows"].max() < N and len(np.unique(out["rows"])) == out["m"]
    assert np.linalg.norm(out["x"] - xr) <= 1e-8 * np.linalg.norm(xr)

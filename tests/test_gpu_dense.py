"""GPU parity of the dense path (ls_dense_hashing_blendenpik and _noCPQR)
against the oracle and the reference's golden data.  Tolerances: DHT and
sketch to 2e-6 normwise in FP32 (1e-12 in FP64); x to 1e-8 relative on
full-rank inputs; backward error <= 1e-10."""
import numpy as np
import pytest

import skills_gb300 as skl
import ski_lls_oracle as orc
from conftest import FULL_RANK_TAGS

pytestmark = pytest.mark.gpu

XTOL = 1e-8
BETOL = 1e-10


def _dense(n, d, kappa_exp, seed, noise=1e-4):
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.standard_normal((n, d)))
    V, _ = np.linalg.qr(rng.standard_normal((d, d)))
    A = np.asfortranarray((U * np.logspace(0, -kappa_exp, d)) @ V.T)
    xt = rng.standard_normal(d)
    return A, A @ xt + noise * rng.standard_normal(n)


@pytest.mark.parametrize("N", [4, 50, 100, 120, 2 * 3 * 5 * 7 * 4, 40000])
def test_dht_matches_numpy(N):
    rng = np.random.default_rng(N)
    A = rng.standard_normal((N, 3))
    D = np.where(rng.random(N) < 0.5, -1.0, 1.0)
    ref = orc.unitary_dht(A, D)
    for prec, tol in (("mixed", 2e-6), ("fp64", 1e-12)):
        Y = skl.dht(A, D, N, precision=prec)
        assert np.linalg.norm(Y - ref) <= tol * np.linalg.norm(ref), prec


def test_dht_zero_padding():
    rng = np.random.default_rng(3)
    n, N = 97, skl.dht_length(97)
    assert N >= n and N % 2 == 0
    A = rng.standard_normal((n, 2))
    D = np.ones(n)
    ref = orc.unitary_dht(A, D, N)
    Y = skl.dht(A, D, N, precision="fp64")
    assert np.linalg.norm(Y - ref) <= 1e-12 * np.linalg.norm(ref)
    np.testing.assert_allclose(np.linalg.norm(Y, axis=0), np.linalg.norm(A, axis=0), rtol=1e-12)


def test_dense_sketch_vs_oracle():
    rng = np.random.default_rng(5)
    n, d, m, k = 4000, 60, 102, 2
    A = rng.standard_normal((n, d))
    b = rng.standard_normal(n)
    g = orc.Rng(9)
    D = orc.rand_signs(g, n)
    rows, vals = orc.gen_hashing(g, m, n, k)
    Y = orc.unitary_dht(A, D)
    SA_ref = orc.dense_sketch(Y, m, k, rows, vals)
    Sb_ref = orc.dense_sketch(orc.unitary_dht(b, D), m, k, rows, vals)[:, 0]
    for prec, tol in (("mixed", 2e-6), ("fp64", 1e-12)):
        SA, Sb = skl.sketch_dense(A, b, D, n, m, k, rows, vals, precision=prec)
        assert np.linalg.norm(SA - SA_ref) <= tol * np.linalg.norm(SA_ref), prec
        assert np.linalg.norm(Sb - Sb_ref) <= 1e-12 * np.linalg.norm(Sb_ref)


def test_dense_example_known_answer(fixtures):
    A = fixtures["dense_example/A"]
    b = fixtures["dense_example/b"]
    for seed in (1, 2, 3):
        res = skl.ls_dense_hashing_blendenpik(A, b, 1.1, 3, seed=seed)
        np.testing.assert_allclose(res.x, fixtures["dense_example/x_expected"], atol=5e-5)


@pytest.mark.parametrize("tag", FULL_RANK_TAGS)
def test_full_rank_dense_fixtures(fixtures, tag):
    A = fixtures[f"{tag}DenseFullRank/dense"]
    b = np.ones(A.shape[0])
    xr = np.linalg.lstsq(A, b, rcond=None)[0]
    for prec in ("mixed", "fp64"):
        res = skl.ls_dense_hashing_blendenpik(A, b, 1.7, 1, it_tol=1e-12, seed=4, precision=prec,
                                              backward_tol=BETOL)
        assert np.linalg.norm(res.x - xr) <= XTOL * np.linalg.norm(xr), prec
        assert res.rank == A.shape[1]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_dense_vs_oracle(precision):
    A, b = _dense(6000, 200, 3.0, 11)
    res = skl.ls_dense_hashing_blendenpik(A, b, 1.7, 1, it_tol=1e-12, seed=77, precision=precision,
                                          backward_tol=BETOL)
    ref = orc.ls_dense_hashing_blendenpik(A, b, 1.7, 1, it_tol=1e-12, seed=77,
                                          N=skl.dht_length(6000))
    assert np.linalg.norm(res.x - ref["x"]) <= XTOL * np.linalg.norm(ref["x"])
    r = b - A @ res.x
    assert np.linalg.norm(A.T @ r) / (np.linalg.norm(A) * np.linalg.norm(r)) <= BETOL
    assert res.rank == ref["rank"] == 200


def test_dense_noCPQR():
    A, b = _dense(3000, 100, 2.0, 12)
    xr = np.linalg.lstsq(A, b, rcond=None)[0]
    res = skl.ls_dense_hashing_blendenpik_noCPQR(A, b, 1.7, 1, it_tol=1e-12, seed=5)
    assert res.rank == 100
    assert np.linalg.norm(res.x - xr) <= XTOL * np.linalg.norm(xr)
    ref = orc.ls_dense_hashing_blendenpik_noCPQR(A, b, 1.7, 1, it_tol=1e-12, seed=5,
                                                 N=skl.dht_length(3000))
    assert np.linalg.norm(res.x - ref["x"]) <= XTOL * np.linalg.norm(xr)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_dense_blendenpik_vs_oracle(precision):
    """ls_dense_blendenpik (src/ls_dense_blendenpik.cpp:21-70): same seed, so the
    same signs and sampled rows as the oracle; x to 1e-8 of LAPACK and the
    oracle, and LSQR's iteration count within 2 of the oracle's."""
    A, b = _dense(3000, 100, 2.0, 21)
    xr = np.linalg.lstsq(A, b, rcond=None)[0]
    res = skl.ls_dense_blendenpik(A, b, 2.2, it_tol=1e-12, seed=6, precision=precision)
    ref = orc.ls_dense_blendenpik(A, b, 2.2, it_tol=1e-12, seed=6, N=skl.dht_length(3000))
    assert res.rank == 100 and res.flag == 0
    assert res.info["sketch_rows"] == ref["m"] == 221   # ceil(2.2 * 100) in FP64 arithmetic
    assert np.linalg.norm(res.x - xr) <= XTOL * np.linalg.norm(xr)
    assert np.linalg.norm(res.x - ref["x"]) <= XTOL * np.linalg.norm(xr)
    assert abs(res.it - ref["it"]) <= 2


def test_dense_blendenpik_padded_transform_and_errors():
    # n = 1,001: the transform pads to an even smooth length and the sample is
    # drawn from all N rows (zero rows of D A included)
    A, b = _dense(1001, 60, 1.0, 3)
    N = skl.dht_length(1001)
    assert N > 1001
    xr = np.linalg.lstsq(A, b, rcond=None)[0]
    res = skl.ls_dense_blendenpik(A, b, 2.2, it_tol=1e-12, seed=2)
    ref = orc.ls_dense_blendenpik(A, b, 2.2, it_tol=1e-12, seed=2, N=N)
    assert np.linalg.norm(res.x - xr) <= XTOL * np.linalg.norm(xr)
    assert np.linalg.norm(res.x - ref["x"]) <= XTOL * np.linalg.norm(xr)
    r1 = skl.ls_dense_blendenpik(A, b, 2.2, it_tol=1e-10, seed=9)
    r2 = skl.ls_dense_blendenpik(A, b, 2.2, it_tol=1e-10, seed=9)
    assert np.array_equal(r1.x, r2.x)
    with pytest.raises(skl.SklError) as e:
        skl.ls_dense_blendenpik(A[:40], b[:40], seed=1)
    assert e.value.status == skl.SKL_ERR_NOT_OVERDETERMINED
    with pytest.raises(skl.SklError) as e:
        skl.ls_dense_blendenpik(A[:100], b[:100], 2.0, seed=1)   # 120 rows of 100
    assert e.value.status == skl.SKL_ERR_INVALID


def test_dense_rank_deficient_absolute_rule():
    # duplicated columns: the absolute |R_ii| > rcond rule drops them when rcond
    # sits above the working precision's noise on |R_ii| (~1e-7 |R_00| in FP32)
    rng = np.random.default_rng(2)
    A = rng.standard_normal((3000, 80))
    A[:, 10] = A[:, 3]
    A[:, 50] = 2 * A[:, 7] - A[:, 9]
    b = rng.standard_normal(3000)
    for prec in ("mixed", "fp64"):
        res = skl.ls_dense_hashing_blendenpik(A, b, 1.7, 1, rcond=1e-3, it_tol=1e-12, seed=3,
                                              backward_tol=BETOL, precision=prec)
        assert res.rank == 78
        xr = np.linalg.lstsq(A, b, rcond=None)[0]
        assert abs(np.linalg.norm(b - A @ res.x) - np.linalg.norm(b - A @ xr)) <= 1e-9 * np.linalg.norm(b)


def test_dense_bitwise_reproducible_and_errors():
    A, b = _dense(2000, 50, 2.0, 4)
    r1 = skl.ls_dense_hashing_blendenpik(A, b, 1.7, 1, it_tol=1e-10, seed=8)
    r2 = skl.ls_dense_hashing_blendenpik(A, b, 1.7, 1, it_tol=1e-10, seed=8)
    assert np.array_equal(r1.x, r2.x)
    with pytest.raises(skl.SklError) as e:
        skl.ls_dense_hashing_blendenpik(A[:40], b[:40], seed=1)
    assert e.value.status == skl.SKL_ERR_NOT_OVERDETERMINED

"""GPU parity of the sparse path (ls_sparse_spqr) against the oracle and the
reference's golden data.  Tolerances: x to 1e-8 relative on full-rank inputs,
backward error <= 1e-10, fixture residuals to the 6 digits the reference prints."""
import numpy as np
import pytest
import scipy.sparse as sp

import skills_gb300 as skl
import ski_lls_oracle as orc
from conftest import RANK_DEF_NAMES, FULL_RANK_TAGS, fixture_csc, residual_matches

pytestmark = pytest.mark.gpu

XTOL = 1e-8
BETOL = 1e-10


def _problem(n, d, density, seed, noise=1e-3, scale_exp=0.0):
    rng = np.random.default_rng(seed)
    A = sp.random(n, d, density=density, random_state=seed + 1, format="csc")
    A.data = rng.standard_normal(A.nnz)
    if scale_exp:
        A = A @ sp.diags(10.0 ** rng.uniform(0, scale_exp, d))
        A = A.tocsc()
    A.sort_indices()
    xt = rng.standard_normal(d)
    b = A @ xt + noise * rng.standard_normal(n)
    return A, b


def _be(A, x, b):
    r = b - A @ x
    return np.linalg.norm(A.T @ r) / (sp.linalg.norm(A, "fro") * np.linalg.norm(r))


def test_sparse_example_known_answer(fixtures):
    p, i, x = (fixtures[f"sparse_example/{k}"] for k in ("indptr", "indices", "data"))
    res = skl.ls_sparse_spqr((p, i, x, (4, 3)), fixtures["sparse_example/b"], 1.1, 3, seed=1)
    np.testing.assert_allclose(res.x, fixtures["sparse_example/x_expected"], atol=5e-5)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_random_sparse_vs_oracle(precision):
    A, b = _problem(3000, 80, 0.03, 3)
    res = skl.ls_sparse_spqr(A, b, 1.7, 2, it_tol=1e-12, seed=1, precision=precision,
                             backward_tol=BETOL)
    ref = orc.ls_sparse_spqr(3000, 80, A.indptr, A.indices, A.data, b, 1.7, 2, it_tol=1e-12,
                             rng=orc.Rng(1))
    assert np.linalg.norm(res.x - ref["x"]) <= XTOL * np.linalg.norm(ref["x"])
    assert res.info["backward_error"] <= BETOL
    assert abs(_be(A, res.x, b) - res.info["backward_error"]) < 1e-12 + 0.1 * res.info["backward_error"]
    assert res.rank == ref["rank"] == 80


def test_column_scaled_rank_deficient():
    # 1e4 column scaling and planted dependent columns, as in the
    # 120,000 x 5,000 configuration (smaller size)
    A, b = _problem(6000, 300, 0.02, 5, noise=1e-6, scale_exp=4.0)
    A = A.tolil()
    rng = np.random.default_rng(9)
    for j in range(5):
        p, q = rng.choice(np.arange(10, 300), 2, replace=False)
        A[:, j] = rng.standard_normal() * A[:, p] + rng.standard_normal() * A[:, q]
    A = A.tocsc()
    A.sort_indices()
    res = skl.ls_sparse_spqr(A, b, 1.7, 2, it_tol=1e-12, seed=1, backward_tol=BETOL)
    assert res.rank == 295
    assert _be(A, res.x, b) <= BETOL
    ref = np.linalg.lstsq(A.toarray(), b, rcond=None)[0]
    r_gpu = np.linalg.norm(b - A @ res.x)
    r_ref = np.linalg.norm(b - A @ ref)
    assert abs(r_gpu - r_ref) <= 1e-9 * r_ref


def test_mixed_sketch_solution_matches_fp64():
    # Column scales up to 1e8 and planted dependent columns leave the FP32
    # sketch solution ~1e-6 off; the mixed path refines it against the FP64
    # residual, so its explicit residual and LSQR iteration count match the
    # FP64 path's (the reference forms x_s from an FP64 factorization).
    import synthetic
    A, b, _ = synthetic.sparse_illcond(seed=11, n=24000, d=1000, per_col=240, n_dep=10)
    out = {}
    for precision in ("mixed", "fp64"):
        out[precision] = skl.ls_sparse_spqr(A, b, 1.7, 2, it_tol=1e-10, seed=1,
                                            precision=precision)
    mixed, fp64 = out["mixed"], out["fp64"]
    assert mixed.info["sketch_refine_steps"] >= 1
    assert fp64.info["sketch_refine_steps"] == 0
    xr_m, xr_d = mixed.info["explicit_residual"], fp64.info["explicit_residual"]
    # the two factorizations keep different (equally valid) column sets, so the
    # sketched optima differ slightly; unrefined, xr_m would be ~1e-6 ||b|| larger
    assert abs(xr_m - xr_d) <= 1e-2 * xr_d, (xr_m, xr_d)
    assert mixed.it <= fp64.it + 5, (mixed.it, fp64.it)
    assert mixed.rank == fp64.rank == 990


@pytest.mark.parametrize("name", RANK_DEF_NAMES)
def test_rank_deficient_fixture_residuals(fixtures, name):
    n, d, p, i, x = fixture_csc(fixtures, name)
    b = np.ones(n)
    for precision in ("mixed", "fp64"):
        res = skl.ls_sparse_spqr((p, i, x, (n, d)), b, 1.4, 2, seed=1, precision=precision)
        A = sp.csc_matrix((x, i, p), shape=(n, d))
        r = float(np.linalg.norm(b - A @ res.x))
        assert residual_matches(r, float(fixtures[name + "/expected_residual"])), (precision, r)


@pytest.mark.parametrize("tag", FULL_RANK_TAGS)
def test_full_rank_sparse_fixtures(fixtures, tag):
    n, d, p, i, x = fixture_csc(fixtures, f"{tag}SparseFullRank")
    A = sp.csc_matrix((x, i, p), shape=(n, d))
    b = np.ones(n)
    xr = np.linalg.lstsq(A.toarray(), b, rcond=None)[0]
    res = skl.ls_sparse_spqr(A, b, 1.4, 2, it_tol=1e-12, seed=1, backward_tol=BETOL)
    assert np.linalg.norm(res.x - xr) <= XTOL * np.linalg.norm(xr)


def test_bitwise_reproducible():
    A, b = _problem(4000, 120, 0.02, 21)
    r1 = skl.ls_sparse_spqr(A, b, 1.7, 2, it_tol=1e-10, seed=3)
    r2 = skl.ls_sparse_spqr(A, b, 1.7, 2, it_tol=1e-10, seed=3)
    assert np.array_equal(r1.x, r2.x) and r1.it == r2.it


def test_errors():
    A, b = _problem(100, 10, 0.2, 1)
    with pytest.raises(skl.SklError) as e:
        skl.ls_sparse_spqr(A.T.tocsc(), np.ones(10), seed=1)
    assert e.value.status == skl.SKL_ERR_NOT_OVERDETERMINED
    assert "not overdetermined" in str(e.value)
    bad = A.copy()
    bad.indices = bad.indices.copy()
    bad.indices[0] = 1000
    with pytest.raises(skl.SklError) as e:
        skl.ls_sparse_spqr((bad.indptr, bad.indices, bad.data, bad.shape), b, seed=1)
    assert e.value.status == skl.SKL_ERR_INVALID
    nanA = A.copy()
    nanA.data = nanA.data.copy()
    nanA.data[3] = np.nan
    with pytest.raises(skl.SklError) as e:
        skl.ls_sparse_spqr(nanA, b, seed=1)
    assert e.value.status == skl.SKL_ERR_NONFINITE
    # the library stays usable after errors
    res = skl.ls_sparse_spqr(A, b, 1.7, 2, seed=1, it_tol=1e-12)
    assert np.isfinite(res.x).all()


def test_max_it_flag():
    A, b = _problem(3000, 80, 0.03, 3)
    res = skl.ls_sparse_spqr(A, b, 1.7, 2, it_tol=1e-30, max_it=3, seed=1, abs_tol=0.0)
    assert res.flag == 1 and res.it == 3


def test_building_blocks_sketch_and_cpqr():
    A, b = _problem(2000, 50, 0.05, 8)
    m, k = 85, 2
    rows, vals = orc.gen_hashing(orc.Rng(4), m, 2000, k)
    SA_ref, Sb_ref = orc.sparse_sketch(2000, 50, A.indptr, A.indices, A.data, b, m, k, rows, vals)
    for prec, tol in (("mixed", 1e-6), ("fp64", 1e-13)):
        SA, Sb = skl.sketch_sparse(A, b, m, k, rows, vals, precision=prec)
        assert np.max(np.abs(SA - SA_ref)) <= tol * np.max(np.abs(SA_ref))
        np.testing.assert_array_equal(Sb, Sb_ref)   # same order and arithmetic as cs_dl_gaxpy
    QR, jpvt, tau = skl.cpqr(SA_ref, precision="fp64")
    R = np.triu(QR[:50, :50])
    # A P = Q R  => ||A P||_col norms equal ||R||_col norms, and R^T R = (A P)^T (A P)
    AP = SA_ref[:, jpvt]
    np.testing.assert_allclose(R.T @ R, AP.T @ AP, rtol=1e-9, atol=1e-9 * np.linalg.norm(AP) ** 2)
    assert sorted(jpvt.tolist()) == list(range(50))
    Rm = np.triu(skl.cpqr(SA_ref, precision="mixed")[0][:50, :50])
    assert np.all(np.abs(np.diag(Rm)) > 0)
    x = np.random.default_rng(0).standard_normal(50)
    np.testing.assert_allclose(skl.trsv_upper(R, x, "n", "fp64"), orc.usolve(R, x), rtol=1e-9)
    np.testing.assert_allclose(skl.trsv_upper(R, x, "t", "fp64"), orc.utsolve(R, x), rtol=1e-9)

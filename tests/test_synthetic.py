"""The seeded workload generators behind bench.py produce the shapes and value
distributions their configurations state (checked on reduced sizes, same code)."""
import numpy as np
import scipy.sparse as sp

import synthetic


def test_generators_are_pure_functions_of_the_seed():
    A1, b1 = synthetic.sparse_uniform(500, 40, 10, 7, 1e-3)
    A2, b2 = synthetic.sparse_uniform(500, 40, 10, 7, 1e-3)
    assert (A1 != A2).nnz == 0 and np.array_equal(b1, b2)
    A3, _ = synthetic.sparse_uniform(500, 40, 10, 8, 1e-3)
    assert (A1 != A3).nnz > 0


def test_sparse_uniform_columns_and_rhs():
    n, d, per = 2000, 100, 20
    A, b = synthetic.sparse_uniform(n, d, per, 3, 0.0)
    assert A.shape == (n, d) and A.has_sorted_indices
    cnt = np.diff(A.indptr)
    assert cnt.min() >= 1 and cnt.max() <= per          # duplicates summed, no empty column
    assert abs(cnt.mean() - per) < 0.5                   # ~per distinct rows out of n
    assert np.allclose(A.data.std(), 1.0, atol=0.1)      # N(0, 1) values
    x = np.linalg.lstsq(A.toarray(), b, rcond=None)[0]   # noise 0: b is in the range of A
    assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)


def test_sparse_illcond_scales_and_dependent_columns():
    n, d, n_dep = 3000, 120, 10
    A, b, dep = synthetic.sparse_illcond(seed=5, n=n, d=d, per_col=60, n_dep=n_dep, scale_exp=8.0)
    assert A.shape == (n, d) and len(set(dep)) == n_dep
    norms = sp.linalg.norm(A, axis=0)
    keep = np.setdiff1d(np.arange(d), dep)
    assert norms[keep].max() / norms[keep].min() > 1e6   # 10^U[0,8] column scales
    # each replaced column is a combination of two kept columns: the matrix
    # loses exactly n_dep in rank (scaled so the scales do not hide it)
    As = (A @ sp.diags(1.0 / norms)).toarray()
    sv = np.linalg.svd(As, compute_uv=False)
    assert np.sum(sv > 1e-10 * sv[0]) == d - n_dep


def test_sparse_zipf_counts():
    A, b = synthetic.sparse_zipf(seed=1, n=50000, d=500, cap=2000, target_nnz=100000)
    cnt = np.diff(A.indptr)
    assert cnt.min() >= 1 and cnt.max() <= 2000
    assert 0.8e5 < A.nnz <= 1.1e5
    assert cnt.max() > 20 * np.median(cnt)               # heavy-tailed column counts
    assert b.shape == (50000,)


def test_dense_kappa_singular_values():
    A, b = synthetic.dense_kappa(seed=2, n=600, d=60, kappa_exp=6.0, noise=0.0)
    sv = np.linalg.svd(A, compute_uv=False)
    np.testing.assert_allclose(sv, np.logspace(0.0, -6.0, 60), rtol=1e-6)
    assert A.flags.f_contiguous


def test_batched_problem_ranges():
    probs = synthetic.batched(seed=4, count=6)
    assert len(probs) == 6
    for A, b in probs:
        n, d = A.shape
        assert 50 <= d <= 500 and n >= 20 * d and n >= 2000
        assert b.shape == (n,)
        dens = A.nnz / (n * d)
        assert 0.003 < dens < 0.06

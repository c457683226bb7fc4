"""Seeded synthetic least-squares problems with the shapes and value
distributions of the solver's benchmark configurations.

No public dataset is involved; every generator is a pure function of its seed.

  sparse_uniform_1pct   20,000 x 1,000, 200 nnz/column, N(0,1), b = A x* + 1e-3 N(0,1)
  dense_kappa1e6        40,000 x 4,000, A = U diag(logspace(0,-6)) V^T, b = A x* + 1e-4 noise
  sparse_illcond        120,000 x 5,000, 1,200 nnz/column, N(0,1), column scales 10^U[0,8],
                        50 columns replaced by combinations of two others,
                        b = A x* + 1e-6 noise
  sparse_zipf           1,000,000 x 10,000, column nnz ~ Zipf(1.2) capped at 20,000
                        (about 1e7 nnz), N(0,1), b ~ N(0,1)
  batched               512 problems, n ~ U[2000, 50000], d ~ U[50, 500], n >= 20 d,
                        density ~ U[0.5%, 5%], column scales 10^U[0,4], b ~ N(0,1)
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def _csc_from_columns(n, d, rows, cols, vals):
    A = sp.csc_matrix((vals, (rows, cols)), shape=(n, d))
    A.sum_duplicates()
    A.sort_indices()
    return A


def _reseed_empty(A, rng):
    """Give every empty column one N(0,1) entry (full column rank check)."""
    counts = np.diff(A.indptr)
    empty = np.flatnonzero(counts == 0)
    if empty.size == 0:
        return A
    n = A.shape[0]
    extra = sp.csc_matrix((rng.standard_normal(empty.size), (rng.integers(0, n, empty.size), empty)),
                          shape=A.shape)
    A = (A + extra).tocsc()
    A.sort_indices()
    return A


def sparse_uniform(n, d, per_col, seed, noise):
    rng = np.random.default_rng(seed)
    rows = rng.integers(0, n, size=d * per_col)
    cols = np.repeat(np.arange(d), per_col)
    vals = rng.standard_normal(d * per_col)
    A = _reseed_empty(_csc_from_columns(n, d, rows, cols, vals), rng)
    xs = rng.standard_normal(d)
    b = A @ xs + noise * rng.standard_normal(n)
    return A, b


def sparse_uniform_1pct(seed=2024):
    return sparse_uniform(20000, 1000, 200, seed, 1e-3)


def sparse_illcond(seed=2024, n=120000, d=5000, per_col=1200, n_dep=50, scale_exp=8.0):
    rng = np.random.default_rng(seed)
    rows = rng.integers(0, n, size=d * per_col)
    cols = np.repeat(np.arange(d), per_col)
    vals = rng.standard_normal(d * per_col)
    A = _reseed_empty(_csc_from_columns(n, d, rows, cols, vals), rng)
    A = (A @ sp.diags(10.0 ** rng.uniform(0.0, scale_exp, d))).tocsc()
    # replace n_dep columns by a*A_p + b*A_q with p, q outside the replaced set
    dep = rng.choice(d, size=n_dep, replace=False)
    keep = np.setdiff1d(np.arange(d), dep)
    if n_dep:
        p = rng.choice(keep, size=n_dep)
        q = rng.choice(keep, size=n_dep)
        a = rng.standard_normal(n_dep)
        c = rng.standard_normal(n_dep)
        A = A.tocsc()
        mix = sp.csc_matrix((np.concatenate([a, c]),
                             (np.concatenate([p, q]), np.concatenate([np.arange(n_dep)] * 2))),
                            shape=(d, n_dep))
        newcols = (A @ mix).tocsc()
        # assemble: columns `dep` taken from newcols, others from A
        order = np.empty(d, dtype=np.int64)
        order[keep] = np.arange(keep.size)
        order[dep] = keep.size + np.arange(n_dep)
        stacked = sp.hstack([A[:, keep], newcols], format="csc")
        A = stacked[:, order].tocsc()
    A.sort_indices()
    xs = rng.standard_normal(d)
    b = A @ xs + 1e-6 * rng.standard_normal(n)
    return A, b, dep


def sparse_zipf(seed=2024, n=1_000_000, d=10_000, cap=20_000, target_nnz=10_000_000):
    rng = np.random.default_rng(seed)
    raw = np.minimum(rng.zipf(1.2, size=d), cap).astype(np.float64)
    counts = np.maximum(1, np.round(raw * (target_nnz / raw.sum()))).astype(np.int64)
    counts = np.minimum(counts, cap)
    cols = np.repeat(np.arange(d), counts)
    rows = rng.integers(0, n, size=cols.size)
    vals = rng.standard_normal(cols.size)
    A = _reseed_empty(_csc_from_columns(n, d, rows, cols, vals), rng)
    b = rng.standard_normal(n)
    return A, b


def dense_kappa(seed=2024, n=40000, d=4000, kappa_exp=6.0, noise=1e-4):
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.standard_normal((n, d)))
    V, _ = np.linalg.qr(rng.standard_normal((d, d)))
    sigma = np.logspace(0.0, -kappa_exp, d)
    A = np.asfortranarray((U * sigma) @ V.T)
    xs = rng.standard_normal(d)
    b = A @ xs + noise * rng.standard_normal(n)
    return A, b


def batched(seed=2024, count=512):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        d = int(rng.integers(50, 501))
        n = int(max(rng.integers(2000, 50001), 20 * d))
        dens = rng.uniform(0.005, 0.05)
        per_col = max(1, int(round(dens * n)))
        A, _ = sparse_uniform(n, d, per_col, int(rng.integers(1 << 30)), 0.0)
        A = (A @ sp.diags(10.0 ** rng.uniform(0.0, 4.0, d))).tocsc()
        A.sort_indices()
        out.append((A, rng.standard_normal(n)))
    return out


WORKLOADS = {
    "sparse_uniform_20000x1000": dict(kind="sparse", gen=lambda: sparse_uniform_1pct(),
                                      gamma=1.7, k=2),
    "dense_kappa1e6_40000x4000": dict(kind="dense", gen=lambda: dense_kappa(), gamma=1.7, k=1),
    "sparse_illcond_120000x5000": dict(kind="sparse", gen=lambda: sparse_illcond()[:2],
                                       gamma=1.7, k=2),
    "sparse_zipf_1000000x10000": dict(kind="sparse", gen=lambda: sparse_zipf(), gamma=1.5, k=3),
    # the Blendenpik comparison solver on the dense matrix above, at its
    # driver's gamma (test/ls_blendenpik.cpp:61): 8,800 sampled rows
    "dense_blendenpik_40000x4000": dict(kind="dense", gen=lambda: dense_kappa(), gamma=2.2, k=1,
                                        solver="blendenpik"),
}

"""skl_batched_sparse_solve: many independent sparse problems in one call
(the batched configuration: d in [50, 500], n >= 20 d, column scales up to
1e4).  Each x must be bit-identical to a loop of single solves drawing the
same hash streams, and each must meet the solver's own accuracy bar against
the oracle's least-squares answer."""
import numpy as np
import pytest
import scipy.sparse as sp

import skills_gb300 as skl


def _problems(count, seed, dmax=120):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        d = int(rng.integers(20, dmax))
        n = int(max(rng.integers(600, 4000), 20 * d))
        per_col = max(2, int(rng.uniform(0.005, 0.05) * n))
        rows = np.concatenate([rng.choice(n, per_col, replace=False) for _ in range(d)])
        cols = np.repeat(np.arange(d), per_col)
        A = sp.csc_matrix((rng.standard_normal(rows.size), (rows, cols)), shape=(n, d))
        A = (A @ sp.diags(10.0 ** rng.uniform(0.0, 4.0, d))).tocsc()
        A.sort_indices()
        out.append((A, rng.standard_normal(n)))
    return out


def test_batched_rejects_underdetermined_problem():
    # validated before any device work (no GPU needed)
    A = sp.random(5, 9, density=0.5, format="csc", random_state=1)
    good = _problems(1, 3)[0]
    with pytest.raises(skl.SklError) as e:
        skl.batched_sparse_spqr([good, (A, np.ones(5))], 1.7, 2, seed=1)
    assert e.value.status == skl.SKL_ERR_NOT_OVERDETERMINED


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batched_matches_loop_of_single_solves(precision):
    probs = _problems(12, 7)
    xs, infos, status = skl.batched_sparse_spqr(probs, 1.7, 2, it_tol=1e-12, seed=11,
                                                precision=precision)
    assert status == [0] * len(probs)
    for p, (A, b) in enumerate(probs):
        ref = skl.ls_sparse_spqr(A, b, 1.7, 2, it_tol=1e-12, seed=11, precision=precision)
        assert np.array_equal(xs[p], ref.x), p
        assert infos[p].it == ref.it and infos[p].rank == ref.rank
        xr = np.linalg.lstsq(A.toarray(), b, rcond=None)[0]
        assert np.linalg.norm(xs[p] - xr) <= 1e-8 * np.linalg.norm(xr), p


@pytest.mark.gpu
def test_batched_library_stream_order():
    # without a seed, problem p hashes from the library stream after problems
    # 0..p-1, as consecutive single solves would
    probs = _problems(6, 9)
    skl.srand(5)
    xs, _, _ = skl.batched_sparse_spqr(probs, 1.7, 2, it_tol=1e-12)
    skl.srand(5)
    for p, (A, b) in enumerate(probs):
        ref = skl.ls_sparse_spqr(A, b, 1.7, 2, it_tol=1e-12)
        assert np.array_equal(xs[p], ref.x), p

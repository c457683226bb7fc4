"""The autotuner (skl_opts.autotune): the first solve of a shape class times
the candidate launch shapes on its own data and caches the fastest; later
solves of the class reuse them.  Checked: every tuned choice is one of the
candidates, the tuned solve agrees with the untuned one (the LS solution is
unique on this full-rank input), and a second solve of the class reuses the
cached shapes and reproduces the first bit for bit."""
import numpy as np
import pytest

import skills_gb300 as skl
import synthetic

pytestmark = pytest.mark.gpu


def test_autotune_chooses_candidates_and_caches():
    A, b = synthetic.sparse_uniform(12000, 600, 120, 31, 1e-3)
    plain = skl.ls_sparse_spqr(A, b, 1.7, 2, it_tol=1e-12, seed=1)
    # untuned: the fixed heuristics, and the panel width the CPQR used
    assert plain.info["tuned"][0] == 0 and plain.info["tuned"][2:] == [0, 0]
    assert plain.info["tuned"][1] in (32, 40, 48, 56, 64)
    first = skl.ls_sparse_spqr(A, b, 1.7, 2, it_tol=1e-12, seed=1, autotune=1)
    sk, nb, ln, lt = first.info["tuned"]
    assert sk in (256, 512, 1024) and nb in (32, 40, 48, 56, 64)
    assert ln in (4, 8, 16, 32) and lt in (4, 8, 16, 32)
    assert np.linalg.norm(first.x - plain.x) <= 1e-8 * np.linalg.norm(plain.x)
    second = skl.ls_sparse_spqr(A, b, 1.7, 2, it_tol=1e-12, seed=1, autotune=1)
    assert second.info["tuned"] == first.info["tuned"]
    assert np.array_equal(second.x, first.x)
    # FP64 path: its own class (the panel width is not tuned there)
    f64 = skl.ls_sparse_spqr(A, b, 1.7, 2, it_tol=1e-12, seed=1, autotune=1, precision="fp64")
    assert f64.info["tuned"][1] == 0 and f64.info["tuned"][2] in (4, 8, 16, 32)
    assert np.linalg.norm(f64.x - plain.x) <= 1e-8 * np.linalg.norm(plain.x)

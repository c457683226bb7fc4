"""The CPQR's block-reflector product W = V^T A on the tensor cores (tcgen05,
3xTF32) against an FP64 product and the CUDA-core FP32 kernel.

The shapes cover the first panel of the 120,000 x 5,000 workload's sketch
(8,500 x 4,936 trailing columns, 64 reflectors), row counts that are not a
multiple of the 32-row stage, column counts that leave a partial 128-column
tile, panels narrower than 64 and a single column.  Error measure: |W - W64|
divided by |V|^T |A| entry by entry (FP32 accumulation over up to 8,500 terms
gives ~sqrt(K) 2^-24 there; a wrong descriptor or layout gives O(1)).
"""
import numpy as np
import pytest

import skills_gb300 as skl

pytestmark = pytest.mark.gpu

SHAPES = [(8500, 4936, 64), (8500, 200, 64), (1000, 300, 40), (97, 130, 64), (33, 1, 64),
          (4100, 1000, 8)]


def _case(M, N, b, seed):
    rng = np.random.default_rng(seed)
    V = rng.standard_normal((M, b)).astype(np.float32)
    A = (rng.standard_normal((M, N)) * 10.0 ** rng.uniform(-3, 3, N)).astype(np.float32)
    W64 = V.astype(np.float64).T @ A.astype(np.float64)
    bound = np.abs(V.astype(np.float64)).T @ np.abs(A.astype(np.float64))
    return V, A, W64, bound


@pytest.mark.parametrize("shape", SHAPES)
def test_tensor_core_vta_accuracy(shape):
    M, N, b = shape
    V, A, W64, bound = _case(M, N, b, M + N + b)
    for tensor in (True, False):
        W = skl.gemm_vta(V, A, tensor=tensor).astype(np.float64)
        rel = np.abs(W - W64) / bound
        assert rel.max() <= 2.0 ** -14, (shape, tensor, rel.max())
        assert rel.mean() <= 2.0 ** -18, (shape, tensor, rel.mean())


def test_tensor_core_vta_matches_cuda_core_kernel():
    V, A, W64, bound = _case(8500, 4936, 64, 3)
    Wt = skl.gemm_vta(V, A, tensor=True).astype(np.float64)
    Ws = skl.gemm_vta(V, A, tensor=False).astype(np.float64)
    # both within FP32 accumulation error of the exact product, and of each other
    assert np.max(np.abs(Wt - Ws) / bound) <= 2.0 ** -14
    # deterministic: a second call gives the same bits
    assert np.array_equal(skl.gemm_vta(V, A, tensor=True), Wt.astype(np.float32))


UPDATE_SHAPES = [(8500, 4936, 64, 64), (8500, 130, 64, 64), (1000, 300, 40, 40), (97, 130, 64, 0),
                 (33, 1, 64, 0), (4100, 1000, 8, 8)]


@pytest.mark.parametrize("shape", UPDATE_SHAPES)
def test_tensor_core_update_accuracy(shape):
    """C[r0:] -= V[r0:] Z (the trailing update): rows above r0 untouched, the
    rest within ~2^-21 of |C| + |V| |Z| entry by entry (FP32-class)."""
    M, N, b, r0 = shape
    rng = np.random.default_rng(M + 3 * N + b)
    V = rng.standard_normal((M, b)).astype(np.float32)
    Z = (rng.standard_normal((b, N)) * 10.0 ** rng.uniform(-2, 2, N)).astype(np.float32)
    C = (rng.standard_normal((M, N)) * 10.0 ** rng.uniform(-2, 2, N)).astype(np.float32)
    exact = C.astype(np.float64).copy()
    exact[r0:] -= V[r0:].astype(np.float64) @ Z.astype(np.float64)
    bound = np.abs(C.astype(np.float64))
    bound[r0:] += np.abs(V[r0:].astype(np.float64)) @ np.abs(Z.astype(np.float64))
    for tensor in (True, False):
        out = skl.gemm_update(C, V, Z, r0, tensor=tensor)
        assert np.array_equal(out[:r0], C[:r0]), (shape, tensor)
        rel = np.abs(out.astype(np.float64) - exact) / bound
        assert rel.max() <= 2.0 ** -20, (shape, tensor, rel.max())

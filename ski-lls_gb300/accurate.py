"""Residuals evaluated to full FP64 accuracy, for comparing least-squares
solutions whose residual is many orders of magnitude below ||A|| ||x||.

r_i = b_i - sum_j a_ij x_j is formed exactly: every product a_ij x_j is split
into p + e with p = fl(a_ij x_j) and e its exact rounding error (Dekker's
TwoProduct, no FMA needed), and each row's terms are summed by math.fsum,
which returns the correctly rounded sum.  So r is the correctly rounded exact
residual on every platform, whatever its long double is.
"""
import math

import numpy as np
import scipy.sparse as sp

_SPLIT = 134217729.0   # 2^27 + 1


def _split(a):
    c = _SPLIT * a
    hi = c - (c - a)
    return hi, a - hi


def two_product(a, b):
    """p, e with p = fl(a*b) and p + e == a*b exactly (no overflow/underflow)."""
    p = a * b
    ah, al = _split(a)
    bh, bl = _split(b)
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    return p, e


def residual(A, x, b):
    """Correctly rounded r = b - A x for a scipy sparse or dense A."""
    b = np.asarray(b, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    if sp.issparse(A):
        R = A.tocsr()
        R.sort_indices()
        p, e = two_product(R.data, x[R.indices])
        bounds = R.indptr[1:-1]
        ps = np.split(p, bounds)
        es = np.split(e, bounds)
        out = np.empty(R.shape[0])
        for i in range(R.shape[0]):
            out[i] = math.fsum(np.concatenate(([b[i]], -ps[i], -es[i])))
        return out
    A = np.asarray(A, dtype=np.float64)
    out = np.empty(A.shape[0])
    for i in range(A.shape[0]):
        p, e = two_product(A[i], x)
        out[i] = math.fsum(np.concatenate(([b[i]], -p, -e)))
    return out


def residual_norm(A, x, b):
    r = residual(A, x, b)
    return float(math.sqrt(math.fsum(r * r)))


def backward_error(A, x, b):
    """||A^T r|| / (||A||_F ||r||) with the correctly rounded r."""
    r = residual(A, x, b)
    nr = math.sqrt(math.fsum(r * r))
    if nr == 0.0:
        return 0.0
    if sp.issparse(A):
        g = A.T @ r
        fro = math.sqrt(math.fsum(A.data * A.data))
    else:
        g = np.asarray(A).T @ r
        fro = float(np.linalg.norm(A))
    return float(np.linalg.norm(g) / (fro * nr))

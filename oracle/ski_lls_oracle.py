"""CPU ORACLE for the Ski-LLS solve path -- test infrastructure only.

This module restates the reference's two solver entry points on the CPU so
that the GPU solver can be checked against them.  It is imported only by
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s ``cpu_baseline`` /
``--impl reference`` legs, always as the checker, never as the thing shipped.

Pieces and the reference code they follow:

* ``Rng``                       glibc ``rand()`` (TYPE_3), used by
                                src/sparse_helpers.cpp:74-115 and
                                src/dense_helpers.cpp:7-16 (C, skills_oracle.c)
* ``gen_hashing``               src/sparse_helpers.cpp:66-116 (C)
* ``sparse_sketch``             src/sketching.cpp:90-112 (C)
* ``dense_sketch``              src/sketching.cpp:39-62 (C)
* ``unitary_dht``               src/fast_unitary_transform.cpp:42-121 with the
                                FFTW_DHT kind of src/fftw_r2r.cpp:33-51,
                                restated with numpy's FFT (DHT = Re F - Im F)
* ``ls_sparse_spqr``            src/ls_sparse_spqr.cpp:79-214.  SuiteSparseQR
                                (third-party, absent) is replaced by LAPACK
                                dgeqp3 of the densified sketch with SPQR's
                                default rank tolerance; its R, pivots and rank
                                can differ from SPQR's (parity of those is
                                unpinned; x and residuals are compared).
* ``ls_dense_hashing_blendenpik`` src/ls_dense_hashing_blendenpik.cpp:23-149.
                                HQRRP (d >= 1000) is replaced by dgeqp3, which
                                is what the reference itself calls for d < 1000
                                (hqrrp/.../NoFLA_HQRRP_WY_blk_var4_skint.c:205-208).
* ``ls_dense_blendenpik``       src/ls_dense_blendenpik.cpp:21-70 with
                                rand_subsampled_dct / random_sample
                                (src/dense_helpers.cpp:19-59); dense_qr is
                                numpy's QR (LAPACK dgeqrf, as the reference)
* ``random_sample_rows``        select_k_from_n, src/sparse_helpers.cpp:74-86
* ``lsqr``                      src/IterSolver.cpp:160-305 (C)
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import time

import numpy as np
import scipy.linalg.lapack as lapack

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_i64p = ctypes.POINTER(ctypes.c_int64)
_f64p = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)


def build():
    """Compile the C restatement (gcc) into oracle/_build/liboracle.so."""
    subprocess.check_call(["make", "-s", "-C", _HERE, "liboracle"])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.orc_rng_seed.argtypes = [ctypes.c_void_p, ctypes.c_uint32]
        L.orc_rng_next.argtypes = [ctypes.c_void_p]
        L.orc_rng_next.restype = ctypes.c_int32
        L.orc_rng_size.restype = ctypes.c_size_t
        L.orc_rng_fill.argtypes = [ctypes.c_void_p, ctypes.c_int64, _i32p]
        L.orc_gen_hashing.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                      ctypes.c_int64, _i64p, _f64p]
        L.orc_rand_signs.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, _f64p]
        L.orc_sparse_sketch.argtypes = [ctypes.c_int64, ctypes.c_int64, _i64p, _i64p, _f64p,
                                        _f64p, ctypes.c_int64, ctypes.c_int64, _i64p, _f64p,
                                        _f64p, _f64p]
        L.orc_dense_sketch.argtypes = [ctypes.c_int64, ctypes.c_int64, _f64p, ctypes.c_int64,
                                       ctypes.c_int64, ctypes.c_int64, _i64p, _f64p, _f64p]
        L.orc_usolve.argtypes = [ctypes.c_int64, _f64p, ctypes.c_int64, _f64p,
                                 ctypes.c_int, ctypes.c_double]
        L.orc_utsolve.argtypes = L.orc_usolve.argtypes
        L.orc_lsqr.argtypes = [ctypes.c_int64, ctypes.c_int64, _i64p, _i64p, _f64p,
                               _f64p, ctypes.c_int64, _i64p, ctypes.c_int64, _f64p,
                               ctypes.c_int64, ctypes.c_int, ctypes.c_double, _f64p,
                               ctypes.c_double, ctypes.c_int64, _f64p,
                               ctypes.POINTER(ctypes.c_int), _i64p]
        L.orc_csc_residual.argtypes = [ctypes.c_int64, ctypes.c_int64, _i64p, _i64p, _f64p,
                                       _f64p, _f64p, _f64p]
        L.orc_dense_residual.argtypes = [ctypes.c_int64, ctypes.c_int64, _f64p, ctypes.c_int64,
                                         _f64p, _f64p, _f64p]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


class Rng:
    """glibc rand() stream; a fresh process starts from seed 1."""

    def __init__(self, seed: int = 1):
        self._buf = ctypes.create_string_buffer(lib().orc_rng_size())
        self.seed(seed)

    def seed(self, seed: int):
        lib().orc_rng_seed(self._buf, ctypes.c_uint32(seed & 0xFFFFFFFF))

    def next(self) -> int:
        return lib().orc_rng_next(self._buf)

    def fill(self, count: int) -> np.ndarray:
        out = np.empty(count, dtype=np.int32)
        lib().orc_rng_fill(self._buf, count, _p(out, _i32p))
        return out

    @property
    def handle(self):
        return self._buf


def gen_hashing(rng: Rng, m: int, n: int, k: int):
    """Hash rows (int64, n*k) and values (+-1/sqrt(k)) of an m x n s-hashing matrix."""
    rows = np.empty(n * k, dtype=np.int64)
    vals = np.empty(n * k, dtype=np.float64)
    rc = lib().orc_gen_hashing(rng.handle, m, n, k, _p(rows, _i64p), _p(vals, _f64p))
    if rc != 0:
        raise ValueError("gen_hashing: need 1 <= k <= m")
    return rows, vals


def rand_signs(rng: Rng, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.float64)
    lib().orc_rand_signs(rng.handle, n, 1.0, _p(out, _f64p))
    return out


def _csc(indptr, indices, data):
    return (np.ascontiguousarray(indptr, dtype=np.int64),
            np.ascontiguousarray(indices, dtype=np.int64),
            np.ascontiguousarray(data, dtype=np.float64))


def sparse_sketch(n, d, indptr, indices, data, b, m, k, rows, vals):
    """Dense m x d (Fortran order) S*A and S*b for CSC A."""
    Ap, Ai, Ax = _csc(indptr, indices, data)
    SA = np.empty((m, d), dtype=np.float64, order="F")
    Sb = np.empty(m, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    lib().orc_sparse_sketch(n, d, _p(Ap, _i64p), _p(Ai, _i64p), _p(Ax, _f64p), _p(bb, _f64p),
                            m, k, _p(rows, _i64p), _p(vals, _f64p), _p(SA, _f64p), _p(Sb, _f64p))
    return SA, Sb


def dense_sketch(Y, m, k, rows, vals):
    """alpha*S*Y with alpha = 1/sqrt(k) (net entries +-1/k), Fortran-order result."""
    Y = np.asfortranarray(Y, dtype=np.float64)
    N, d = Y.shape
    SA = np.empty((m, d), dtype=np.float64, order="F")
    lib().orc_dense_sketch(N, d, _p(Y, _f64p), max(N, 1), m, k, _p(rows, _i64p),
                           _p(vals, _f64p), _p(SA, _f64p))
    return SA


def unitary_dht(A, D, N=None):
    """y = DHT_N( [D * A; 0] / sqrt(N) ) column-wise; N = rows(A) unless a
    padded length is given (the reference pads in its wisdom mode,
    src/fast_unitary_transform.cpp:63-64, :98-99)."""
    A = np.asarray(A, dtype=np.float64)
    if A.ndim == 1:
        A = A[:, None]
    n = A.shape[0]
    N = n if N is None else N
    y = np.zeros((N, A.shape[1]))
    y[:n] = (1.0 / math.sqrt(N)) * D[:, None] * A
    F = np.fft.fft(y, axis=0)
    return np.asfortranarray(F.real - F.imag)


def dht_unscaled(x):
    """Plain DHT H[k] = sum_n x[n] cas(2 pi n k / N) along axis 0."""
    F = np.fft.fft(np.asarray(x, dtype=np.float64), axis=0)
    return F.real - F.imag


def usolve(R, x, success=1, perturb=1e-10):
    R = np.asfortranarray(R, dtype=np.float64)
    x = np.array(x, dtype=np.float64)
    r = R.shape[1]
    lib().orc_usolve(r, _p(R, _f64p), max(R.shape[0], 1), _p(x, _f64p), int(success), perturb)
    return x


def utsolve(R, x, success=1, perturb=1e-10):
    R = np.asfortranarray(R, dtype=np.float64)
    x = np.array(x, dtype=np.float64)
    r = R.shape[1]
    lib().orc_utsolve(r, _p(R, _f64p), max(R.shape[0], 1), _p(x, _f64p), int(success), perturb)
    return x


def lsqr(n, d, b, cols, R, tol, max_it, csc=None, dense=None, success=1, perturb=1e-10):
    """Preconditioned LSQR on A(:,cols) R^{-1}; returns (y, flag, it)."""
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    R = np.asfortranarray(R, dtype=np.float64)
    r = len(cols)
    y = np.zeros(r, dtype=np.float64)
    flag = ctypes.c_int(0)
    it = ctypes.c_int64(0)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    if csc is not None:
        Ap, Ai, Ax = _csc(*csc)
        args = (_p(Ap, _i64p), _p(Ai, _i64p), _p(Ax, _f64p), None, 0)
    else:
        Ad = np.asfortranarray(dense, dtype=np.float64)
        args = (None, None, None, _p(Ad, _f64p), max(Ad.shape[0], 1))
    lib().orc_lsqr(n, d, *args, _p(cols, _i64p), r, _p(R, _f64p), max(R.shape[0], 1),
                   int(success), perturb, _p(bb, _f64p), tol, max_it, _p(y, _f64p),
                   ctypes.byref(flag), ctypes.byref(it))
    return y, flag.value, it.value


def csc_residual(n, d, indptr, indices, data, x, b):
    Ap, Ai, Ax = _csc(indptr, indices, data)
    r = np.empty(n, dtype=np.float64)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    lib().orc_csc_residual(n, d, _p(Ap, _i64p), _p(Ai, _i64p), _p(Ax, _f64p), _p(xx, _f64p),
                           _p(bb, _f64p), _p(r, _f64p))
    return r


def _cpqr(SA):
    """LAPACK dgeqp3: returns (QR, jpvt 0-based, tau)."""
    qr, jpvt, tau, work, info = lapack.dgeqp3(np.asfortranarray(SA), overwrite_a=1)
    if info != 0:
        raise RuntimeError(f"dgeqp3 info={info}")
    return qr, np.asarray(jpvt, dtype=np.int64) - 1, tau


def _apply_qt(qr, tau, c):
    """c <- Q^T c via dormqr('L','T'), src/ls_dense_hashing_blendenpik.cpp:70-76."""
    cq, work, info = lapack.dormqr("L", "T", qr, tau, c.reshape(-1, 1).copy(order="F"),
                                   max(1, 64 * qr.shape[1]))
    if info != 0:
        raise RuntimeError(f"dormqr info={info}")
    return cq[:, 0]


def spqr_default_tol(SA):
    """SuiteSparseQR's SPQR_DEFAULT_TOL: 20*(m+n)*eps*max column 2-norm."""
    m, d = SA.shape
    maxnorm = float(np.max(np.linalg.norm(SA, axis=0))) if d else 0.0
    return 20.0 * (m + d) * np.finfo(np.float64).eps * maxnorm


def ls_sparse_spqr(n, d, indptr, indices, data, b, gamma, k, abs_tol=1e-8, it_tol=1e-6,
                   max_it=10000, rcond_threshold=1e-10, perturb=1e-10, rng=None):
    """Restates ls_sparse_spqr (src/ls_sparse_spqr.cpp:79-214) on the CPU."""
    if n < d:
        raise RuntimeError("Matrix is not overdetermined.")
    if rng is None:
        rng = Rng(1)
    t0 = time.perf_counter()
    m = int(math.ceil(d * gamma))
    rows, vals = gen_hashing(rng, m, n, k)
    SA, Sb = sparse_sketch(n, d, indptr, indices, data, b, m, k, rows, vals)
    t1 = time.perf_counter()
    qr, E, tau = _cpqr(SA)
    c = _apply_qt(qr, tau, Sb)
    diag = np.abs(np.diag(qr))
    tol = spqr_default_tol(SA)
    rank = 0
    while rank < min(m, d) and diag[rank] > tol:
        rank += 1
    if rank == 0:
        raise RuntimeError("SPQR Factorization fails")
    R11 = np.asfortranarray(np.triu(qr[:rank, :rank]))
    rcond, info = lapack.dtrcon(R11, norm="I", uplo="U", diag="N")
    success = 1 if rcond > rcond_threshold else 0
    # explicit sketch solution, x[E[i]] = (R11^{-1} c)[i] (:144-151)
    cs = usolve(R11, c[:rank], 1, perturb)
    x = np.zeros(d)
    x[E[:rank]] = cs
    r_s = csc_residual(n, d, indptr, indices, data, x, b)
    res = float(np.linalg.norm(r_s))
    t2 = time.perf_counter()
    out = dict(m=m, rank=rank, success=success, rcond=float(rcond), E=E, rows=rows, vals=vals,
               SA=SA, Sb=Sb, tol=tol, explicit_residual=res,
               phases_s=dict(sketch=t1 - t0, qr=t2 - t1, lsqr=0.0))
    if res < abs_tol:
        out.update(x=x, flag=0, it=0)
        return out
    y, flag, it = lsqr(n, d, r_s, E[:rank], R11, it_tol, max_it,
                       csc=(indptr, indices, data), success=success, perturb=perturb)
    # y = R11^{-1} y + c, x = P y (:188-208); the reference's final usolve
    # uses the default arguments (success=1).
    y = usolve(R11, y, 1, perturb) + cs
    x = np.zeros(d)
    x[E[:rank]] = y
    out["phases_s"]["lsqr"] = time.perf_counter() - t2
    out.update(x=x, flag=flag, it=it)
    return out


def ls_dense_hashing_blendenpik(A, b, gamma, k, abs_tol=1e-8, rcond=1e-10, it_tol=1e-6,
                                max_it=10000, seed=1, N=None):
    """Restates ls_dense_hashing_blendenpik (src/ls_dense_hashing_blendenpik.cpp:23-149).

    The reference seeds with srand(time(NULL)) (src/dense_helpers.cpp:92, :12);
    the oracle takes that seed as an argument.
    """
    A = np.asfortranarray(A, dtype=np.float64)
    n, d = A.shape
    if n < d:
        raise RuntimeError("Matrix is not overdetermined.")
    t0 = time.perf_counter()
    m = int(math.ceil(d * gamma))
    N = n if N is None else N
    rng = Rng(seed)
    D = rand_signs(rng, n)
    Y = unitary_dht(A, D, N)
    yb = unitary_dht(np.asarray(b, dtype=np.float64), D, N)[:, 0]
    rows, vals = gen_hashing(rng, m, N, k)
    SA = dense_sketch(Y, m, k, rows, vals)
    Sb = dense_sketch(yb[:, None], m, k, rows, vals)[:, 0]
    del Y
    t1 = time.perf_counter()
    qr, E, tau = _cpqr(SA.copy(order="F"))
    c = _apply_qt(qr, tau, Sb)
    rank = 0
    while rank < d and abs(qr[rank, rank]) > rcond:
        rank += 1
    R = np.asfortranarray(np.triu(qr[:rank, :rank]))
    cs = usolve(R, c[:rank], 1, 0.0) if rank else np.zeros(0)
    x = np.zeros(d)
    x[E[:rank]] = cs
    rs = np.asarray(b, dtype=np.float64) - A @ x
    res = float(np.linalg.norm(rs))
    t2 = time.perf_counter()
    out = dict(m=m, rank=rank, E=E, D=D, rows=rows, vals=vals, SA=SA, Sb=Sb,
               explicit_residual=res, phases_s=dict(sketch=t1 - t0, qr=t2 - t1, lsqr=0.0))
    if res < abs_tol:
        out.update(x=x, flag=0, it=0)
        return out
    xs = x.copy()
    y, flag, it = lsqr(n, d, rs, E[:rank], R, it_tol, max_it, dense=A)
    y = usolve(R, y, 1, 0.0)
    x = np.zeros(d)
    x[E[:rank]] = y
    x = xs + x
    out["phases_s"]["lsqr"] = time.perf_counter() - t2
    out.update(x=x, flag=flag, it=it)
    return out


def ls_dense_hashing_blendenpik_noCPQR(A, b, gamma, k, it_tol=1e-6, max_it=10000, seed=1,
                                       N=None):
    """Restates ls_dense_hashing_blendenpik_noCPQR
    (src/ls_dense_hashing_blendenpik_noCPQR.cpp:23-59): sketch A only, unpivoted
    QR (dense_qr, src/dense_qr.cpp:8-32), LSQR on (A, b) from zero, x = R^{-1} y."""
    A = np.asfortranarray(A, dtype=np.float64)
    n, d = A.shape
    if n < d:
        raise RuntimeError("Matrix is not overdetermined.")
    m = int(math.ceil(d * gamma))
    N = n if N is None else N
    rng = Rng(seed)
    D = rand_signs(rng, n)
    Y = unitary_dht(A, D, N)
    rows, vals = gen_hashing(rng, m, N, k)
    SA = dense_sketch(Y, m, k, rows, vals)
    R = np.asfortranarray(np.linalg.qr(SA, mode="r")[:d, :d])
    y, flag, it = lsqr(n, d, np.asarray(b, dtype=np.float64), np.arange(d), R, it_tol, max_it,
                       dense=A)
    x = usolve(R, y, 1, 0.0)
    return dict(m=m, rank=d, x=x, flag=flag, it=it, SA=SA)


def random_sample_rows(rng: Rng, N: int, m: int) -> np.ndarray:
    """Rows random_sample keeps (src/dense_helpers.cpp:19-39): gen_0_to_n(N),
    then select_k_from_n(N, m) (src/sparse_helpers.cpp:74-86), the first m
    entries of the partially shuffled array."""
    if not 0 <= m <= N:
        raise ValueError("random_sample: need 0 <= m <= N")
    idx = np.arange(N, dtype=np.int64)
    for i in range(m):
        j = rng.next() % (N - i) + i
        idx[i], idx[j] = idx[j], idx[i]
    return idx[:m].copy()


def ls_dense_blendenpik(A, b, gamma, it_tol=1e-6, max_it=10000, seed=1, N=None):
    """Restates ls_dense_blendenpik (src/ls_dense_blendenpik.cpp:21-70):
    rand_subsampled_dct (src/dense_helpers.cpp:42-59) -- signs from the stream
    seeded with `seed`, the orthonormal DHT, then m = ceil(gamma d) rows drawn
    from the stream seeded again with the same value (the reference calls
    srand(time(NULL)) before each) --, unpivoted QR (dense_qr), LSQR on (A, b)
    from zero preconditioned by R, x = R^{-1} y, rank = d."""
    A = np.asfortranarray(A, dtype=np.float64)
    n, d = A.shape
    if n < d:
        raise RuntimeError("Matrix is not overdetermined.")
    m = int(math.ceil(d * gamma))
    N = n if N is None else N
    t0 = time.perf_counter()
    rng = Rng(seed)
    D = rand_signs(rng, n)
    Y = unitary_dht(A, D, N)
    rng.seed(seed)
    rows = random_sample_rows(rng, N, m)
    SA = np.asfortranarray(Y[rows, :])
    t1 = time.perf_counter()
    R = np.asfortranarray(np.linalg.qr(SA, mode="r")[:d, :d])
    t2 = time.perf_counter()
    y, flag, it = lsqr(n, d, np.asarray(b, dtype=np.float64), np.arange(d), R, it_tol, max_it,
                       dense=A)
    x = usolve(R, y, 1, 0.0)
    t3 = time.perf_counter()
    return dict(m=m, rank=d, x=x, flag=flag, it=it, SA=SA, rows=rows,
                phases_s={"sketch": t1 - t0, "qr": t2 - t1, "lsqr": t3 - t2})


def backward_error(A_mv, A_rmv, fro, x, b):
    """||A^T r|| / (||A||_F ||r||) with r = b - A x."""
    r = b - A_mv(x)
    nr = float(np.linalg.norm(r))
    if nr == 0.0:
        return 0.0
    return float(np.linalg.norm(A_rmv(r))) / (fro * nr)

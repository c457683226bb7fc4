"""Python host interface of the GB300 Ski-LLS solver (ctypes over the C ABI).

Mirrors the reference's entry points (include/ski-lls.h:15-28):

    ls_sparse_spqr(A, b, gamma, k, abs_tol, ordering, it_tol, max_it,
                   rcond_threshold, perturb, debug)          -> Result
    ls_dense_hashing_blendenpik(A, b, gamma, k, abs_tol, rcond, it_tol,
                                max_it, debug, wisdom)       -> Result
    ls_dense_hashing_blendenpik_noCPQR(A, b, gamma, k, it_tol, max_it,
                                       debug, wisdom)        -> Result

Result carries x and the reference's output arguments (rank, flag, it) plus
the solver's diagnostics.  Errors raise RuntimeError with the reference's
messages ("Matrix is not overdetermined.", "SPQR Factorization fails").
There is no CPU fallback: if libskills_gb300.so is missing or no GB300 is
visible, the calls raise.
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("SKILLS_LIB", os.path.join(_HERE, "lib", "libskills_gb300.so"))

SKL_OK = 0
SKL_ERR_INVALID = 1
SKL_ERR_NOT_OVERDETERMINED = 2
SKL_ERR_RANK_ZERO = 3
SKL_ERR_CUDA = 4
SKL_ERR_NO_DEVICE = 5
SKL_ERR_TIMEOUT = 6
SKL_ERR_ALLOC = 7
SKL_ERR_NONFINITE = 8

PREC = {"mixed": 0, "fp64": 1}

# include/bench_config.hpp:7-20
IT_TOL = 1e-6
MAX_IT = 10000
OVER_SAMPLING_RATIO = 1.1
NNZ_PER_COLUMN = 3
PERTURB = 1e-10
RCOND_THRESHOLD = 1e-10
ABS_TOL = 1e-8
SPQR_ORDERING = 2


class SklCsc(ctypes.Structure):
    _fields_ = [("m", ctypes.c_int64), ("n", ctypes.c_int64), ("nzmax", ctypes.c_int64),
                ("p", ctypes.c_void_p), ("i", ctypes.c_void_p), ("x", ctypes.c_void_p)]


class SklOpts(ctypes.Structure):
    _fields_ = [("gamma", ctypes.c_double), ("k", ctypes.c_int64), ("abs_tol", ctypes.c_double),
                ("it_tol", ctypes.c_double), ("max_it", ctypes.c_int64),
                ("rcond_threshold", ctypes.c_double), ("perturb", ctypes.c_double),
                ("rcond", ctypes.c_double), ("rank_tol", ctypes.c_double),
                ("precision", ctypes.c_int), ("use_cpqr", ctypes.c_int),
                ("seed_mode", ctypes.c_int), ("seed", ctypes.c_uint32), ("wisdom", ctypes.c_int),
                ("backward_tol", ctypes.c_double), ("max_refine", ctypes.c_int64),
                ("device", ctypes.c_int), ("stream", ctypes.c_void_p), ("profile", ctypes.c_int),
                ("autotune", ctypes.c_int)]


class SklInfo(ctypes.Structure):
    _fields_ = [("rank", ctypes.c_int64), ("flag", ctypes.c_int), ("it", ctypes.c_int64),
                ("success", ctypes.c_int), ("sketch_rows", ctypes.c_int64),
                ("rcond_r11", ctypes.c_double), ("explicit_residual", ctypes.c_double),
                ("residual_norm", ctypes.c_double), ("backward_error", ctypes.c_double),
                ("t_total_ms", ctypes.c_double), ("t_upload_ms", ctypes.c_double),
                ("t_setup_ms", ctypes.c_double), ("t_sketch_ms", ctypes.c_double),
                ("t_qr_ms", ctypes.c_double), ("t_precond_ms", ctypes.c_double),
                ("t_lsqr_ms", ctypes.c_double), ("t_host_hash_ms", ctypes.c_double),
                ("kernel_launches", ctypes.c_int64), ("prof_ms", ctypes.c_double * 4),
                ("prof_launches", ctypes.c_int64 * 4), ("qr_prof_ms", ctypes.c_double * 9),
                ("sketch_refine_steps", ctypes.c_int64), ("unresolved_cols", ctypes.c_int64),
                ("fp64_fallback", ctypes.c_int), ("tuned", ctypes.c_int64 * 4)]

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if isinstance(v, ctypes.Array) else v
        return out


_lib = None


def lib():
    """Load libskills_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        L = ctypes.CDLL(LIB_PATH)
        vp, i64, dbl = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double
        L.skl_default_opts.argtypes = [ctypes.POINTER(SklOpts)]
        L.skl_last_error.restype = ctypes.c_char_p
        L.skl_version.restype = ctypes.c_char_p
        L.skl_srand.argtypes = [ctypes.c_uint32]
        for name in ("skl_sparse_solve", "skl_sparse_solve_device"):
            f = getattr(L, name)
            f.argtypes = [ctypes.POINTER(SklCsc), vp, vp, ctypes.POINTER(SklOpts),
                          ctypes.POINTER(SklInfo)]
            f.restype = ctypes.c_int
        L.skl_batched_sparse_solve.argtypes = [i64, ctypes.POINTER(SklCsc), vp, vp,
                                               ctypes.POINTER(SklOpts), ctypes.POINTER(SklInfo), vp]
        L.skl_batched_sparse_solve.restype = ctypes.c_int
        for name in ("skl_dense_solve", "skl_dense_solve_device", "skl_dense_blendenpik_solve",
                     "skl_dense_blendenpik_solve_device"):
            f = getattr(L, name)
            f.argtypes = [vp, i64, i64, i64, vp, vp, ctypes.POINTER(SklOpts),
                          ctypes.POINTER(SklInfo)]
            f.restype = ctypes.c_int
        L.skl_hash_generate.argtypes = [i64, i64, i64, ctypes.c_int, ctypes.c_uint32, vp, vp]
        L.skl_hash_generate.restype = ctypes.c_int
        L.skl_subsample_rows.argtypes = [i64, i64, ctypes.c_int, ctypes.c_uint32, vp]
        L.skl_subsample_rows.restype = ctypes.c_int
        L.skl_sketch_sparse.argtypes = [ctypes.POINTER(SklCsc), vp, i64, i64, vp, vp, ctypes.c_int,
                                        ctypes.c_int, vp, vp]
        L.skl_sketch_sparse.restype = ctypes.c_int
        L.skl_dht.argtypes = [vp, i64, i64, i64, vp, i64, ctypes.c_int, vp]
        L.skl_dht.restype = ctypes.c_int
        L.skl_dht_device_noalloc.argtypes = [vp, i64, i64, i64, vp, i64, ctypes.c_int, vp, i64,
                                             vp]
        L.skl_dht_device_noalloc.restype = ctypes.c_int
        L.skl_dht_length.argtypes = [i64, ctypes.c_int]
        L.skl_dht_length.restype = i64
        L.skl_sketch_dense.argtypes = [vp, i64, i64, i64, vp, vp, i64, i64, i64, vp, vp,
                                       ctypes.c_int, vp, vp]
        L.skl_sketch_dense.restype = ctypes.c_int
        L.skl_cpqr.argtypes = [vp, i64, i64, ctypes.c_int, vp, vp]
        L.skl_cpqr.restype = ctypes.c_int
        L.skl_trsv_upper.argtypes = [vp, i64, i64, ctypes.c_char, ctypes.c_int, vp]
        L.skl_trsv_upper.restype = ctypes.c_int
        L.skl_csc_mv.argtypes = [ctypes.POINTER(SklCsc), ctypes.c_char, vp, vp, ctypes.c_int]
        L.skl_csc_mv.restype = ctypes.c_int
        L.skl_gemm_vta.argtypes = [i64, i64, i64, vp, i64, vp, i64, vp, ctypes.c_int]
        L.skl_gemm_vta.restype = ctypes.c_int
        L.skl_gemm_update.argtypes = [i64, i64, i64, i64, vp, i64, vp, i64, vp, i64, ctypes.c_int]
        L.skl_gemm_update.restype = ctypes.c_int
        _lib = L
    return _lib


def last_error() -> str:
    return lib().skl_last_error().decode()


class SklError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


def _check(rc):
    if rc != SKL_OK:
        raise SklError(rc, last_error())


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else ctypes.c_void_p(0)


def default_opts() -> SklOpts:
    o = SklOpts()
    lib().skl_default_opts(ctypes.byref(o))
    return o


@dataclass
class Result:
    x: np.ndarray
    rank: int
    flag: int
    it: int
    info: dict = field(default_factory=dict)


def _as_csc(A):
    """(indptr, indices, data, shape) with int64 indices, from a scipy matrix or a tuple."""
    if hasattr(A, "tocsc"):
        C = A.tocsc()
        return (np.ascontiguousarray(C.indptr, dtype=np.int64),
                np.ascontiguousarray(C.indices, dtype=np.int64),
                np.ascontiguousarray(C.data, dtype=np.float64), C.shape)
    indptr, indices, data, shape = A
    return (np.ascontiguousarray(indptr, dtype=np.int64),
            np.ascontiguousarray(indices, dtype=np.int64),
            np.ascontiguousarray(data, dtype=np.float64), tuple(int(s) for s in shape))


def ls_sparse_spqr(A, b, gamma=OVER_SAMPLING_RATIO, k=NNZ_PER_COLUMN, abs_tol=ABS_TOL,
                   ordering=SPQR_ORDERING, it_tol=IT_TOL, max_it=MAX_IT,
                   rcond_threshold=RCOND_THRESHOLD, perturb=PERTURB, debug=0, *,
                   precision="mixed", seed=None, backward_tol=0.0, max_refine=3,
                   rank_tol=0.0, device=0, stream=None, profile=0, autotune=0) -> Result:
    """GPU counterpart of ls_sparse_spqr (src/ls_sparse_spqr.cpp:79-214).

    `ordering` and `debug` are accepted for signature parity (the GPU path
    factorizes the sketch densely; SPQR's fill-reducing ordering has no role).
    seed=None continues the library's glibc-compatible stream (a fresh process
    is seed 1, like the reference); an integer reseeds first.
    """
    indptr, indices, data, (n, d) = _as_csc(A)
    b = np.ascontiguousarray(b, dtype=np.float64)
    if b.shape != (n,):
        raise ValueError("b must have A.m entries")
    x = np.zeros(d, dtype=np.float64)
    csc = SklCsc(n, d, int(indptr[-1]) if len(indptr) else 0, indptr.ctypes.data,
                 indices.ctypes.data if indices.size else 0, data.ctypes.data if data.size else 0)
    o = default_opts()
    o.gamma, o.k, o.abs_tol, o.it_tol, o.max_it = gamma, k, abs_tol, it_tol, max_it
    o.rcond_threshold, o.perturb, o.precision = rcond_threshold, perturb, PREC[precision]
    o.seed_mode, o.seed = (0, 0) if seed is None else (1, int(seed) & 0xFFFFFFFF)
    o.backward_tol, o.max_refine, o.rank_tol, o.device = backward_tol, max_refine, rank_tol, device
    o.stream, o.profile, o.autotune = stream, profile, autotune
    info = SklInfo()
    _check(lib().skl_sparse_solve(ctypes.byref(csc), _ptr(b), _ptr(x), ctypes.byref(o),
                                  ctypes.byref(info)))
    return Result(x, info.rank, info.flag, info.it, info.as_dict())


def sparse_solve_device(n, d, p_ptr, i_ptr, x_ptr, b_ptr, xout_ptr, nnz, gamma, k, *,
                        precision="mixed", seed=None, it_tol=IT_TOL, max_it=MAX_IT,
                        abs_tol=ABS_TOL, backward_tol=0.0, stream=None, profile=0,
                        device=0, autotune=0) -> SklInfo:
    """skl_sparse_solve_device on device pointers (CSC with int64 indices)."""
    csc = SklCsc(n, d, nnz, p_ptr, i_ptr, x_ptr)
    o = default_opts()
    o.gamma, o.k, o.abs_tol, o.it_tol, o.max_it = gamma, k, abs_tol, it_tol, max_it
    o.precision = PREC[precision]
    o.seed_mode, o.seed = (0, 0) if seed is None else (1, int(seed) & 0xFFFFFFFF)
    o.backward_tol, o.device, o.stream, o.profile = backward_tol, device, stream, profile
    o.autotune = autotune
    info = SklInfo()
    _check(lib().skl_sparse_solve_device(ctypes.byref(csc), ctypes.c_void_p(b_ptr),
                                         ctypes.c_void_p(xout_ptr), ctypes.byref(o),
                                         ctypes.byref(info)))
    return info


def dense_solve_device(n, d, a_ptr, lda, b_ptr, xout_ptr, gamma, k, *, precision="mixed",
                       seed=1, rcond=1e-10, it_tol=IT_TOL, max_it=MAX_IT, abs_tol=ABS_TOL,
                       use_cpqr=1, stream=None, profile=0, device=0) -> SklInfo:
    """skl_dense_solve_device on device pointers (column-major A, lda >= n)."""
    o = default_opts()
    o.gamma, o.k, o.abs_tol, o.it_tol, o.max_it, o.rcond = gamma, k, abs_tol, it_tol, max_it, rcond
    o.precision = PREC[precision]
    o.seed_mode, o.seed = 1, int(seed) & 0xFFFFFFFF
    o.use_cpqr, o.device, o.stream, o.profile = use_cpqr, device, stream, profile
    info = SklInfo()
    _check(lib().skl_dense_solve_device(ctypes.c_void_p(a_ptr), lda, n, d, ctypes.c_void_p(b_ptr),
                                        ctypes.c_void_p(xout_ptr), ctypes.byref(o),
                                        ctypes.byref(info)))
    return info


def batched_sparse_spqr(problems, gamma=OVER_SAMPLING_RATIO, k=NNZ_PER_COLUMN, *,
                        abs_tol=ABS_TOL, it_tol=IT_TOL, max_it=MAX_IT, precision="mixed",
                        seed=None, backward_tol=0.0, max_refine=3, device=0):
    """skl_batched_sparse_solve over [(A, b), ...] (scipy CSC, host arrays).
    Returns (list of x, list of SklInfo, list of status codes)."""
    nprob = len(problems)
    keep = []
    cscs = (SklCsc * max(nprob, 1))()
    bptr = (ctypes.c_void_p * max(nprob, 1))()
    xptr = (ctypes.c_void_p * max(nprob, 1))()
    xs = []
    for p, (A, b) in enumerate(problems):
        A = A.tocsc()
        ip = np.ascontiguousarray(A.indptr, dtype=np.int64)
        ii = np.ascontiguousarray(A.indices, dtype=np.int64)
        xx = np.ascontiguousarray(A.data, dtype=np.float64)
        bb = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(A.shape[1], dtype=np.float64)
        keep += [ip, ii, xx, bb]
        xs.append(x)
        cscs[p] = SklCsc(A.shape[0], A.shape[1], int(A.nnz), _ptr(ip).value, _ptr(ii).value,
                         _ptr(xx).value)
        bptr[p] = _ptr(bb).value
        xptr[p] = _ptr(x).value
    o = default_opts()
    o.gamma, o.k, o.abs_tol, o.it_tol, o.max_it = gamma, k, abs_tol, it_tol, max_it
    o.precision = PREC[precision]
    o.seed_mode, o.seed = (0, 0) if seed is None else (1, int(seed) & 0xFFFFFFFF)
    o.backward_tol, o.max_refine = backward_tol, max_refine
    o.device = device
    infos = (SklInfo * max(nprob, 1))()
    status = (ctypes.c_int * max(nprob, 1))()
    rc = lib().skl_batched_sparse_solve(nprob, cscs, ctypes.cast(bptr, ctypes.c_void_p),
                                        ctypes.cast(xptr, ctypes.c_void_p), ctypes.byref(o),
                                        infos, ctypes.cast(status, ctypes.c_void_p))
    _check(rc)
    return xs, [infos[p] for p in range(nprob)], [status[p] for p in range(nprob)]


def ls_dense_hashing_blendenpik(A, b, gamma=OVER_SAMPLING_RATIO, k=NNZ_PER_COLUMN,
                                abs_tol=ABS_TOL, rcond=1e-10, it_tol=IT_TOL, max_it=MAX_IT,
                                debug=0, wisdom=0, *, precision="mixed", seed=0,
                                backward_tol=0.0, max_refine=3, use_cpqr=1,
                                device=0, stream=None, profile=0) -> Result:
    """GPU counterpart of ls_dense_hashing_blendenpik
    (src/ls_dense_hashing_blendenpik.cpp:23-149).  seed=0 seeds from time(NULL)
    like the reference (src/dense_helpers.cpp:92); pass a seed to reproduce."""
    A = np.asfortranarray(A, dtype=np.float64)
    n, d = A.shape
    b = np.ascontiguousarray(b, dtype=np.float64)
    if b.shape != (n,):
        raise ValueError("b must have A.m entries")
    x = np.zeros(d, dtype=np.float64)
    o = default_opts()
    o.gamma, o.k, o.abs_tol, o.rcond, o.it_tol, o.max_it = gamma, k, abs_tol, rcond, it_tol, max_it
    o.wisdom, o.precision, o.seed_mode, o.seed = wisdom, PREC[precision], 1, int(seed) & 0xFFFFFFFF
    o.backward_tol, o.max_refine, o.use_cpqr, o.device = backward_tol, max_refine, use_cpqr, device
    o.stream, o.profile = stream, profile
    info = SklInfo()
    _check(lib().skl_dense_solve(_ptr(A), max(n, 1), n, d, _ptr(b), _ptr(x), ctypes.byref(o),
                                 ctypes.byref(info)))
    return Result(x, info.rank, info.flag, info.it, info.as_dict())


def ls_dense_hashing_blendenpik_noCPQR(A, b, gamma=OVER_SAMPLING_RATIO, k=NNZ_PER_COLUMN,
                                       it_tol=IT_TOL, max_it=MAX_IT, debug=0, wisdom=0,
                                       **kw) -> Result:
    """GPU counterpart of ls_dense_hashing_blendenpik_noCPQR
    (src/ls_dense_hashing_blendenpik_noCPQR.cpp:23-60): unpivoted QR, LSQR from 0."""
    return ls_dense_hashing_blendenpik(A, b, gamma, k, abs_tol=0.0, rcond=0.0, it_tol=it_tol,
                                       max_it=max_it, debug=debug, wisdom=wisdom, use_cpqr=0, **kw)


def ls_dense_blendenpik(A, b, gamma=2.2, it_tol=IT_TOL, max_it=MAX_IT, debug=0, wisdom=0, *,
                        precision="mixed", seed=0, device=0, stream=None, profile=0) -> Result:
    """GPU counterpart of Blendenpik, ls_dense_blendenpik (src/ls_dense_blendenpik.cpp:21-70):
    m = ceil(gamma*d) rows of the randomized DHT of A drawn without replacement
    (rand_subsampled_dct, src/dense_helpers.cpp:42-59), unpivoted QR, LSQR
    preconditioned by R from 0, rank = d.  gamma defaults to the reference
    driver's 2.2 (test/ls_blendenpik.cpp:61).  seed=0 seeds from time(NULL)."""
    A = np.asfortranarray(A, dtype=np.float64)
    n, d = A.shape
    b = np.ascontiguousarray(b, dtype=np.float64)
    if b.shape != (n,):
        raise ValueError("b must have A.m entries")
    x = np.zeros(d, dtype=np.float64)
    o = default_opts()
    o.gamma, o.it_tol, o.max_it, o.wisdom = gamma, it_tol, max_it, wisdom
    o.precision, o.seed_mode, o.seed = PREC[precision], 1, int(seed) & 0xFFFFFFFF
    o.device, o.stream, o.profile = device, stream, profile
    info = SklInfo()
    _check(lib().skl_dense_blendenpik_solve(_ptr(A), max(n, 1), n, d, _ptr(b), _ptr(x),
                                            ctypes.byref(o), ctypes.byref(info)))
    return Result(x, info.rank, info.flag, info.it, info.as_dict())


def dense_blendenpik_device(n, d, a_ptr, lda, b_ptr, xout_ptr, gamma, *, precision="mixed",
                            seed=1, it_tol=IT_TOL, max_it=MAX_IT, stream=None, profile=0,
                            device=0) -> SklInfo:
    """skl_dense_blendenpik_solve_device on device pointers (column-major A, lda >= n)."""
    o = default_opts()
    o.gamma, o.it_tol, o.max_it = gamma, it_tol, max_it
    o.precision = PREC[precision]
    o.seed_mode, o.seed = 1, int(seed) & 0xFFFFFFFF
    o.device, o.stream, o.profile = device, stream, profile
    info = SklInfo()
    _check(lib().skl_dense_blendenpik_solve_device(ctypes.c_void_p(a_ptr), lda, n, d,
                                                   ctypes.c_void_p(b_ptr), ctypes.c_void_p(xout_ptr),
                                                   ctypes.byref(o), ctypes.byref(info)))
    return info


def subsample_rows(N, m, seed=None):
    """The m rows (of N, int64, draw order) random_sample keeps (src/dense_helpers.cpp:19-39)."""
    rows = np.empty(m, dtype=np.int64)
    mode, sd = (0, 0) if seed is None else (1, int(seed) & 0xFFFFFFFF)
    _check(lib().skl_subsample_rows(N, m, mode, sd, _ptr(rows)))
    return rows


def hash_generate(m, n, k, seed=None):
    """Rows (int64, n*k) and values (+-1/sqrt(k)) of the s-hashing matrix."""
    rows = np.empty(n * k, dtype=np.int64)
    vals = np.empty(n * k, dtype=np.float64)
    mode, sd = (0, 0) if seed is None else (1, int(seed) & 0xFFFFFFFF)
    _check(lib().skl_hash_generate(m, n, k, mode, sd, _ptr(rows), _ptr(vals)))
    return rows, vals


def srand(seed):
    lib().skl_srand(int(seed) & 0xFFFFFFFF)


def sketch_sparse(A, b, m, k, rows, vals, precision="mixed", equilibrate=False):
    indptr, indices, data, (n, d) = _as_csc(A)
    csc = SklCsc(n, d, int(indptr[-1]), indptr.ctypes.data,
                 indices.ctypes.data if indices.size else 0, data.ctypes.data if data.size else 0)
    SA = np.zeros((m, d), dtype=np.float64, order="F")
    Sb = np.zeros(m, dtype=np.float64)
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    _check(lib().skl_sketch_sparse(ctypes.byref(csc), _ptr(bb), m, k, _ptr(rows), _ptr(vals),
                                   PREC[precision], int(equilibrate), _ptr(SA), _ptr(Sb)))
    return SA, Sb


def cpqr(A, precision="mixed"):
    """Randomized CPQR on the GPU: returns (QR, jpvt 0-based, tau)."""
    QR = np.array(A, dtype=np.float64, order="F", copy=True)
    m, d = QR.shape
    jpvt = np.zeros(d, dtype=np.int64)
    tau = np.zeros(min(m, d), dtype=np.float64)
    _check(lib().skl_cpqr(_ptr(QR), m, d, PREC[precision], _ptr(jpvt), _ptr(tau)))
    return QR, jpvt, tau


def trsv_upper(R, x, trans="n", precision="mixed"):
    R = np.asfortranarray(R, dtype=np.float64)
    xx = np.array(x, dtype=np.float64, copy=True)
    r = R.shape[1]
    _check(lib().skl_trsv_upper(_ptr(R), max(R.shape[0], 1), r, trans.encode(), PREC[precision],
                                _ptr(xx)))
    return xx


def csc_mv(A, x, trans="n", precision="mixed"):
    """y = A x ('n') or A^T x ('t') through the solve's LSQR product kernels
    (mixed: equilibrated float-pair storage, float-float accumulation)."""
    indptr, indices, data, shape = _as_csc(A)
    n, d = shape
    xx = np.ascontiguousarray(x, dtype=np.float64)
    if xx.shape != ((d,) if trans == "n" else (n,)):
        raise ValueError("x has the wrong length")
    y = np.zeros(n if trans == "n" else d, dtype=np.float64)
    csc = SklCsc(n, d, int(indptr[-1]), indptr.ctypes.data, indices.ctypes.data, data.ctypes.data)
    _check(lib().skl_csc_mv(ctypes.byref(csc), trans.encode(), _ptr(xx), _ptr(y), PREC[precision]))
    return y


def gemm_vta(V, A, tensor=True):
    """W = V^T A in FP32 through the CPQR's block-reflector product
    (tensor=True: tcgen05 3xTF32 kernel; False: CUDA-core FP32 kernel)."""
    V = np.asfortranarray(V, dtype=np.float32)
    A = np.asfortranarray(A, dtype=np.float32)
    M, b = V.shape
    if A.shape[0] != M:
        raise ValueError("V and A need the same number of rows")
    N = A.shape[1]
    W = np.zeros((b, N), dtype=np.float32, order="F")
    _check(lib().skl_gemm_vta(M, N, b, _ptr(V), M, _ptr(A), M, _ptr(W), 1 if tensor else 0))
    return W


def gemm_update(C, V, Z, r0=0, tensor=True):
    """C[r0:, :] - V[r0:, :] Z in FP32 (returns a new array) through the CPQR's
    trailing-update product (tensor=True: tcgen05 3xTF32 kernel)."""
    C = np.array(C, dtype=np.float32, order="F", copy=True)
    V = np.asfortranarray(V, dtype=np.float32)
    Z = np.asfortranarray(Z, dtype=np.float32)
    M, N = C.shape
    b = V.shape[1]
    _check(lib().skl_gemm_update(M, N, b, r0, _ptr(V), M, _ptr(Z), b, _ptr(C), M,
                                 1 if tensor else 0))
    return C


def dht_length(n, wisdom=0):
    return int(lib().skl_dht_length(n, wisdom))


def dht(A, D, N=None, precision="mixed"):
    """Y = DHT_N(D*A/sqrt(N)) column-wise (zero padded to N rows) on the GPU."""
    A = np.asfortranarray(A, dtype=np.float64)
    if A.ndim == 1:
        A = A[:, None]
    n, d = A.shape
    N = dht_length(n) if N is None else N
    Y = np.zeros((N, d), dtype=np.float64, order="F")
    D = np.ascontiguousarray(D, dtype=np.float64)
    _check(lib().skl_dht(_ptr(A), max(n, 1), n, d, _ptr(D), N, PREC[precision], _ptr(Y)))
    return Y


def dht_device_noalloc(A_ptr, lda, n, d, D_ptr, N, Y_ptr, ldy, precision="mixed", stream=0):
    """skl_dht on device pointers with static scratch (no device allocation);
    enqueued on `stream` (a raw cudaStream_t handle, 0 = default stream)."""
    _check(lib().skl_dht_device_noalloc(ctypes.c_void_p(A_ptr), lda, n, d, ctypes.c_void_p(D_ptr),
                                        N, PREC[precision], ctypes.c_void_p(Y_ptr), ldy,
                                        ctypes.c_void_p(stream)))


def sketch_dense(A, b, D, N, m, k, rows, vals, precision="mixed"):
    A = np.asfortranarray(A, dtype=np.float64)
    n, d = A.shape
    SA = np.zeros((m, d), dtype=np.float64, order="F")
    Sb = np.zeros(m, dtype=np.float64)
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    _check(lib().skl_sketch_dense(_ptr(A), max(n, 1), n, d, _ptr(np.ascontiguousarray(b, dtype=np.float64)),
                                  _ptr(np.ascontiguousarray(D, dtype=np.float64)), N, m, k,
                                  _ptr(rows), _ptr(vals), PREC[precision], _ptr(SA), _ptr(Sb)))
    return SA, Sb


def finalize():
    lib().skl_finalize()

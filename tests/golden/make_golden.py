"""Generate the committed golden fixtures from the reference's own test data.

Run where the reference source tree is available, with SKILLS_REF_DIR set to
its root.  Produces:

  fixtures.npz   the 12 full-rank matrices of data/*.mtx and the 12
                 rank-deficient matrices of data/rank_deficient_sparse_paper/
                 (CSC, fat inputs transposed as test/ls_qr.cpp:56-63 does),
                 plus the expected residual norms of test/test_solvers.sh:138-141
                 and the known answers of the two example programs.
  rand_glibc.npz first outputs of the host C library's rand() for several
                 seeds (the RNG behind src/sparse_helpers.cpp:74-115).
  hashing.npz    gen_hashing_matrix outputs (rows, signs) for a few (m, n, k)
                 from a fresh-process stream (seed 1), produced by the
                 reference's own src/sparse_helpers.cpp when oracle/_ref is
                 built, else by the oracle (recorded in 'source').
"""
import ctypes
import os
import sys

import numpy as np
import scipy.io
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("SKILLS_REF_DIR")

FULL_RANK = ["50by15", "50by20", "100by15", "100by20", "120by15", "120by20"]
# test/test_solvers.sh:138-141 (matrix order and expected residual of b = ones)
RANK_DEF = [("lp_ship12l", 18.3360), ("Franz1", 26.5028), ("GL7d26", 50.8747),
            ("cis-n4c6-b2", 6.12592e-14), ("lp_modszk1", 33.2357), ("rel5", 14.0199),
            ("ch5-5-b1", 7.31938), ("n3c5-b2", 8.99553e-15), ("ch4-4-b1", 4.23281),
            ("n3c5-b1", 3.46410), ("n3c4-b1", 1.82574), ("cis-n4c6-b3", 30.9959)]


def _to_csc_tall(M):
    M = sp.csc_matrix(M)
    if M.shape[0] < M.shape[1]:
        M = sp.csc_matrix(M.T)
    M.sort_indices()
    return M


def fixtures():
    out = {}
    names = []
    for tag in FULL_RANK:
        for kind in ("Dense", "Sparse"):
            name = f"{tag}{kind}FullRank"
            M = scipy.io.mmread(os.path.join(REF, "data", name + ".mtx"))
            if kind == "Dense":
                out[name + "/dense"] = np.asfortranarray(np.asarray(M, dtype=np.float64))
            else:
                C = _to_csc_tall(M)
                out[name + "/indptr"] = C.indptr.astype(np.int64)
                out[name + "/indices"] = C.indices.astype(np.int64)
                out[name + "/data"] = C.data.astype(np.float64)
                out[name + "/shape"] = np.array(C.shape, dtype=np.int64)
            names.append(name)
    for name, res in RANK_DEF:
        M = scipy.io.mmread(os.path.join(REF, "data", "rank_deficient_sparse_paper", name + ".mtx"))
        C = _to_csc_tall(M)
        out[name + "/indptr"] = C.indptr.astype(np.int64)
        out[name + "/indices"] = C.indices.astype(np.int64)
        out[name + "/data"] = C.data.astype(np.float64)
        out[name + "/shape"] = np.array(C.shape, dtype=np.int64)
        out[name + "/expected_residual"] = np.array(res)
        names.append(name)
    out["names"] = np.array(names)
    # test/ski-llsDenseExample.cpp:9-12 and :48 ; test/ski-llsSparseExample.cpp:56-62, :72, :107
    out["dense_example/A"] = np.asfortranarray(np.array(
        [0.306051, -1.53078, 1.64493, -1.61322, -0.2829, 0.474476, -0.586278, -0.610202]
    ).reshape(2, 4).T)
    out["dense_example/b"] = np.array([0.0649338, 0.845946, -0.0164085, 0.247119])
    out["dense_example/x_expected"] = np.array([-0.2122, 0.0720])
    out["sparse_example/indptr"] = np.array([0, 1, 3, 5], dtype=np.int64)
    out["sparse_example/indices"] = np.array([0, 0, 2, 1, 3], dtype=np.int64)
    out["sparse_example/data"] = np.array([2.0, 3.0, 1.0, 4.0, 5.0])
    out["sparse_example/b"] = np.array([0.0649338, 0.845946, -0.0164085, 0.247119])
    out["sparse_example/x_expected"] = np.array([0.0571, -0.0164, 0.1127])
    np.savez_compressed(os.path.join(HERE, "fixtures.npz"), **out)


def rand_glibc():
    libc = ctypes.CDLL("libc.so.6")
    out = {}
    seeds = [1, 12, 42, 2**31 + 7, 4294967295]
    for s in seeds:
        libc.srand(ctypes.c_uint(s))
        out[f"seed_{s}"] = np.array([libc.rand() for _ in range(1000)], dtype=np.int32)
    out["seeds"] = np.array(seeds, dtype=np.uint64)
    np.savez_compressed(os.path.join(HERE, "rand_glibc.npz"), **out)


CASES = [(17, 40, 1), (17, 40, 3), (1700, 20000, 2), (8500, 5000, 2), (5, 100, 5)]


def hashing():
    sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
    import ski_lls_oracle as orc
    ref = None
    ref_path = os.path.join(HERE, "..", "..", "oracle", "_ref", "libskills_ref.so")
    if os.path.exists(ref_path):
        ref = ctypes.CDLL(ref_path)
    out = {"source": np.array("reference" if ref else "oracle")}
    for (m, n, k) in CASES:
        if ref is not None:
            rows = np.empty(n * k, dtype=np.int64)
            cols = np.empty(n + 1, dtype=np.int64)
            vals = np.empty(n * k, dtype=np.float64)
            ref.skref_reset_rand()
            ref.gen_hashing_matrix_c(ctypes.c_long(m), ctypes.c_long(n), ctypes.c_long(k),
                                     rows.ctypes.data_as(ctypes.c_void_p),
                                     cols.ctypes.data_as(ctypes.c_void_p),
                                     vals.ctypes.data_as(ctypes.c_void_p))
        else:
            rows, vals = orc.gen_hashing(orc.Rng(1), m, n, k)
        out[f"{m}_{n}_{k}/rows"] = rows.astype(np.int32)
        out[f"{m}_{n}_{k}/signs"] = (vals > 0).astype(np.uint8)
    np.savez_compressed(os.path.join(HERE, "hashing.npz"), **out)


if __name__ == "__main__":
    if not REF:
        raise SystemExit("set SKILLS_REF_DIR to the reference source tree")
    fixtures()
    rand_glibc()
    hashing()
    print("golden fixtures written to", HERE)

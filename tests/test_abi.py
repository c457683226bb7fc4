"""C-ABI library: builds, loads, exports every declared symbol; host-side pieces (no GPU)."""
import math
import os
import re

import numpy as np
import pytest

import skills_gb300 as skl
import ski_lls_oracle as orc
from conftest import ROOT, GOLDEN


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"\b(skl_[a-z_0-9]+)\s*\(", txt))
    return sorted(names)


@pytest.fixture(scope="module")
def L():
    if not os.path.exists(skl.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    return skl.lib()


def test_library_exports_declared_symbols(L):
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, f"declared in include/ but not exported: {missing}"


def test_version(L):
    assert b"sm_103a" in L.skl_version()


def test_default_opts_match_reference_macros():
    o = skl.default_opts()
    # include/bench_config.hpp:7-20
    assert (o.it_tol, o.max_it, o.gamma, o.k) == (1e-6, 10000, 1.1, 3)
    assert (o.perturb, o.rcond_threshold, o.abs_tol) == (1e-10, 1e-10, 1e-8)


def test_hash_stream_bit_exact_vs_oracle_and_golden():
    z = np.load(os.path.join(GOLDEN, "hashing.npz"))
    from make_golden import CASES
    for (m, n, k) in CASES:
        rows, vals = skl.hash_generate(m, n, k, seed=1)
        np.testing.assert_array_equal(rows, z[f"{m}_{n}_{k}/rows"])
        np.testing.assert_array_equal((vals > 0).astype(np.uint8), z[f"{m}_{n}_{k}/signs"])
        r2, v2 = orc.gen_hashing(orc.Rng(1), m, n, k)
        np.testing.assert_array_equal(rows, r2)
        np.testing.assert_array_equal(vals, v2)


def test_hash_stream_continues_like_global_rand():
    # two draws without reseeding continue one stream, as the reference's
    # global rand() does across calls (src/sparse_helpers.cpp:90-116)
    skl.srand(99)
    a_rows, _ = skl.hash_generate(50, 30, 2)
    b_rows, _ = skl.hash_generate(50, 30, 2)
    g = orc.Rng(99)
    r1, _ = orc.gen_hashing(g, 50, 30, 2)
    r2, _ = orc.gen_hashing(g, 50, 30, 2)
    np.testing.assert_array_equal(a_rows, r1)
    np.testing.assert_array_equal(b_rows, r2)


def test_hash_stream_large_draws_split_across_threads():
    # n*k >= 2^15: worker threads draw the swap targets and signs from the
    # generator state jumped to their chunk of the stream; rows, signs and the
    # continuing stream must stay identical to one sequential stream
    skl.srand(7)
    a_rows, a_vals = skl.hash_generate(8500, 30000, 2)
    b_rows, b_vals = skl.hash_generate(900, 40000, 1)
    g = orc.Rng(7)
    r1, v1 = orc.gen_hashing(g, 8500, 30000, 2)
    r2, v2 = orc.gen_hashing(g, 900, 40000, 1)
    np.testing.assert_array_equal(a_rows, r1)
    np.testing.assert_array_equal(a_vals, v1)
    np.testing.assert_array_equal(b_rows, r2)
    np.testing.assert_array_equal(b_vals, v2)


def test_subsample_rows_bit_exact_vs_oracle():
    # random_sample's draw (src/dense_helpers.cpp:19-39): select_k_from_n over
    # 0..N-1 on the reseeded stream; the stream then continues like rand()
    for (N, m, seed) in ((10, 10, 1), (4000, 340, 5), (40000, 6800, 77)):
        rows = skl.subsample_rows(N, m, seed=seed)
        np.testing.assert_array_equal(rows, orc.random_sample_rows(orc.Rng(seed), N, m))
        assert len(np.unique(rows)) == m and rows.min() >= 0 and rows.max() < N
    skl.srand(3)
    a = skl.subsample_rows(500, 40)
    b = skl.subsample_rows(500, 40)
    g = orc.Rng(3)
    np.testing.assert_array_equal(a, orc.random_sample_rows(g, 500, 40))
    np.testing.assert_array_equal(b, orc.random_sample_rows(g, 500, 40))
    with pytest.raises(skl.SklError) as e:
        skl.subsample_rows(10, 11, seed=1)
    assert e.value.status == skl.SKL_ERR_INVALID


def test_hash_stream_chunked_draws_k3():
    # n*k = 300,009: up to 16 worker chunks whose starts fall inside a column
    # (chunk start not a multiple of k), then the stream continues
    skl.srand(11)
    a_rows, a_vals = skl.hash_generate(15000, 100003, 3)
    c_rows, _ = skl.hash_generate(40, 25, 3)
    g = orc.Rng(11)
    r1, v1 = orc.gen_hashing(g, 15000, 100003, 3)
    r3, _ = orc.gen_hashing(g, 40, 25, 3)
    np.testing.assert_array_equal(a_rows, r1)
    np.testing.assert_array_equal(a_vals, v1)
    np.testing.assert_array_equal(c_rows, r3)


def test_hash_rejects_bad_sizes():
    with pytest.raises(skl.SklError):
        skl.hash_generate(3, 10, 5, seed=1)


def test_solve_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    import scipy.sparse as sp
    A = sp.random(40, 5, density=0.5, random_state=1, format="csc")
    with pytest.raises(skl.SklError) as e:
        skl.ls_sparse_spqr(A, np.ones(40), seed=1)
    assert e.value.status in (skl.SKL_ERR_NO_DEVICE, skl.SKL_ERR_CUDA)


def test_argument_errors_come_before_any_device_work(L):
    """The argument checks run before a device is touched, so they answer on a
    machine without a GPU, with the reference's message for m < n
    (src/ls_sparse_spqr.cpp:98-101, src/ls_dense_hashing_blendenpik.cpp:41-44);
    d = 0 is an empty solve.  The library stays usable after each error."""
    import ctypes
    vp = ctypes.c_void_p

    def sparse(m, n, p, b, x, **opt):
        o = skl.default_opts()
        for k, v in opt.items():
            setattr(o, k, v)
        A = skl.SklCsc(m, n, int(p[-1]) if p is not None else 0,
                       p.ctypes.data if p is not None else None, None, None)
        info = skl.SklInfo()
        return L.skl_sparse_solve(ctypes.byref(A), vp(b), vp(x), ctypes.byref(o), ctypes.byref(info))

    def dense(n, d, lda, **opt):
        o = skl.default_opts()
        for k, v in opt.items():
            setattr(o, k, v)
        a, b, x = np.zeros(max(lda * d, 1)), np.ones(max(n, 1)), np.zeros(max(d, 1))
        info = skl.SklInfo()
        return L.skl_dense_solve(vp(a.ctypes.data), lda, n, d, vp(b.ctypes.data), vp(x.ctypes.data),
                                 ctypes.byref(o), ctypes.byref(info))

    b, x = np.ones(8), np.zeros(8)
    p5 = np.zeros(6, np.int64)
    assert sparse(4, 5, p5, b.ctypes.data, x.ctypes.data) == skl.SKL_ERR_NOT_OVERDETERMINED
    assert skl.last_error() == "Matrix is not overdetermined."
    assert L.skl_sparse_solve(None, vp(b.ctypes.data), vp(x.ctypes.data), None, None) == skl.SKL_ERR_INVALID
    assert "A is null" in skl.last_error()
    p3 = np.zeros(4, np.int64)
    assert sparse(8, 3, p3, b.ctypes.data, x.ctypes.data, gamma=0.0) == skl.SKL_ERR_INVALID
    assert "gamma" in skl.last_error()
    assert sparse(8, 3, p3, b.ctypes.data, x.ctypes.data, k=0) == skl.SKL_ERR_INVALID
    assert sparse(8, 3, p3, b.ctypes.data, x.ctypes.data, precision=7) == skl.SKL_ERR_INVALID
    assert sparse(8, 3, p3, None, x.ctypes.data) == skl.SKL_ERR_INVALID
    assert "null" in skl.last_error()
    assert sparse(8, 0, np.zeros(1, np.int64), b.ctypes.data, x.ctypes.data) == skl.SKL_OK
    assert skl.last_error() == ""

    assert dense(4, 5, 4) == skl.SKL_ERR_NOT_OVERDETERMINED
    assert skl.last_error() == "Matrix is not overdetermined."
    assert dense(8, 3, 5) == skl.SKL_ERR_INVALID
    assert "lda" in skl.last_error()
    assert dense(8, 0, 8) == skl.SKL_OK
    # Blendenpik (src/ls_dense_blendenpik.cpp:38-40): the same checks, before the device
    def blendenpik(n, d, lda):
        o = skl.default_opts()
        a, bb, xx = np.zeros(max(lda * d, 1)), np.ones(max(n, 1)), np.zeros(max(d, 1))
        info = skl.SklInfo()
        return L.skl_dense_blendenpik_solve(vp(a.ctypes.data), lda, n, d, vp(bb.ctypes.data),
                                            vp(xx.ctypes.data), ctypes.byref(o), ctypes.byref(info))
    assert blendenpik(4, 5, 4) == skl.SKL_ERR_NOT_OVERDETERMINED
    assert skl.last_error() == "Matrix is not overdetermined."
    assert blendenpik(8, 3, 5) == skl.SKL_ERR_INVALID
    assert blendenpik(8, 0, 8) == skl.SKL_OK


def test_python_structs_match_the_c_header(tmp_path):
    # the ctypes mirrors of skl_csc / skl_opts / skl_info must have the C
    # layout: size and the offset of every field, from a program compiled
    # against include/skills_gb300.h
    import ctypes
    import subprocess
    structs = {"skl_csc": skl.SklCsc, "skl_opts": skl.SklOpts, "skl_info": skl.SklInfo}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "skills_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0; }"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    cuda_inc = "/usr/local/cuda/include"
    r = subprocess.run(["gcc", "-std=c11", "-I", inc, "-I", cuda_inc, str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            parts = line.split()
            got[(parts[0], parts[1])] = int(parts[2])
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_batched_draws_every_stream_in_problem_order():
    """skl_batched_sparse_solve draws each problem's hashing from the library
    stream in problem order (a producer thread, while the workers solve), so
    afterwards the stream stands exactly where a loop of single solves leaves
    it -- also when every solve fails (here: no GPU), since the draws do not
    depend on the solves.  Mixed sizes cover the serial and threaded draws."""
    import scipy.sparse as sp
    shapes = [(3000, 60), (20000, 400), (2500, 50), (40000, 300), (5000, 100)]
    probs = []
    for i, (n, d) in enumerate(shapes):
        A = sp.random(n, d, density=0.01, random_state=i, format="csc")
        probs.append((A, np.ones(n)))
    skl.srand(21)
    try:
        skl.batched_sparse_spqr(probs, 1.7, 2)
    except skl.SklError:
        pass
    rows, _ = skl.hash_generate(100, 10, 2)
    g = orc.Rng(21)
    for (n, d) in shapes:
        orc.gen_hashing(g, int(math.ceil(1.7 * d)), n, 2)
    ref, _ = orc.gen_hashing(g, 100, 10, 2)
    np.testing.assert_array_equal(rows, ref)

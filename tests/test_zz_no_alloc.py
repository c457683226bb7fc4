"""skl_dht_device_noalloc: the column DHT on caller-owned device buffers with
its scratch in a static device array (no device allocation).  Checked bit for
bit against skl_dht, the allocating host-buffer entry point, on two calls in a
row with different data, in both precisions and on both DHT code paths (FP32
in shared memory, ping-pong through the scratch); the size limit is checked
without a GPU.  The file name makes it run after every other test, so the
entry point is also exercised after the rest of the library has run."""
import ctypes

import numpy as np
import pytest

import skills_gb300 as skl

MAX_N = 4194304   # SKL_DHT_NOALLOC_MAX_N


def test_rejects_transform_beyond_scratch_limit():
    # rejected by the size check before any CUDA call (the pointers are never used)
    fake = ctypes.c_void_p(256)
    rc = skl.lib().skl_dht_device_noalloc(fake, MAX_N + 2, MAX_N + 2, 1, fake, MAX_N + 2,
                                          skl.PREC["fp64"], fake, MAX_N + 2, None)
    assert rc == skl.SKL_ERR_INVALID
    msg = skl.last_error()
    assert "static scratch limit" in msg and str(MAX_N) in msg


def _inputs(seed, n, d, lda):
    rng = np.random.default_rng(seed)
    A = np.zeros((lda, d), order="F")
    A[:n] = rng.standard_normal((n, d))
    D = np.where(rng.random(n) < 0.5, -1.0, 1.0)
    return A, D


@pytest.mark.gpu
@pytest.mark.parametrize("prec,n,N,d", [
    ("fp64", 2999, 3000, 5),        # global ping-pong scratch, every column at once
    ("mixed", 4000, 4000, 9),       # FP32 in shared memory (scratch unused)
    ("mixed", 60000, 60000, 3),     # FP32 L = 30000: past the shared-memory limit
    ("fp64", 599999, 600000, 8),    # 9.6 MB per column: 6 columns at a time, scratch reused
])
def test_matches_allocating_entry_point_two_calls(prec, n, N, d):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    lda, ldy = n + 3, N + 5
    side = torch.cuda.Stream()
    free_after = []
    for call, seed in enumerate((11, 12)):
        A, D = _inputs(seed * 1000 + N, n, d, lda)
        ref = skl.dht(A[:n], D, N, precision=prec)
        Ad = torch.from_numpy(A.ravel(order="F")).to(dev)
        Dd = torch.from_numpy(D).to(dev)
        Yd = torch.full((d * ldy,), np.nan, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(dev)[0]
        stream = side if call == 1 else torch.cuda.current_stream()
        skl.dht_device_noalloc(Ad.data_ptr(), lda, n, d, Dd.data_ptr(), N, Yd.data_ptr(), ldy,
                               precision=prec, stream=stream.cuda_stream)
        stream.synchronize()
        free_after.append((free_before, torch.cuda.mem_get_info(dev)[0]))
        Y = Yd.cpu().numpy().reshape(d, ldy).T
        assert np.array_equal(Y[:N], ref), (prec, call)
        assert np.isnan(Y[N:]).all()          # rows N..ldy-1 untouched
    # the second call (set-up done by the first) takes no device memory
    assert free_after[1][0] == free_after[1][1]

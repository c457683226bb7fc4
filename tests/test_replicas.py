"""Multi-rank host logic of bench.py on CPU: world size 2 over gloo.

The solve path does not shard (one problem per GPU, no data-path exchange), so
a torchrun launch runs replicas; the only collectives are the barrier around
the timed region and the max / sum of a scalar over ranks, which these tests
exercise without a GPU.  The reference arm runs on rank 0 only."""
import contextlib
import io
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    try:
        import bench
        r = bench.Replicas(world, "gloo")
        r.barrier()
        out = {
            "max": r.max(0.25 * (rank + 1)),            # step times differ by rank
            "sum": r.sum(100 + rank),                    # problems per rank
            "flag": r.sum(1 if rank == 1 else 0) == 0,   # a mismatch on one rank is seen by all
        }
        r.barrier()
        r.close()
        q.put((rank, out))
    except Exception as e:   # reported to the parent, which fails the test
        q.put((rank, repr(e)))


def test_two_ranks_reduce_max_and_sum_over_gloo():
    pytest.importorskip("torch.distributed")
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in range(world):
        assert isinstance(res[rank], dict), res[rank]
        assert res[rank]["max"] == 0.5
        assert res[rank]["sum"] == 201.0
        assert res[rank]["flag"] is False


def test_single_process_needs_no_process_group():
    import bench
    r = bench.Replicas(1)
    r.barrier()
    assert r.max(0.125) == 0.125 and r.sum(7) == 7.0
    r.close()


def test_reference_arm_runs_on_rank_zero_only():
    import bench
    args = bench.argparse.Namespace(workload="no-such-workload", warmup=1, steps=1, gpus=2)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(args, rank=1)   # returns before building the workload
    assert buf.getvalue() == ""

"""Runs ONE solve of a named synthetic workload through the C ABI (device
pointers, no warm-up) and prints its diagnostics -- a small driver for
profilers (ncu) and for per-phase timing.

    python ski-lls_gb300/profile_solve.py [workload] [mixed|fp64] [repeats]
"""
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import numpy as np  # noqa: E402
import torch  # noqa: E402

import skills_gb300 as skl  # noqa: E402
import synthetic  # noqa: E402


def main():
    name = sys.argv[1] if len(sys.argv) > 1 else "sparse_illcond_120000x5000"
    prec = sys.argv[2] if len(sys.argv) > 2 else "mixed"
    reps = int(sys.argv[3]) if len(sys.argv) > 3 else 1
    w = synthetic.WORKLOADS[name]
    A, b = w["gen"]()
    dev = torch.device("cuda", 0)
    if w["kind"] == "dense":
        n, d = A.shape
        Ad = torch.from_numpy(np.asfortranarray(A).ravel(order="F")).to(dev)
        bd = torch.from_numpy(b).to(dev)
        xd = torch.zeros(d, dtype=torch.float64, device=dev)
        for _ in range(reps):
            info = skl.dense_solve_device(n, d, Ad.data_ptr(), n, bd.data_ptr(), xd.data_ptr(),
                                          w["gamma"], w["k"], precision=prec, seed=1,
                                          it_tol=1e-10, profile=1)
        print(json.dumps(info.as_dict()))
        return
    A = A.tocsc()
    n, d = A.shape
    Ap = torch.from_numpy(A.indptr.astype(np.int64)).to(dev)
    Ai = torch.from_numpy(A.indices.astype(np.int64)).to(dev)
    Ax = torch.from_numpy(A.data).to(dev)
    bd = torch.from_numpy(b).to(dev)
    xd = torch.zeros(d, dtype=torch.float64, device=dev)
    for _ in range(reps):
        info = skl.sparse_solve_device(n, d, Ap.data_ptr(), Ai.data_ptr(), Ax.data_ptr(),
                                       bd.data_ptr(), xd.data_ptr(), int(A.nnz), w["gamma"],
                                       w["k"], precision=prec, seed=1, it_tol=1e-10, profile=1)
    print(json.dumps(info.as_dict()))


if __name__ == "__main__":
    main()

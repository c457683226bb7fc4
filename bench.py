#!/usr/bin/env python3
"""Time-to-solve benchmark of the GB300 Ski-LLS solve path.

One step = one full solve (sketch -> randomized CPQR -> preconditioned LSQR)
of the named workload, inputs resident in HBM.  Default workload: the
120,000 x 5,000, 1 %-dense, column-scaled (kappa ~ 1e8), rank-deficient
sparse problem, s = 2, m = 1.7 d, LSQR tolerance 1e-10, mixed precision.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME] [--no-cpu-baseline] [--no-fp64] [--no-e2e]
    python bench.py --workload NAME --profile-one [--precision mixed|fp64] [--repeats R]

Workloads: sparse_uniform_20000x1000, dense_kappa1e6_40000x4000,
sparse_illcond_120000x5000 (default), sparse_zipf_1000000x10000,
batched_sparse, and dense_blendenpik_40000x4000 (the Blendenpik comparison
solver on the dense matrix).  Prints ONE JSON line on rank 0.  Multi-GPU (torchrun): every
rank solves its own replica (the single-problem path does not shard); the
reported time is the max over ranks.  The reference arm (--impl reference)
times the CPU oracle, a restatement of the reference algorithm, on the host
cores.  --profile-one runs one solve with the library's per-kernel events on
(the command the ncu summaries under profiles/ were taken with).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for sub in ("ski-lls_gb300", "oracle"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "time-to-solve @ backward err <=1e-10: mixed vs FP64 path on 1 GB300 (s, %HBM)"
DEFAULT_WORKLOAD = "sparse_illcond_120000x5000"
IT_TOL = 1e-10
BATCH_BACKWARD_TOL = 1e-10   # batched problems: restarts until the metric's bound holds


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # 20 solves (~1.2 s timed) give the 200 ms clock sampler several readings
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--batch-count", type=int, default=512,
                    help="problems in the batched_sparse workload")
    ap.add_argument("--autotune", action="store_true",
                    help="sparse workloads: autotuned launch shapes (tuned during the warm-up)")
    ap.add_argument("--profile-one", action="store_true",
                    help="one solve with per-kernel events, for profilers")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--repeats", type=int, default=1)
    ap.add_argument("--oracle-once", default=None, help=argparse.SUPPRESS)
    return ap.parse_args()


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), float(pk["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------- replicas --
class Replicas:
    """The ranks of a torchrun launch, one GPU each.  Every rank solves its own
    problems (the path has no exchange step), so the only collectives are a
    barrier around the timed region and the max (or sum) of a scalar over
    ranks.  With one process there is no process group and these are no-ops."""

    def __init__(self, world, backend="nccl", device=None):
        self.world = world
        self.device = device
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            kw = {"device_id": device} if backend == "nccl" and device is not None else {}
            dist.init_process_group(backend, **kw)
            self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def _reduce(self, x, op):
        if self.dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x):
        return self._reduce(x, self.dist.ReduceOp.MAX if self.dist else None)

    def sum(self, x):
        return self._reduce(x, self.dist.ReduceOp.SUM if self.dist else None)

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


# --------------------------------------------------------------- workload --
def make_workload(name):
    import synthetic
    if name not in synthetic.WORKLOADS:
        raise SystemExit(f"unknown workload {name}; choose from {sorted(synthetic.WORKLOADS)} "
                         "or batched_sparse")
    w = synthetic.WORKLOADS[name]
    t0 = time.perf_counter()
    A, b = w["gen"]()
    if w["kind"] == "sparse":
        A = A.tocsc()
        A.sort_indices()
    else:
        A = np.asfortranarray(A)
    return w, A, b, time.perf_counter() - t0


def oracle_sample_text(kind):
    """What the CPU oracle restates for a workload kind (for the baseline's `sample`)."""
    if kind == "blendenpik":
        return ("restatement of ls_dense_blendenpik: the random signs and row sample from the C "
                "library's stream, numpy's FFT for the DHT, LAPACK dgeqrf through numpy's OpenBLAS "
                "on all cores, LSQR in C loops single-threaded")
    return ("restatement of the reference algorithm: C loops single-threaded as the reference's "
            "MAX_NUM_THREADS = 1, LAPACK dgeqp3/dormqr/dtrcon through numpy's OpenBLAS on all "
            "cores; SPQR replaced by dense CPQR of the sketch")


def oracle_kind(w):
    """Which oracle solver a workload runs: "sparse", "dense" or "blendenpik"."""
    return "blendenpik" if w.get("solver") == "blendenpik" else w["kind"]


def oracle_solve(kind, A, b, gamma, k):
    import ski_lls_oracle as orc
    if kind == "blendenpik":
        return orc.ls_dense_blendenpik(A, b, gamma, it_tol=IT_TOL, seed=1)
    if kind == "sparse":
        return orc.ls_sparse_spqr(A.shape[0], A.shape[1], A.indptr, A.indices, A.data, b, gamma,
                                  k, it_tol=IT_TOL, rng=orc.Rng(1))
    return orc.ls_dense_hashing_blendenpik(A, b, gamma, k, it_tol=IT_TOL, seed=1)


def exact_quality(A, x, b):
    """||b - A x|| and ||A^T r|| / (||A||_F ||r||) with r correctly rounded."""
    import accurate
    r = accurate.residual(A, x, b)
    nr = math.sqrt(math.fsum(r * r))
    import scipy.sparse as sp
    fro = math.sqrt(math.fsum(A.data * A.data)) if sp.issparse(A) else float(np.linalg.norm(A))
    be = float(np.linalg.norm(A.T @ r) / (fro * nr)) if nr > 0 else 0.0
    return {"residual_norm": nr, "backward_error": be}


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


def oracle_once_child(args):
    """--oracle-once: one oracle solve of the workload saved by the parent (run
    with the BLAS thread count the parent set in the environment)."""
    z = np.load(args.oracle_once, allow_pickle=False)
    if z["kind"] == "sparse":
        import scipy.sparse as sp
        A = sp.csc_matrix((z["data"], z["indices"], z["indptr"]), shape=tuple(z["shape"]))
    else:
        A = np.asfortranarray(z["A"])
    t0 = time.perf_counter()
    out = oracle_solve(str(z["kind"]), A, z["b"], float(z["gamma"]), int(z["k"]))
    print(json.dumps({"value": time.perf_counter() - t0, "phases_s": out["phases_s"],
                      "it": int(out["it"]), "rank": int(out["rank"])}), flush=True)


def cpu_baseline_run(kind, name, A, b, gamma, k):
    """The CPU oracle on the host cores: one solve with BLAS on all cores (the
    reported value), then one with BLAS on one thread (in a child process,
    skipped when the all-cores solve took over 30 s).  Per-phase times."""
    t0 = time.perf_counter()
    out = oracle_solve(kind, A, b, gamma, k)
    t_all = time.perf_counter() - t0
    one = None
    if t_all < 30.0:
        import tempfile
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "w.npz")
            if kind == "sparse":
                np.savez(path, kind=kind, gamma=gamma, k=k, b=b, indptr=A.indptr,
                         indices=A.indices, data=A.data, shape=np.array(A.shape))
            else:
                np.savez(path, kind=kind, gamma=gamma, k=k, b=b, A=A)
            env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")
            try:
                p = subprocess.run([sys.executable, os.path.abspath(__file__), "--oracle-once",
                                    path, "--workload", name], env=env, capture_output=True,
                                   text=True, timeout=300)
                one = json.loads(p.stdout.strip().splitlines()[-1]) if p.returncode == 0 else \
                    {"error": p.stderr[-300:]}
            except (subprocess.SubprocessError, ValueError, IndexError) as e:
                one = {"error": str(e)[:300]}
    cpu = {"value": t_all, "unit": "s", "cores": os.cpu_count(), "kind": "port",
           "cpu_model": cpu_model(),
           "sample": "one full solve of the workload by the CPU oracle (%s)" % oracle_sample_text(kind),
           "phases_s": out["phases_s"], "it": int(out["it"]), "rank": int(out["rank"]),
           "blas_one_thread": one}
    return cpu, out


# ---------------------------------------------------------- reference arm --
def run_reference(args, rank):
    if rank != 0:
        return
    w, A, b, _ = make_workload(args.workload)
    warm = min(args.warmup, 1)
    steps = max(1, min(args.steps, 5))
    for _ in range(warm):
        oracle_solve(oracle_kind(w), A, b, w["gamma"], w["k"])
    times = []
    out = None
    for _ in range(steps):
        t0 = time.perf_counter()
        out = oracle_solve(oracle_kind(w), A, b, w["gamma"], w["k"])
        times.append(time.perf_counter() - t0)
    v = statistics.median(times)
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "requested_steps": args.steps,
        "requested_warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "shape": list(A.shape),
                   "nnz": int(getattr(A, "nnz", A.size)), "gamma": w["gamma"], "k": w["k"],
                   "it_tol": IT_TOL},
        "cpu_baseline": {"value": v, "unit": "s", "cores": cores, "kind": "port",
                         "cpu_model": cpu_model(),
                         "sample": "full solve of the workload per step, median of the timed "
                                   "steps; CPU oracle (%s)" % oracle_sample_text(oracle_kind(w))},
        "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "solve": {"rank": int(out["rank"]), "it": int(out["it"]), "flag": int(out["flag"]),
                  "phases_s": out["phases_s"], "step_s": times,
                  **exact_quality(A, out["x"], b)},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------ problem on device --
class SparseOnDevice:
    kind = "sparse"

    def __init__(self, A, b, dev, torch):
        self.A, self.b = A, b
        self.n, self.d = A.shape
        self.nnz = int(A.nnz)
        self.Ap = torch.from_numpy(A.indptr.astype(np.int64)).to(dev)
        self.Ai = torch.from_numpy(A.indices.astype(np.int64)).to(dev)
        self.Ax = torch.from_numpy(A.data.astype(np.float64)).to(dev)
        self.bd = torch.from_numpy(b.astype(np.float64)).to(dev)
        self.xd = torch.zeros(self.d, dtype=torch.float64, device=dev)

    autotune = 0

    def solve(self, skl, precision, profile, stream, device, gamma, k):
        return skl.sparse_solve_device(self.n, self.d, self.Ap.data_ptr(), self.Ai.data_ptr(),
                                       self.Ax.data_ptr(), self.bd.data_ptr(), self.xd.data_ptr(),
                                       self.nnz, gamma, k, precision=precision, seed=1,
                                       it_tol=IT_TOL, stream=stream, profile=profile,
                                       device=device, autotune=self.autotune)

    def host_solver(self, skl, torch, opts):
        """Returns (call, x_host, h2d, d2h): call() runs skl_sparse_solve on
        pinned host buffers."""
        import ctypes
        A = self.A
        hp = torch.from_numpy(A.indptr.astype(np.int64)).pin_memory()
        hi = torch.from_numpy(A.indices.astype(np.int64)).pin_memory()
        hx = torch.from_numpy(A.data.astype(np.float64)).pin_memory()
        hb = torch.from_numpy(self.b.astype(np.float64)).pin_memory()
        hxo = torch.zeros(self.d, dtype=torch.float64).pin_memory()
        csc = skl.SklCsc(self.n, self.d, self.nnz, hp.data_ptr(), hi.data_ptr(), hx.data_ptr())
        keep = (hp, hi, hx, hb, hxo, csc)

        def call():
            info = skl.SklInfo()
            rc = skl.lib().skl_sparse_solve(ctypes.byref(keep[5]), ctypes.c_void_p(hb.data_ptr()),
                                            ctypes.c_void_p(hxo.data_ptr()), ctypes.byref(opts),
                                            ctypes.byref(info))
            if rc != 0:
                raise RuntimeError(skl.last_error())
            return info
        return call, hxo, 8 * (self.d + 1) + 16 * self.nnz + 8 * self.n, 8 * self.d

    def product_bytes(self, r):
        n, d, nnz = self.n, self.d, self.nnz
        return {
            # CSR: column index 4 B + (hi, lo) value 8 B per nnz, row pointers,
            # z gather (d pairs), u read + write
            "lsqr_spmv_csr_Az": 12 * nnz + 4 * (n + 1) + 8 * d + 16 * n,
            # CSC over all columns: row index + value, u reads counted once, t write
            "lsqr_spmv_csc_ATu": 12 * nnz + 4 * (d + 1) + 8 * n + 8 * r,
            "lsqr_trmv_Mv": 4 * r * (r + 1) // 2 + 8 * r + 16 * r,
            "lsqr_trmv_MTt": 4 * r * (r + 1) // 2 + 8 * r + 16 * r,
        }

    def config(self):
        return {"n": self.n, "d": self.d, "nnz": self.nnz,
                "l2": "inputs larger than L2 (CSC + CSR copies and the m x d sketch exceed "
                      "129 MB at the benchmark sizes) and a 256 MB buffer written between steps"}


class DenseOnDevice:
    kind = "dense"

    def __init__(self, A, b, dev, torch, blendenpik=False):
        self.A, self.b = A, b
        self.n, self.d = A.shape
        self.blendenpik = blendenpik   # ls_dense_blendenpik instead of the hashing solver
        self.Ad = torch.from_numpy(np.asfortranarray(A).ravel(order="F")).to(dev)
        self.bd = torch.from_numpy(b.astype(np.float64)).to(dev)
        self.xd = torch.zeros(self.d, dtype=torch.float64, device=dev)

    def solve(self, skl, precision, profile, stream, device, gamma, k):
        if self.blendenpik:
            return skl.dense_blendenpik_device(self.n, self.d, self.Ad.data_ptr(), self.n,
                                               self.bd.data_ptr(), self.xd.data_ptr(), gamma,
                                               precision=precision, seed=1, it_tol=IT_TOL,
                                               stream=stream, profile=profile, device=device)
        return skl.dense_solve_device(self.n, self.d, self.Ad.data_ptr(), self.n,
                                      self.bd.data_ptr(), self.xd.data_ptr(), gamma, k,
                                      precision=precision, seed=1, it_tol=IT_TOL, stream=stream,
                                      profile=profile, device=device)

    def host_solver(self, skl, torch, opts):
        import ctypes
        hA = torch.from_numpy(np.asfortranarray(self.A).ravel(order="F")).pin_memory()
        hb = torch.from_numpy(self.b.astype(np.float64)).pin_memory()
        hxo = torch.zeros(self.d, dtype=torch.float64).pin_memory()
        n, d = self.n, self.d
        entry = skl.lib().skl_dense_blendenpik_solve if self.blendenpik else skl.lib().skl_dense_solve

        def call():
            info = skl.SklInfo()
            rc = entry(ctypes.c_void_p(hA.data_ptr()), n, n, d,
                                           ctypes.c_void_p(hb.data_ptr()),
                                           ctypes.c_void_p(hxo.data_ptr()), ctypes.byref(opts),
                                           ctypes.byref(info))
            if rc != 0:
                raise RuntimeError(skl.last_error())
            return info
        call.keep = (hA, hb)
        return call, hxo, 8 * n * d + 8 * n, 8 * d

    def product_bytes(self, r):
        n, d = self.n, self.d
        return {
            # the r selected columns of the (hi, lo) copy of A, z, u read + write
            "lsqr_gemv_dense_Az": 8 * n * r + 8 * r + 16 * n,
            "lsqr_gemv_dense_ATu": 8 * n * r + 8 * n + 8 * r,
            "lsqr_trmv_Mv": 4 * r * (r + 1) // 2 + 8 * r + 16 * r,
            "lsqr_trmv_MTt": 4 * r * (r + 1) // 2 + 8 * r + 16 * r,
        }

    def config(self):
        return {"n": self.n, "d": self.d,
                "l2": "inputs larger than L2 (A 1.28 GB FP64 plus its float-pair copy) and a "
                      "256 MB buffer written between steps"}


def on_device(w, A, b, dev, torch):
    if w["kind"] == "sparse":
        return SparseOnDevice(A, b, dev, torch)
    return DenseOnDevice(A, b, dev, torch, blendenpik=w.get("solver") == "blendenpik")


def profile_one(args):
    """--profile-one: ONE solve of the workload on device-resident inputs with
    the library's per-kernel events on, no warm-up: a short, fixed command for
    ncu captures and per-phase timing."""
    import torch
    import skills_gb300 as skl
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    w, A, b, _ = make_workload(args.workload)
    P = on_device(w, A, b, dev, torch)
    info = None
    for _ in range(max(1, args.repeats)):
        info = P.solve(skl, args.precision, 1, None, 0, w["gamma"], w["k"])
    print(json.dumps(info.as_dict()), flush=True)


# ---------------------------------------------------------------- our arm --
def run_ours(args, rank, world):
    import torch
    import skills_gb300 as skl

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ranks = Replicas(world, "nccl", dev)
    barrier = ranks.barrier

    w, A, b, gen_s = make_workload(args.workload)
    gamma, k = w["gamma"], w["k"]
    hbm_peak, _, peak_kind = load_peaks()
    P = on_device(w, A, b, dev, torch)
    if args.autotune and P.kind == "sparse":
        P.autotune = 1
    n, d = P.n, P.d
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)   # > 129 MB L2
    stream = torch.cuda.Stream(device=dev)

    def timed(precision, steps, warmup, profile):
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                P.solve(skl, precision, profile, stream.cuda_stream, local, gamma, k)
            torch.cuda.synchronize()
            barrier()
            torch.cuda.synchronize()
            evs = []
            infos = []
            t0 = time.perf_counter()
            for _ in range(steps):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                infos.append(P.solve(skl, precision, profile, stream.cuda_stream, local, gamma, k))
                e1.record(stream)
                evs.append((e0, e1))
            torch.cuda.synchronize()
            barrier()
            wall = time.perf_counter() - t0
        ms = [a.elapsed_time(b_) for a, b_ in evs]
        return ms, infos, wall

    clocks = ClockSampler(local)
    clocks.start()
    ms, infos0, wall = timed("mixed", args.steps, max(3, args.warmup), 0)
    clk = clocks.stop()
    # the same steps again with the library's per-kernel CUDA events enabled
    # (event records between launches cost a few ms per solve, so the value
    # above is timed without them); the kernel roofline uses these events
    _, infos, _ = timed("mixed", args.steps, 1, 1)
    x_mixed = P.xd.cpu().numpy()
    step_s = ranks.max(statistics.mean(ms) / 1e3)
    last = infos[-1]

    def phases(i):
        return {"setup": i.t_setup_ms, "sketch": i.t_sketch_ms, "qr": i.t_qr_ms,
                "precond": i.t_precond_ms, "lsqr": i.t_lsqr_ms, "host_hash": i.t_host_hash_ms}

    fp64 = None
    x64 = None
    if not args.no_fp64:
        ms64, inf64, _ = timed("fp64", max(1, min(args.steps, 3)), 1, 0)
        x64 = P.xd.cpu().numpy()
        fp64 = {"value": statistics.mean(ms64) / 1e3, "unit": "s",
                "mixed_speedup": statistics.mean(ms64) / statistics.mean(ms),
                "it": int(inf64[-1].it), "rank": int(inf64[-1].rank),
                "phases_ms": phases(inf64[-1])}

    # ---- per-kernel live event times -> achieved bandwidth
    r = int(last.rank) + int(last.unresolved_cols)
    prof_ms = np.sum([np.array(list(i.prof_ms)) for i in infos], axis=0)
    prof_n = np.sum([np.array(list(i.prof_launches)) for i in infos], axis=0)
    kernels = {}
    for q, (name, nbytes) in enumerate(P.product_bytes(r).items()):
        if prof_n[q] > 0:
            per = prof_ms[q] / prof_n[q]
            ach = nbytes / (per * 1e-3) / 1e9
            kernels[name] = {"launches": int(prof_n[q]), "ms_per_launch": per,
                             "total_ms": float(prof_ms[q]), "alg_bytes": int(nbytes),
                             "achieved_gbs": ach, "frac": ach / hbm_peak}
    # the sample QRP (k_yqrp_reg, one launch per panel but the last): live
    # event time per launch from the QR sub-step events; algorithmic bytes =
    # one read of the (nb+16) x (d-j) FP32 sample block per launch, nb the
    # panel width the solve used
    nb = int(last.tuned[1]) or 64
    nbp = nb + 16
    mrows = int(last.sketch_rows)
    mn = min(mrows, d)
    yq_js = [j for j in range(0, mn, nb) if j + nb < mrows and j + nb < d]
    yq_ms = float(np.sum([i.qr_prof_ms[0] for i in infos]))
    if yq_js and yq_ms > 0:   # no sample QRP on the unpivoted (Blendenpik) path
        yq_n = len(yq_js) * len(infos)
        yq_bytes = int(np.mean([4 * nbp * (d - j) for j in yq_js]))
        per = yq_ms / yq_n
        ach = yq_bytes / (per * 1e-3) / 1e9
        kernels["k_yqrp_reg"] = {"launches": yq_n, "ms_per_launch": per, "total_ms": yq_ms,
                                 "alg_bytes": yq_bytes, "achieved_gbs": ach, "frac": ach / hbm_peak,
                                 "note": "latency-bound: %d dependent pivot steps per launch, each an "
                                         "mbarrier-completed candidate exchange among 16 CTAs" % nb}
    if P.kind == "dense":
        # DHT + hash: read A once (FP64), write the m x d FP32 sketch
        sk_ms = float(np.sum([i.t_sketch_ms for i in infos]))
        sk_bytes = 8 * n * d + 4 * mrows * d
        per = sk_ms / len(infos)
        ach = sk_bytes / (per * 1e-3) / 1e9
        kernels["k_dht_hash"] = {"launches": len(infos), "ms_per_launch": per,
                                 "total_ms": sk_ms, "alg_bytes": sk_bytes, "achieved_gbs": ach,
                                 "frac": ach / hbm_peak}
    dom = max(kernels, key=lambda kk: kernels[kk]["total_ms"]) if kernels else None
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath) and dom:
        with open(tpath) as f:
            traffic = json.load(f).get(args.workload, {}).get(dom)
    roofline = None
    if dom:
        kk = kernels[dom]
        roofline = {"kernel": dom, "bound": "hbm", "achieved": kk["achieved_gbs"],
                    "peak": hbm_peak, "unit": "GB/s", "frac": kk["frac"], "traffic": traffic,
                    "peak_kind": peak_kind, "alg_bytes_per_launch": kk["alg_bytes"]}
        if "note" in kk:
            roofline["note"] = kk["note"]

    # ---- e2e through the host-pointer C ABI (pinned host buffers, copies timed)
    e2e = None
    if not args.no_e2e:
        o = skl.default_opts()
        o.gamma, o.k, o.it_tol, o.seed_mode, o.seed, o.device = gamma, k, IT_TOL, 1, 1, local
        o.stream = stream.cuda_stream
        o.autotune = getattr(P, "autotune", 0)
        call, hxo, h2d, d2h = P.host_solver(skl, torch, o)
        times = []
        for q in range(max(3, args.warmup) + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            call()
            t = time.perf_counter() - t0
            if q >= max(3, args.warmup):
                times.append(t)
        e2e = {"value": ranks.max(statistics.mean(times)), "unit": "s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "x_matches_device_path": bool(np.array_equal(hxo.numpy(), x_mixed))}

    cpu = None
    oracle = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, oracle = cpu_baseline_run(oracle_kind(w), args.workload, A, b, gamma, k)

    if rank != 0:
        return
    quality = {"mixed": exact_quality(A, x_mixed, b)}
    if x64 is not None:
        quality["fp64"] = exact_quality(A, x64, b)
    if oracle is not None:
        quality["oracle"] = exact_quality(A, oracle["x"], b)
        quality["oracle"]["rank"] = int(oracle["rank"])
        quality["x_rel_diff_mixed_vs_oracle"] = float(
            np.linalg.norm(x_mixed - oracle["x"]) / np.linalg.norm(oracle["x"]))
        rn0 = quality["oracle"]["residual_norm"]
        for key in ("mixed", "fp64"):
            if key in quality and rn0 > 0:
                quality[key]["residual_rel_excess_vs_oracle"] = \
                    (quality[key]["residual_norm"] - rn0) / rn0
    line = {
        "metric": METRIC, "value": step_s, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": step_s * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+ff+f64", "data": "synthetic",
        "config": {"workload": args.workload, **P.config(), "gamma": gamma, "k": k,
                   "sketch_rows": mrows, "it_tol": IT_TOL,
                   "precision": "mixed: FP32 sketch, QR and R^-1; LSQR products in float-float "
                                "(FP32 pairs, ~2^-48 relative) over (hi, lo) pairs of A's values "
                                "(48 of 53 bits); FP64 recurrences, norms, solution assembly "
                                "and residual",
                   "parallelism": "replicas"},
        "e2e": e2e,
        "gpu_launches": int(sum(i.kernel_launches for i in infos0)),
        "roofline": roofline,
        "kernels": kernels,
        "cpu_baseline": cpu,
        "clocks": clk,
        "fp64_path": fp64,
        "solve": {"rank": int(last.rank), "unresolved_cols": int(last.unresolved_cols),
                  "it": int(last.it), "flag": int(last.flag), "success": int(last.success),
                  "rcond_r11": last.rcond_r11, "fp64_fallback": int(last.fp64_fallback),
                  "explicit_residual": last.explicit_residual,
                  "sketch_refine_steps": int(last.sketch_refine_steps),
                  "tuned_launch_shapes": dict(zip(("sketch_threads", "panel_width", "lanes_Az",
                                                   "lanes_ATu"), [int(v) for v in last.tuned])),
                  "quality_exact": quality,
                  "phases_ms": phases(last),
                  "qr_substeps_ms": {nm: float(v) for nm, v in zip(
                      ("sample_qrp", "moves", "panel", "qtc", "W", "Z", "update", "downdate",
                       "sample0"), last.qr_prof_ms)},
                  "step_ms": ms, "wall_s": wall, "workload_gen_s": gen_s},
    }
    print(json.dumps(line), flush=True)


def run_batched(args, rank, world):
    """Batched configuration: many independent sparse problems (d in [50, 500],
    n >= 20 d, density 0.5-5 %, column scales 10^U[0,4], b ~ N(0,1); s = 2,
    m = 1.7 d, FP32 sketch/QR, LSQR to 1e-10) through skl_batched_sparse_solve
    (host buffers, H2D/D2H inside the timing), against a loop of single
    skl_sparse_solve calls on the same GPU.  Metric: problems per second."""
    import torch
    import skills_gb300 as skl
    import synthetic

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ranks = Replicas(world, "nccl", torch.device("cuda", local))
    t0 = time.perf_counter()
    probs = synthetic.batched(seed=2024 + rank, count=args.batch_count)   # this rank's shard
    gen_s = time.perf_counter() - t0
    total = int(ranks.sum(len(probs)))
    warm = probs[: min(8, len(probs))]
    # the metric's backward-error condition holds for every problem: LSQR
    # restarts from the FP64 residual until it is met
    bopts = dict(it_tol=IT_TOL, seed=1, backward_tol=BATCH_BACKWARD_TOL, device=local)
    skl.batched_sparse_spqr(warm, 1.7, 2, **bopts)
    batched_s = []
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        ranks.barrier()
        t0 = time.perf_counter()
        xs, infos, status = skl.batched_sparse_spqr(probs, 1.7, 2, **bopts)
        batched_s.append(ranks.max(time.perf_counter() - t0))   # the slowest rank's time
    # a loop of single solves (one pass; it is the slow reference point)
    torch.cuda.synchronize()
    ranks.barrier()
    t0 = time.perf_counter()
    same = True
    for p, (A, b) in enumerate(probs):
        r = skl.ls_sparse_spqr(A, b, 1.7, 2, **bopts)
        same = same and np.array_equal(r.x, xs[p])
    loop_s = ranks.max(time.perf_counter() - t0)
    same = ranks.sum(0 if same else 1) == 0
    be = [exact_quality(A, xs[p], b)["backward_error"] for p, (A, b) in enumerate(probs)]
    if rank != 0:
        return
    best = min(batched_s)
    line = {
        "metric": "batched sparse solves per second", "value": total / best,
        "unit": "problems/s", "n_gpus": world, "steps": len(batched_s), "warmup": 1,
        "ms_per_step": best * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": "batched_sparse", "problems": total,
                   "problems_per_rank": len(probs),
                   "d_range": [50, 500], "n_rule": "n ~ U[2000, 50000], n >= 20 d",
                   "streams": int(os.environ.get("SKILLS_BATCH_STREAMS", "8")), "gamma": 1.7,
                   "k": 2, "it_tol": IT_TOL, "backward_tol": BATCH_BACKWARD_TOL, "inputs": "host buffers (H2D inside the timing)"},
        "e2e": {"value": total / best, "unit": "problems/s",
                "h2d_bytes_per_step": int(sum(16 * A.nnz + 8 * (A.shape[1] + 1) + 8 * A.shape[0]
                                              for A, _ in probs)),
                "d2h_bytes_per_step": int(sum(8 * A.shape[1] for A, _ in probs))},
        "loop_of_single_solves": {"value": total / loop_s, "unit": "problems/s",
                                  "batched_speedup": loop_s / best,
                                  "x_bit_identical": bool(same)},
        "status_ok": int(sum(1 for s_ in status if s_ == 0)),
        "backward_error": {"max": float(max(be)), "median": float(statistics.median(be)),
                           "over": len(be), "evaluation": "correctly rounded residual"},
        "gpu_launches": int(sum(i.kernel_launches for i in infos)),
        "step_s": batched_s, "workload_gen_s": gen_s,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.oracle_once:
        oracle_once_child(args)
        return
    if args.profile_one:
        profile_one(args)
        return
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.workload == "batched_sparse":
        run_batched(args, rank, world)
        return
    run_ours(args, rank, world)


if __name__ == "__main__":
    main()

#!/usr/bin/env python
"""bench.py -- kNN query columns per second on GB300.

Default line (--config dense): the precision path.  A resident 256 x
2,000,000 FP32 embedding matrix (i.i.d. N(0,1) columns mixed with 1,000
Gaussian clusters, sigma 0.3, and 1 % near duplicates at 1e-6; seeded,
generated on the GPU by sparsedist_gb300/synth.py).  One step = one block of
4,096 columns of that matrix searched as query vectors against all 2,000,000
columns, cosine, k = 20: sparseKNN(X[, block], X) with the reference's idx
and FP64 distances (R/sparseKNN.R:183-301 on the dgCMatrix of the same data).

* value: columns / s of the BF16-screened path (the fused tcgen05 screen
  k_dense_tc + exact FP64 re-rank), inputs resident in HBM, CUDA events on
  the library's stream (torch's current stream).
* plain_fp32 / vs_plain_fp32: the same blocks through the plain GPU FP32
  path (FP32 SGEMM, top-k on the FP32 values, no re-rank) and the ratio.
* e2e: the same blocks submitted as host FP32 vectors to the serving loop
  (sdg_server_create_dense / submit / wait / result), host idx / dist back,
  two requests in flight; p50 / p99 request latency beside it.
* roofline: k_dense_tc per launch, 2 * 256 * 2,000,000 * 4,096 BF16 flops
  over its average CUDA-event duration, against the measured BF16 burst.
* cpu_baseline + parity: the oracle (the reference's algorithm, OpenMP over
  all host cores) on the first 128 columns of one block against the whole
  reference; the GPU's result for the same columns is compared with it (idx
  and distances bit for bit for the screened path; agreement and the
  largest distance error for the plain FP32 path).

--config logcount: sparse kNN at scale (30,000 x 200,000 log-count CSC,
cosine k = 20, 4,096-query blocks of sparseKNN(X[, block], X)), with the
same keys and a bit-for-bit parity check of a 256-column oracle sample.
--impl reference times the oracle alone on bounded samples of the chosen
workload.  Multi-GPU (torchrun): each rank searches its own query blocks
against its own replica of the reference (query-column sharding, no
collective on the data path); value = all ranks' columns / max-over-ranks
time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METHOD_CODES = {"binary": 0, "cosine": 1, "euclidean": 2, "manhattan": 3, "pearson": 4, "js": 5}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--method", default="cosine")
    ap.add_argument("--k", type=int, default=20)
    ap.add_argument("--block", type=int, default=4096, help="query columns per step")
    ap.add_argument("--ncol", type=int, default=200000)
    ap.add_argument("--nrow", type=int, default=30000)
    ap.add_argument("--mean-nnz", type=float, default=1800.0)
    ap.add_argument("--engine", type=int, default=0, help="0 auto, 1 exact slab, 2 FP32 screen, 3 tensor-core screen")
    ap.add_argument("--cpu-cols", type=int, default=256, help="query columns of the CPU sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--dist-cols", type=int, default=10000)
    ap.add_argument("--dist-long", action="store_true",
                    help="long columns (the 30,000-row log-count generator)")
    ap.add_argument("--config", default="dense",
                    choices=["dense", "logcount", "uniform", "serve", "dist", "snn", "batched"],
                    help="dense: the default line (256 x 2,000,000 embeddings, BF16-screened vs plain "
                         "FP32, served e2e); logcount: 30,000 x 200,000 log-count sparse kNN; uniform: "
                         "the CPU-runnable 2,000 x 10,000 case; serve: the sparse serving loop; dist: "
                         "full-matrix sparseDist; snn: sparseSNN; batched: 512 uneven sparseKNNCross "
                         "problems through sdg_knn_cross_batch")
    ap.add_argument("--serve-ref-cols", type=int, default=1000000)
    ap.add_argument("--dense-cols", type=int, default=2000000)
    ap.add_argument("--dense-mode", type=int, default=0, choices=[0, 3],
                    help="BF16-screened mode of the dense line: 0 (one CTA per query group), 3 (CTA pairs)")
    ap.add_argument("--dense-block", type=int, default=4096)
    ap.add_argument("--dense-cpu-cols", type=int, default=128,
                    help="query columns of the dense CPU-baseline / parity sample")
    ap.add_argument("--batch-problems", type=int, default=512)
    ap.add_argument("--batch-scale", type=float, default=1.0, help="multiplies the batched problems' column counts")
    ap.add_argument("--batch-check", type=int, default=16, help="smallest problems checked against the oracle")
    ap.add_argument("--batch-group", type=int, default=32,
                    help="problems per sdg_knn_cross_batch call (bounds host memory)")
    ap.add_argument("--ref-cols", type=int, default=16,
                    help="query columns per step of the dense --impl reference arm")
    ap.add_argument("--serve-requests", type=int, default=80)
    ap.add_argument("--serve-util", type=float, default=0.75)
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([s.strip() for s in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        sm = [float(s[1]) for s in self.samples if len(s) >= 9 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) >= 9 and s[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            if len(s) >= 9:
                for n, v in zip(names, s[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


def measured_peaks():
    """(HBM GB/s, BF16 TFLOP/s burst, kind): the machine's measured peaks, or the
    fallback figures.  The burst BF16 figure is the denominator for the
    tensor-core screen's GEMM: one ~22 ms launch per step, timed alone with
    CUDA events."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


def make_workload(args, device):
    from sparsedist_gb300 import synth
    p, i, x = synth.logcount_csc(nrow=args.nrow, ncol=args.ncol, mean_nnz=args.mean_nnz, seed=2,
                                 device=device)
    return p, i, x


def block_arrays(p, i, x, c0, c1):
    a, b = int(p[c0]), int(p[c1])
    return (p[c0:c1 + 1] - a).astype(np.int32), i[a:b], x[a:b]


def bytes_alg(p, c0, c1, nnz_ref, ncol_ref, k, method):
    """Per-launch algorithmic bytes: s * (nr * NNZ_Q + nq * NNZ_R) + nq * k * 12."""
    s = 4 if method == "binary" else 12
    nq = c1 - c0
    nnz_q = int(p[c1]) - int(p[c0])
    return s * (ncol_ref * nnz_q + nq * nnz_ref) + nq * k * 12


def cpu_baseline(p, i, x, nrow, ncol, method, k, cols, threads, keep=False):
    import scipy.sparse as sp
    from oracle import build as obuild
    from oracle.pyoracle import Oracle
    obuild.build_oracle()
    orc = Oracle(threads=threads)
    ref = sp.csc_matrix((x, i, p), shape=(nrow, ncol))
    qp, qi, qx = block_arrays(p, i, x, 0, cols)
    Q = sp.csc_matrix((qx, qi, qp), shape=(nrow, cols))
    t0 = time.perf_counter()
    idx, dst, _ = orc.knn(Q, ref, k=k, method=method, block_size=256)
    dt = time.perf_counter() - t0
    if keep:
        return cols / dt, dt, (idx, dst)
    return cols / dt, dt


def run_reference(args):
    """--impl reference: the reference's algorithm on the host cores."""
    import torch
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    device = "cuda" if torch.cuda.is_available() else "cpu"
    p, i, x = make_workload(args, device)
    threads = os.cpu_count() or 1
    cols = args.cpu_cols
    for _ in range(args.warmup):
        cpu_baseline(p, i, x, args.nrow, args.ncol, args.method, args.k, cols, threads)
    t = 0.0
    for _ in range(args.steps):
        _, dt = cpu_baseline(p, i, x, args.nrow, args.ncol, args.method, args.k, cols, threads)
        t += dt
    v = cols * args.steps / t
    print(json.dumps({
        "impl": "reference", "metric": "kNN query columns/s (sparseKNN %s k=%d, 30000x200000 log-count)" % (args.method, args.k),
        "value": v, "unit": "columns/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args, cols),
        "cpu_baseline": {"value": v, "unit": "columns/s", "cores": threads, "kind": "port",
                         "sample": "%d query columns x %d reference columns per step" % (cols, args.ncol)},
        "e2e": {"value": v, "unit": "columns/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def workload_config(args, block):
    return {"workload": "sparseKNN(X[, block], X) on a resident %dx%d log-count CSC "
                        "(nnz/col lognormal mean %.0f), %s, k=%d" % (args.nrow, args.ncol,
                                                                    args.mean_nnz, args.method, args.k),
            "nrow": args.nrow, "ncol": args.ncol, "query_block": block, "method": args.method,
            "k": args.k, "l2": "inputs larger than L2: the 4.3 GB reference is streamed every step"}


def run_uniform(args):
    """The CPU-runnable case: 2,000 x 10,000 CSC, 2 % uniform pattern, |N(0,1)|
    values; sparseKNN binary and cosine (k = 15, self-search), then
    sparseSNN(prune = 1/15, symmetrise = TRUE), through the Python API (host
    buffers in and out), against the CPU port on all host cores."""
    import torch
    import sparsedist_gb300 as sdg
    from sparsedist_gb300 import synth
    from oracle import build as obuild
    from oracle.pyoracle import Oracle
    X = synth.uniform_csc(2000, 10000, 0.02, seed=1)
    obuild.build_oracle()
    orc = Oracle(threads=os.cpu_count() or 1)
    out = {}
    for method in ("binary", "cosine"):
        for _ in range(args.warmup):
            sdg.sparseKNN(X, k=15, method=method, verbose=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            nn = sdg.sparseKNN(X, k=15, method=method, verbose=False)
        gpu_s = (time.perf_counter() - t0) / args.steps
        t0 = time.perf_counter()
        ref = orc.knn(X, k=15, method=method)
        cpu_s = time.perf_counter() - t0
        same = bool(np.array_equal(nn["idx"], ref[0]) and
                    np.array_equal(nn["dist"].view(np.uint64), ref[1].view(np.uint64)))
        out[method] = {"gpu_columns_per_s": 10000 / gpu_s, "gpu_ms": 1000 * gpu_s,
                       "cpu_columns_per_s": 10000 / cpu_s, "cpu_s": cpu_s, "identical": same}
    t0 = time.perf_counter()
    g = sdg.sparseSNN(nn, prune=1 / 15, verbose=False)
    out["snn_ms"] = 1000 * (time.perf_counter() - t0)
    out["snn_nnz"] = int(g.nnz)
    print(json.dumps({"metric": "kNN query columns/s, 2000x10000 uniform (e2e through the Python API)",
                      "config": {"workload": "2000x10000 CSC, 2% uniform, |N(0,1)|, k=15, self-search"},
                      "cores": os.cpu_count(), "results": out}))


def run_dist(args):
    """Full-matrix sparseDist(X, full = TRUE) on the 2,000-row uniform matrix
    (2,000 x dist_cols CSC, 2 % uniform pattern, |N(0,1)| values), binary,
    cosine and euclidean: the C-ABI call with host buffers (CSC in, the dense
    n x n result out) per step, the pair kernel timed by CUDA events inside
    it, bit-identical check against the oracle on a column sample, and the
    oracle's single-matrix form on the host cores on a bounded sample."""
    import scipy.sparse as sp
    import torch
    from sparsedist_gb300 import _lib, synth
    from oracle import build as obuild
    from oracle.pyoracle import Oracle
    n = args.dist_cols
    if args.dist_long:
        # long columns: the log-count generator (nnz/col lognormal mean 1,800)
        p, i, x = synth.logcount_csc(nrow=30000, ncol=n, mean_nnz=1800, seed=2, device="cuda")
        X = sp.csc_matrix((np.asarray(x), np.asarray(i), np.asarray(p)), shape=(30000, n))
        shape = "30000x%d log-count CSC (nnz/col lognormal mean 1800)" % n
    else:
        X = synth.uniform_csc(2000, n, 0.02, seed=1)
        shape = "2000x%d CSC, 2%% uniform, |N(0,1)|" % n
    obuild.build_oracle()
    threads = os.cpu_count() or 1
    orc = Oracle(threads=threads)
    ctx = _lib.Context()
    ctx.set_engine(args.engine)
    held = _lib.HeldCSC(X.shape[0], n, X.indptr, X.indices, X.data)
    D = np.empty((n, n), np.float64)
    hbm_peak, _, peak_kind = measured_peaks()
    out = {}
    for method in ("binary", "cosine", "euclidean"):
        code = METHOD_CODES[method]

        def call():
            _lib.check(ctx.lib.sdg_dist(ctx.handle, code, 1, held.ref, 1, 0, D.ctypes.data))

        for _ in range(args.warmup):
            call()
        ctx.kernel_time()
        with ClockSampler(0) as clk:
            t0 = time.perf_counter()
            for _ in range(args.steps):
                call()
            e2e_s = (time.perf_counter() - t0) / args.steps
        kms, kl = ctx.kernel_time()
        pairs = n * (n - 1) / 2
        sample = min(n, 400)
        Xs = X[:, :sample]
        want = orc.dist_single(method, Xs, True, False, True)
        same = bool(np.array_equal(D.T[:sample, :sample].view(np.uint64), want.view(np.uint64)))
        t0 = time.perf_counter()
        cs = min(n, 3000 if not args.dist_long else 600)
        orc.dist_single(method, X[:, :cs], True, False, True)
        cpu_pairs_s = cs * (cs - 1) / 2 / (time.perf_counter() - t0)
        kern_s = kms / 1000.0 / max(kl, 1)
        alg = 8.0 * n * n / 2 + 12.0 * X.nnz      # lower triangle written + the CSC read
        out[method] = {
            "pairs_per_s_e2e": pairs / e2e_s, "ms_per_step_e2e": 1000 * e2e_s,
            "pairs_per_s_kernel": pairs / kern_s, "kernel_ms": 1000 * kern_s,
            "d2h_bytes_per_step": 8 * n * n, "h2d_bytes_per_step": int(4 * (n + 1) + 12 * X.nnz),
            "roofline": {"bound": "hbm", "achieved": alg / kern_s / 1e9, "peak": hbm_peak,
                         "unit": "GB/s", "frac": alg / kern_s / 1e9 / hbm_peak,
                         "peak_kind": peak_kind, "kernel": "k_self_slab",
                         "alg_bytes_per_launch": alg},
            "cpu_baseline": {"value": cpu_pairs_s, "unit": "pairs/s", "cores": threads, "kind": "port",
                             "sample": "sparseDist(X[, 1:%d], full = TRUE)" % cs},
            "identical_on_%d_columns" % sample: same, "clocks": clk.summary()}
        torch.cuda.synchronize()
    print(json.dumps({"metric": "full-matrix sparseDist column pairs/s",
                      "config": {"workload": "sparseDist(X, full = TRUE, diag = FALSE), X " + shape,
                                 "engine": args.engine},
                      "dtype": "f64", "data": "synthetic", "steps": args.steps, "warmup": args.warmup,
                      "results": out}))


def run_snn(args):
    """sparseSNN on the log-count matrix's kNN graph: the self-search
    sparseKNN(X, k = 20, cosine) of the 30,000 x ncol log-count matrix (on
    the GPU, in sdg_knn_block shares), then sparseSNN(prune = 1/15) with
    edges = "knn" (symmetrise = TRUE) and edges = "shared" through the Python
    API (idx in from the host, the dgCMatrix slots out), each checked bit for
    bit against the oracle, which is also timed on all host cores."""
    import torch
    import sparsedist_gb300 as sdg
    from sparsedist_gb300 import _lib
    from oracle import build as obuild
    from oracle.pyoracle import Oracle
    p, i, x = make_workload(args, "cuda")
    ctx = _lib.Context(0)
    ref = _lib.Resident(ctx, args.nrow, args.ncol, p, i, x)
    del p, i, x
    torch.cuda.empty_cache()
    n, k, B = args.ncol, args.k, 8192
    idx = np.empty((n, k), np.int32)
    t0 = time.perf_counter()
    for q0 in range(0, n, B):
        nb = min(B, n - q0)
        bi = np.empty(nb * k, np.int32)
        bv = np.empty(nb * k, np.float64)
        ke, fl = np.zeros(1, np.int32), np.zeros(1, np.int32)
        _lib.check(ctx.lib.sdg_knn_block(ctx.handle, ref.handle, None, q0, nb, METHOD_CODES[args.method], 1, k,
                                         0, 1, bi.ctypes.data, bv.ctypes.data, 0, ke.ctypes.data,
                                         fl.ctypes.data))
        idx[q0:q0 + nb] = bi.reshape(int(ke[0]), nb).T
    knn_s = time.perf_counter() - t0
    ref.free()
    threads = os.cpu_count() or 1
    orc = None
    if not args.no_cpu:
        obuild.build_oracle()
        orc = Oracle(threads=threads)
    out = {"knn_graph_s": knn_s, "n": n, "k": k}
    for edges in ("knn", "shared"):
        for _ in range(args.warmup):
            g = sdg.sparseSNN(idx, prune=1 / 15, edges=edges, verbose=False, ctx=ctx)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            g = sdg.sparseSNN(idx, prune=1 / 15, edges=edges, verbose=False, ctx=ctx)
        gpu_s = (time.perf_counter() - t0) / args.steps
        out[edges] = {"gpu_ms_e2e": 1000 * gpu_s, "nodes_per_s_e2e": n / gpu_s, "nnz": int(g.nnz),
                      "cpu_baseline": None, "identical": None}
        if orc is None:
            continue
        t0 = time.perf_counter()
        if edges == "knn":
            wp, wi, wx = orc.snn_graph(idx, True, 1 / 15, True)
        else:
            wp, wi, wx = orc.snn_graph_shared(idx, True, 1 / 15)
        cpu_s = time.perf_counter() - t0
        out[edges]["identical"] = bool(np.array_equal(g.indptr, wp) and np.array_equal(g.indices, wi) and
                                       np.array_equal(g.data.view(np.uint64), np.asarray(wx).view(np.uint64)))
        out[edges]["cpu_baseline"] = {"value": n / cpu_s, "unit": "nodes/s", "cores": threads, "kind": "port",
                                      "sample": "the whole graph"}
    print(json.dumps({"metric": "sparseSNN nodes/s on the 30000x200000 log-count kNN graph (e2e through the Python API)",
                      "config": {"workload": "sparseSNN(sparseKNN(X, k=%d, %s), prune=1/15), X %dx%d "
                                             "log-count CSC" % (k, args.method, args.nrow, n)},
                      "steps": args.steps, "warmup": args.warmup, "results": out}))


def run_serve(args):
    """The serving loop: a resident 30,000 x serve_ref_cols log-count reference
    (the log-count generator), Poisson arrivals of query matrices with
    1..4,096 columns (log-uniform), methods cycling cosine / binary /
    euclidean, k in {10, 20, 50}, admission under a 120 GB budget; reports
    p50 / p99 latency (submit to completion) and columns/s."""
    import threading
    import torch
    from sparsedist_gb300 import _lib, synth
    nr = args.serve_ref_cols
    t0 = time.perf_counter()
    p, i, x = synth.logcount_csc(nrow=30000, ncol=nr, mean_nnz=1800, seed=3, device="cuda",
                                 keep_on_device=True)
    ctx = _lib.Context()
    ref = _lib.Resident.from_device(ctx, 30000, nr, p, i, x)
    nnz = int(p[-1].item())
    del p, i, x
    torch.cuda.empty_cache()
    qp, qi, qx = synth.logcount_csc(nrow=30000, ncol=20000, mean_nnz=1800, seed=4, device="cuda")
    gen_s = time.perf_counter() - t0
    codes = {"cosine": 1, "binary": 0, "euclidean": 2}
    srv = _lib.Server(ctx, ref, workers=2, max_slots=64, mem_budget=120 << 30,
                      methods=list(codes.values()))
    rng = np.random.default_rng(7)
    n = args.serve_requests
    sizes = np.clip(np.exp(rng.uniform(0, np.log(4096), n)).astype(int), 1, 4096)
    starts = rng.integers(0, 20000 - 4096, n)
    methods = [["cosine", "binary", "euclidean"][r % 3] for r in range(n)]
    ks = rng.choice([10, 20, 50], n)

    def block(c0, m):
        a, b = int(qp[c0]), int(qp[c0 + m])
        return (qp[c0:c0 + m + 1] - a).astype(np.int32), qi[a:b], qx[a:b]

    # service rate with the GPU otherwise idle: one mid-size request per method
    cal = 0.0
    cal_cols = 0
    for meth in codes:
        bp, bi, bx = block(0, 512)
        s0 = time.perf_counter()
        rid = srv.submit(30000, 512, bp, bi, bx, codes[meth], True, 20)
        srv.wait(rid)
        srv.result(rid)
        cal += time.perf_counter() - s0
        cal_cols += 512
    service_cols_per_s = cal_cols / cal
    rate = args.serve_util * service_cols_per_s / float(np.mean(sizes))
    gaps = rng.exponential(1.0 / rate, n)
    srv_stats0 = srv.stats()
    ids = []

    def submitter():
        for r in range(n):
            time.sleep(gaps[r])
            bp, bi, bx = block(int(starts[r]), int(sizes[r]))
            ids.append(srv.submit(30000, int(sizes[r]), bp, bi, bx, codes[methods[r]], True,
                                  int(ks[r])))

    t_start = time.perf_counter()
    th = threading.Thread(target=submitter)
    th.start()
    th.join()
    for rid in ids:
        srv.wait(rid)
        srv.result(rid)
    wall = time.perf_counter() - t_start
    st = srv.stats()
    # latencies of the Poisson requests only (drop the calibration requests)
    print(json.dumps({
        "metric": "served kNN columns/s + p50/p99 latency, resident 30000x1000000 log-count",
        "value": float(sizes.sum()) / wall, "unit": "columns/s",
        "p50_latency_s": st["p50_s"], "p99_latency_s": st["p99_s"], "mean_latency_s": st["mean_s"],
        "requests": n, "columns": int(sizes.sum()), "batches": int(st["batches"] - srv_stats0["batches"]),
        "arrival_rate_per_s": rate, "idle_service_columns_per_s": service_cols_per_s,
        "target_utilisation": args.serve_util, "wall_s": wall, "setup_s": gen_s,
        "config": {"workload": "resident 30000x%d log-count reference (nnz %d), Poisson arrivals, "
                               "1..4096 columns log-uniform, cosine/binary/euclidean, k in "
                               "{10,20,50}, 120 GB admission budget" % (nr, nnz)},
        "note": "latency percentiles include the 3 calibration requests"}))
    srv.close()
    ref.free()


def dense_csc(X):
    """(n, d) float32 embeddings (torch, any device) -> host CSC arrays of the
    d x n dgCMatrix the reference would receive: every value stored (exact
    zeros dropped, as Matrix does)."""
    import scipy.sparse as sp
    A = np.ascontiguousarray(X.double().cpu().numpy())
    n, d = A.shape
    M = sp.csc_matrix((A.ravel(), np.tile(np.arange(d, dtype=np.int32), n),
                       np.arange(0, (n + 1) * d, d, dtype=np.int64)), shape=(d, n))
    M.eliminate_zeros()
    return M


def dense_block_starts(args, n, B, rank, count):
    nblocks = n // B
    return [((rank * count + s) * 7919 % nblocks) * B for s in range(count)]


def dense_workload_config(args, B):
    return {"workload": "sparseKNN(X[, block], X) on resident 256x%d FP32 embeddings (N(0,1) + 1000 "
                        "Gaussian clusters sigma 0.3 + 1%% near duplicates at 1e-6), %s, k=%d, "
                        "BF16 tcgen05 screen + exact FP64 re-rank" % (args.dense_cols, args.method, args.k),
            "d": 256, "ncol": args.dense_cols, "query_block": B, "method": args.method, "k": args.k,
            "l2": "inputs larger than L2: the 1 GB BF16 reference copy is streamed every step"}


def dense_oracle_sample(Xcsc, X, q0, cols, k, method, threads):
    """The oracle's sparseKNN(X[, q0 + 0..cols-1], X) and its wall time."""
    from oracle import build as obuild
    from oracle.pyoracle import Oracle
    obuild.build_oracle()
    orc = Oracle(threads=threads)
    Q = Xcsc[:, q0:q0 + cols]
    t0 = time.perf_counter()
    idx, dst, _ = orc.knn(Q, Xcsc, k=k, method=method, block_size=256)
    return idx, dst, time.perf_counter() - t0


def run_dense_reference(args):
    """--impl reference on the dense workload: the reference's algorithm (the
    oracle port, OpenMP over all host cores) on a bounded sample of each step's
    query block against all reference columns."""
    import torch
    from sparsedist_gb300 import synth
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    d, n, B, k = 256, args.dense_cols, args.dense_block, args.k
    X = synth.dense_embeddings(d=d, n=n, seed=5, device="cuda" if torch.cuda.is_available() else "cpu")
    Xcsc = dense_csc(X)
    threads = os.cpu_count() or 1
    cols = args.ref_cols
    starts = dense_block_starts(args, n, B, 0, args.warmup + args.steps)
    for s in range(args.warmup):
        dense_oracle_sample(Xcsc, X, starts[s], cols, k, args.method, threads)
    t = 0.0
    for s in range(args.steps):
        t += dense_oracle_sample(Xcsc, X, starts[args.warmup + s], cols, k, args.method, threads)[2]
    v = cols * args.steps / t
    print(json.dumps({
        "impl": "reference", "metric": dense_metric(args), "value": v, "unit": "columns/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dense_workload_config(args, cols),
        "cpu_baseline": {"value": v, "unit": "columns/s", "cores": threads, "kind": "port",
                         "sample": "%d query columns x %d reference columns per step" % (cols, n)},
        "e2e": {"value": v, "unit": "columns/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def dense_metric(args):
    return ("kNN query columns/s, served BF16-screened vs plain GPU FP32 at exact top-k "
            "(%s k=%d, 256x%d embeddings)" % (args.method, args.k, args.dense_cols))


def run_dense_main(args):
    """The default line: dense embeddings, 256 x 2,000,000 FP32, cosine k = 20.
    One step = one block of 4,096 query columns (columns of X, passed as
    device-resident FP32 query vectors) searched against all 2,000,000
    columns: sparseKNN(X[, block], X) through sdg_dense_knn_query, mode 0 (the
    fused BF16 tcgen05 screen + exact FP64 re-rank).  The same blocks through
    mode 1 (plain FP32 SGEMM + top-k on FP32 values) give the plain GPU
    figure; e2e submits the same blocks as host vectors to the serving loop
    (sdg_server_create_dense, two workers, two requests in flight) and reads
    the results back.  The oracle computes the CPU-baseline sample, and the
    same columns' GPU results are compared with it bit for bit."""
    import ctypes as C
    import torch
    import torch.distributed as dist
    from sparsedist_gb300 import _lib, synth
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    d, n, B, k = 256, args.dense_cols, args.dense_block, args.k
    code = METHOD_CODES[args.method]
    K, W = args.steps, args.warmup
    X = synth.dense_embeddings(d=d, n=n, seed=5)
    ctx = _lib.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    h = C.c_void_p()
    _lib.check(ctx.lib.sdg_dense_upload(ctx.handle, X.data_ptr(), d, n, C.byref(h)))
    starts = dense_block_starts(args, n, B, rank, W + K)
    d_idx = torch.empty(B * k, dtype=torch.int32, device="cuda")
    d_val = torch.empty(B * k, dtype=torch.float64, device="cuda")
    ke, fl = np.zeros(1, np.int32), np.zeros(1, np.int32)

    def step(q0, mode):
        _lib.check(ctx.lib.sdg_dense_knn_query(ctx.handle, h, X[q0:q0 + B].data_ptr(), d, B, code, k, mode,
                                               d_idx.data_ptr(), d_val.data_ptr(), 1, ke.ctypes.data,
                                               fl.ctypes.data))

    def timed(mode, sample_clocks):
        for s in range(W):
            step(starts[s], mode)
        torch.cuda.synchronize()
        ctx.kernel_time()                       # reset the bounding-kernel timer
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        clk = ClockSampler(local) if sample_clocks else None
        if clk:
            clk.__enter__()
        if sample_clocks:
            torch.cuda.nvtx.range_push("sdg_timed")  # ncu --nvtx --nvtx-include sdg_timed/
        e0.record(stream)
        for s in range(K):
            step(starts[W + s], mode)
        e1.record(stream)
        if sample_clocks:
            torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        if clk:
            clk.__exit__()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        t = torch.tensor([e0.elapsed_time(e1)], dtype=torch.float64, device="cuda")
        if world > 1:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        kms, kl = ctx.kernel_time()
        return float(t.item()), kms, kl, ctx.stats(), (clk.summary() if clk else None)

    ms, kms, klaunch, st, clocks = timed(args.dense_mode, True)
    value = world * B * K / (ms / 1000.0)
    launches = int(st["kernels"]) * K
    ms1, _, _, _, _ = timed(1, False)
    plain = world * B * K / (ms1 / 1000.0)

    # roofline of the fused screen k_dense_tc: 2 * 256 * n * B BF16 flops per launch
    hbm_peak, bf16_peak, peak_kind = measured_peaks()
    flops = 2.0 * d * n * B
    per_launch_ms = kms / max(klaunch, 1)
    achieved = flops / (per_launch_ms / 1000.0) / 1e12 if klaunch else None
    roof = {"bound": "tensor", "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
            "frac": (achieved / bf16_peak) if achieved else None,
            "peak_kind": peak_kind + " (cuBLAS bf16 burst)", "kernel": "k_dense_tc (fused BF16 tcgen05 screen)",
            "flops_per_launch": flops, "kernel_ms_per_launch": per_launch_ms,
            "launches_per_step": klaunch / max(K, 1),
            "traffic": DENSE_TRAFFIC if (n == 2000000 and B == 4096 and args.method == "cosine") else None}

    # e2e: the serving loop with host query vectors, two requests in flight
    e2e = None
    if not args.no_e2e:
        hq = [np.ascontiguousarray(X[q0:q0 + B].cpu().numpy()) for q0 in starts]

        def serve(blocks):
            srv = _lib.Server(ctx, h, workers=2, max_slots=4, mem_budget=64 << 30, dense=True)
            ids, t0 = [], time.perf_counter()
            for j, q in enumerate(blocks):
                if j >= 2:
                    srv.wait(ids[j - 2])
                    srv.result(ids[j - 2])
                ids.append(srv.submit_dense(q, code, k))
            for rid in ids[-2:]:
                srv.wait(rid)
                srv.result(rid)
            dt = time.perf_counter() - t0
            stt = srv.stats()
            srv.close()
            return dt, stt

        serve(hq[:W])
        if world > 1:
            dist.barrier()
        dt, sst = serve(hq[W:])
        et = torch.tensor([dt], dtype=torch.float64, device="cuda")
        if world > 1:
            dist.all_reduce(et, op=dist.ReduceOp.MAX)
        e2e = {"value": world * B * K / float(et.item()), "unit": "columns/s",
               "h2d_bytes_per_step": B * d * 4, "d2h_bytes_per_step": B * k * 12,
               "path": "sdg_server_submit_dense / wait / result (host FP32 queries in, host idx/dist out)",
               "p50_latency_s": sst["p50_s"], "p99_latency_s": sst["p99_s"], "requests": K,
               "in_flight": 2, "batches": int(sst["batches"])}

    cpu, parity = None, None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        Xcsc = dense_csc(X)
        q0 = starts[W]
        cols = args.dense_cpu_cols
        oi, od, dt = dense_oracle_sample(Xcsc, X, q0, cols, k, args.method, threads)
        cpu = {"value": cols / dt, "unit": "columns/s", "cores": threads, "kind": "port",
               "sample": "%d query columns x %d reference columns, %.1f s" % (cols, n, dt)}
        got = {}
        for mode in (0, 1):
            gi = np.empty(cols * k, np.int32)
            gd = np.empty(cols * k, np.float64)
            _lib.check(ctx.lib.sdg_dense_knn_query(ctx.handle, h, X[q0:q0 + cols].data_ptr(), d, cols, code, k,
                                                   mode, gi.ctypes.data, gd.ctypes.data, 0, ke.ctypes.data,
                                                   fl.ctypes.data))
            got[mode] = (gi.reshape(k, cols).T, gd.reshape(k, cols).T)
        parity = {"cols": cols, "vs": "oracle (the reference's algorithm, FP64)",
                  "bf16_screened": {"idx_identical": bool(np.array_equal(got[0][0], oi)),
                                    "dist_bit_identical": bool(np.array_equal(got[0][1].view(np.uint64),
                                                                              od.view(np.uint64))),
                                    "max_abs_dist_err": float(np.max(np.abs(got[0][1] - od)))},
                  "plain_fp32": {"idx_agree_frac": float(np.mean(got[1][0] == oi)),
                                 "rows_identical": int(np.sum(np.all(got[1][0] == oi, axis=1))),
                                 "max_abs_dist_err": float(np.max(np.abs(got[1][1] - od)))}}
    if rank == 0:
        line = {
            "metric": dense_metric(args), "value": value, "unit": "columns/s", "n_gpus": world, "steps": K,
            "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 screen, f64 re-rank", "data": "synthetic",
            "config": dense_workload_config(args, B) | {"parallelism": "query-column shards x%d" % world},
            "plain_fp32": {"value": plain, "unit": "columns/s", "ms_per_step": ms1 / K,
                           "path": "sdg_dense_knn_query mode 1 (FP32 SGEMM, top-k on FP32 values)"},
            "vs_plain_fp32": value / plain,
            "e2e": e2e, "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu, "parity": parity,
            "clocks": clocks, "stats_last_call": st}
        print(json.dumps(line))
    ctx.lib.sdg_dense_free(h)
    if world > 1:
        dist.destroy_process_group()


# dram__bytes_read.sum + dram__bytes_write.sum of one launch of the bounding
# kernel at the bench's full size, from a one-pass ncu capture
# (profiles/k_dense_tc_cosine_2000000x256_q4096.md,
# profiles/launches_logcount_cosine_30000x200000_q4096.md)
DENSE_TRAFFIC = 7.03e9 + 0.145e9
LOGCOUNT_TRAFFIC = 65.22e9 + 0.181e9


def run_batched(args):
    """Batched uneven sparseKNNCross problems (the 512-problem draw of
    synth.cross_draw: nq log-U[100, 50,000], nr log-U[1,000, 200,000], rows
    U[5,000, 30,000], density log-U[0.1 %, 10 %], methods cycling binary /
    cosine / manhattan / js, k in {10, 20, 50}) through sdg_knn_cross_batch,
    --batch-group problems per call (host CSC in, host results out: each call
    uploads its problems, runs every exact-path search in one persistent
    launch and the others on the engines the autotuner picks, and copies the
    results back).  value = forward + reverse query columns / the calls' wall
    time; the problems are generated on the GPU outside the timed calls.  The
    smallest problems are checked against the oracle, which also gives the
    CPU baseline on them."""
    import torch
    from sparsedist_gb300 import _lib, synth
    from oracle import build as obuild
    from oracle.pyoracle import Oracle
    specs = synth.cross_draw(args.batch_problems, seed=4, scale=args.batch_scale)
    ctx = _lib.Context()
    t_calls, cols, pairs = 0.0, 0, 0.0
    engines = {}
    eng_s = [0.0, 0.0, 0.0]
    kept = []
    by_size = sorted(range(len(specs)), key=lambda p: specs[p]["nq"] * specs[p]["nr"])
    check_set = set(by_size[:args.batch_check])
    for g0 in range(0, len(specs), args.batch_group):
        group = specs[g0:g0 + args.batch_group]
        probs = [synth.cross_problem(sp_) for sp_ in group]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc, res = _lib.knn_cross_batch(ctx, [(X, Y, METHOD_CODES[sp_["method"]], True, sp_["k"])
                                             for (X, Y), sp_ in zip(probs, group)])
        t_calls += time.perf_counter() - t0
        for e, sec in enumerate(_lib.knn_cross_batch.engine_seconds):
            eng_s[e] += sec
        if rc != 0:
            raise RuntimeError("sdg_knn_cross_batch: %s" % [r["status"] for r in res])
        for j, ((X, Y), sp_, r) in enumerate(zip(probs, group, res)):
            cols += X.shape[1] + Y.shape[1]
            pairs += 2.0 * X.shape[1] * Y.shape[1]
            for d, e in zip(("forward", "reverse"), r["engines"]):
                key = "%s/engine%d" % (sp_["method"], e)
                engines[key] = engines.get(key, 0) + 1
            if g0 + j in check_set:
                kept.append((X, Y, sp_, r))
        del probs
    obuild.build_oracle()
    threads = os.cpu_count() or 1
    orc = Oracle(threads=threads)
    identical, close, total = 0, 0, 0
    t_cpu, cpu_cols = 0.0, 0
    for X, Y, sp_, r in kept:
        t0 = time.perf_counter()
        (wfi, wfd), (wri, wrd), _ = orc.knn_cross(X, Y, k=sp_["k"], method=sp_["method"])
        t_cpu += time.perf_counter() - t0
        cpu_cols += X.shape[1] + Y.shape[1]
        total += 1
        same = all(np.array_equal(a, b) for a, b in ((r["forward"][0], wfi), (r["reverse"][0], wri))) and all(
            np.array_equal(a.view(np.uint64), b.view(np.uint64)) for a, b in ((r["forward"][1], wfd), (r["reverse"][1], wrd)))
        identical += int(same)
        if not same:
            ok = all(np.allclose(a, b, rtol=1e-12, atol=0, equal_nan=True)
                     for a, b in ((r["forward"][1], wfd), (r["reverse"][1], wrd)))
            close += int(ok)
    print(json.dumps({
        "metric": "batched sparseKNNCross query columns/s (%d uneven problems, forward + reverse, e2e through "
                  "sdg_knn_cross_batch)" % len(specs),
        "value": cols / t_calls, "unit": "columns/s", "n_gpus": 1, "higher_is_better": True,
        "seconds": t_calls, "columns": cols, "pairs": pairs, "calls": (len(specs) + args.batch_group - 1) // args.batch_group,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": "synth.cross_draw(%d, seed=4, scale=%g): nq log-U[100,50000], nr log-U[1000,200000], "
                               "rows U[5000,30000], density log-U[0.1%%,10%%], binary/cosine/manhattan/js, "
                               "k in {10,20,50}" % (len(specs), args.batch_scale),
                   "problems_per_call": args.batch_group},
        "engines": engines,
        "engine_seconds": {"exact_batched": eng_s[0], "fp32_screen": eng_s[1], "tensor_screen": eng_s[2],
                           "other (uploads, preparation, copies)": t_calls - sum(eng_s)},
        "parity": {"problems": total, "bit_identical": identical, "js_within_1e-12": close,
                   "vs": "oracle (the reference's algorithm), the %d smallest problems" % total},
        "cpu_baseline": {"value": cpu_cols / t_cpu if t_cpu else None, "unit": "columns/s", "cores": threads,
                         "kind": "port", "sample": "the %d smallest problems, forward + reverse" % total}}))


def main():
    args = parse()
    if args.config == "dense":
        if args.impl == "reference":
            run_dense_reference(args)
        else:
            run_dense_main(args)
        return
    if args.config == "uniform":
        run_uniform(args)
        return
    if args.config == "serve":
        run_serve(args)
        return
    if args.config == "dist":
        run_dist(args)
        return
    if args.config == "snn":
        run_snn(args)
        return
    if args.config == "batched":
        run_batched(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    run_logcount(args)


def run_logcount(args):
    """--config logcount: sparse kNN at scale (the 30,000 x 200,000 log-count
    matrix, cosine k = 20, 4,096-query blocks), the tensor-core screen of the
    sparse path; the CPU-baseline sample's oracle result is compared with the
    GPU's result on the same columns bit for bit."""
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    from sparsedist_gb300 import _lib
    p, i, x = make_workload(args, "cuda")
    nnz_ref = int(p[-1])
    ctx = _lib.Context(local)
    ctx.set_engine(args.engine)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    lib = ctx.lib
    ref = _lib.Resident(ctx, args.nrow, args.ncol, p, i, x)

    B, K, W, k = args.block, args.steps, args.warmup, args.k
    method = METHOD_CODES[args.method]
    nblocks = args.ncol // B
    steps = [((rank * (K + W) + s) % nblocks) * B for s in range(W + K)]
    queries = [_lib.Resident(ctx, args.nrow, B, *block_arrays(p, i, x, c0, c0 + B)) for c0 in steps]
    d_idx = torch.empty(B * k, dtype=torch.int32, device="cuda")
    d_val = torch.empty(B * k, dtype=torch.float64, device="cuda")
    keff = np.zeros(1, np.int32)
    flags = np.zeros(1, np.int32)

    def step(q):
        _lib.check(lib.sdg_knn_resident_device(ctx.handle, q.handle, ref.handle, method, 1, k, 0, 1,
                                               d_idx.data_ptr(), d_val.data_ptr(),
                                               keff.ctypes.data, flags.ctypes.data))

    for s in range(W):
        step(queries[s])
    torch.cuda.synchronize()
    ctx.kernel_time()                      # reset
    stats_launches = 0
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.nvtx.range_push("sdg_timed")      # ncu --nvtx-include sdg_timed/
        e0.record(stream)
        for s in range(K):
            step(queries[W + s])
        e1.record(stream)
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    kms, klaunch = ctx.kernel_time()
    stats_launches = ctx.stats()["kernels"]
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    value = world * B * K / (ms_max / 1000.0)

    # roofline of the bounding kernel (per launch)
    alg = np.mean([bytes_alg(p, c0, c0 + B, nnz_ref, args.ncol, k, args.method) for c0 in steps[W:]])
    launches_per_step = max(1, klaunch // max(K, 1))
    per_launch_ms = kms / max(klaunch, 1)
    achieved = (alg / launches_per_step) / (per_launch_ms / 1000.0) / 1e9 if klaunch else None
    hbm_peak, bf16_peak, peak_kind = measured_peaks()
    st_last = ctx.stats()
    if st_last.get("tensor_flops", 0) > 0 and klaunch:
        # the tensor-core screen: the fused tcgen05 kernel is the bounding kernel
        flops_launch = st_last["tensor_flops"] / launches_per_step
        roof = {"bound": "tensor", "achieved": flops_launch / (per_launch_ms / 1000.0) / 1e12,
                "peak": bf16_peak, "unit": "TFLOP/s",
                "peak_kind": peak_kind + " (bf16 burst; fp16 runs at the same tensor rate)",
                "kernel": "k_sparse_tc (fused FP16 tcgen05 screen)", "flops_per_launch": flops_launch}
    else:
        roof = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "peak_kind": peak_kind, "kernel": "k_screen", "alg_bytes_per_launch": alg / launches_per_step}
    roof["frac"] = (roof["achieved"] / roof["peak"]) if roof["achieved"] else None
    roof["traffic"] = LOGCOUNT_TRAFFIC if (roof["bound"] == "tensor" and args.ncol == 200000 and
                                          args.nrow == 30000 and B == 4096) else None
    roof["kernel_ms_per_launch"] = per_launch_ms
    # the sparse-slab figure of merit (operand bytes a pairwise merge walk streams)
    roof["sparse_alg_gbs"] = achieved

    # end to end through the C ABI with host buffers (pinned)
    e2e = None
    if not args.no_e2e:
        hq = []
        for c0 in steps:
            bp, bi, bx = block_arrays(p, i, x, c0, c0 + B)
            pins = []
            for a in (bp, bi, bx):
                t_ = torch.empty(a.shape, dtype={np.int32: torch.int32, np.float64: torch.float64}[a.dtype.type],
                                 pin_memory=True)
                t_.numpy()[:] = a
                pins.append(t_)
            hq.append(pins)
        h_idx = torch.empty(B * k, dtype=torch.int32, pin_memory=True)
        h_val = torch.empty(B * k, dtype=torch.float64, pin_memory=True)

        def e2e_step(pins):
            held = _lib.HeldCSC(args.nrow, B, pins[0].numpy(), pins[1].numpy(), pins[2].numpy())
            h = __import__("ctypes").c_void_p()
            _lib.check(lib.sdg_matrix_upload(ctx.handle, held.ref, __import__("ctypes").byref(h)))
            _lib.check(lib.sdg_knn_resident(ctx.handle, h, ref.handle, method, 1, k, 0, 1,
                                            h_idx.data_ptr(), h_val.data_ptr(), keff.ctypes.data,
                                            flags.ctypes.data))
            lib.sdg_matrix_free(h)

        for s in range(W):
            e2e_step(hq[s])
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        t0 = time.perf_counter()
        for s in range(K):
            e2e_step(hq[W + s])
        torch.cuda.synchronize()
        et = torch.tensor([time.perf_counter() - t0], dtype=torch.float64, device="cuda")
        if world > 1:
            dist.all_reduce(et, op=dist.ReduceOp.MAX)
        h2d = int(np.mean([sum(a.numel() * a.element_size() for a in pins) for pins in hq[W:]]))
        e2e = {"value": world * B * K / float(et.item()), "unit": "columns/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": B * k * 12}

    cpu, parity = None, None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, dt, (oi, od) = cpu_baseline(p, i, x, args.nrow, args.ncol, args.method, k, args.cpu_cols, threads,
                                       keep=True)
        cpu = {"value": v, "unit": "columns/s", "cores": threads, "kind": "port",
               "sample": "%d query columns x %d reference columns (one reference block), %.1f s"
                         % (args.cpu_cols, args.ncol, dt)}
        # the same columns through the library (the bench step's call, host outputs)
        cols = args.cpu_cols
        q = _lib.Resident(ctx, args.nrow, cols, *block_arrays(p, i, x, 0, cols))
        gi = np.empty(cols * k, np.int32)
        gd = np.empty(cols * k, np.float64)
        _lib.check(lib.sdg_knn_resident(ctx.handle, q.handle, ref.handle, method, 1, k, 0, 1, gi.ctypes.data,
                                        gd.ctypes.data, keff.ctypes.data, flags.ctypes.data))
        q.free()
        gi, gd = gi.reshape(k, cols).T, gd.reshape(k, cols).T
        parity = {"cols": cols, "vs": "oracle (the reference's algorithm, FP64)",
                  "identical": bool(np.array_equal(gi, oi) and np.array_equal(gd.view(np.uint64),
                                                                               od.view(np.uint64)))}

    if rank == 0:
        st = ctx.stats()
        line = {
            "metric": "kNN query columns/s (sparseKNN %s k=%d, 30000x200000 log-count)" % (args.method, args.k),
            "value": value, "unit": "columns/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, B) | {"parallelism": "query-column shards x%d" % world,
                                                  "nnz": nnz_ref, "engine": args.engine},
            "e2e": e2e,
            "gpu_launches": int(stats_launches) * K,
            "roofline": roof,
            "cpu_baseline": cpu,
            "parity": parity,
            "clocks": clk.summary(),
            "stats_last_call": st,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

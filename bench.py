#!/usr/bin/env python
"""Benchmark of the exact-kNN hot path on one GB300.

Workload (one step): the 784-d quantised Gaussian-mixture set -- N=60,000
points, Q=10,000 held-out queries, SqEuclidean, k=10 -- searched for the
held-out queries AND materialised as the self kNN graph of the 60,000 points
(build_knn_graph semantics).  A step therefore answers 70,000 queries.

Arms
  (default)          the BF16 tensor-core form with certified candidates,
                     exact FP32 rerank and FP64 ordering of near-ties at the
                     k-th distance (MANN_FLAG_FP64_TIES): the sets equal the
                     FP64 oracle's, checked on sampled rows after the timed
                     region.  `value` has the inputs resident in HBM; `e2e`
                     goes through the C ABI with pinned host buffers (copies
                     inside the timed region).  The plain FP32 form and the
                     other workloads (plain 64-d kNN, angular cosine, batched
                     uneven graphs, 1M x 128 IVF with the learned probe) are
                     timed beside it, each with its CPU baseline.
  --impl reference   the reference's BruteForceIndex algorithm restated in C
                     (OpenMP over every host core) on a bounded sample of the
                     same step: held-out queries as one batch (threads over
                     queries) and self-graph columns one query at a time with
                     threads inside the query (src/graphs/knn_graph.jl:63-67),
                     in the step's 1:6 proportion.

Prints ONE JSON line on rank 0.  Multi-GPU (torchrun): replicas only.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_POINTS, N_QUERIES, DIM, K = 60000, 10000, 784, 10
WORKLOAD = "quantized-mixture-784d: N=60000 points + Q=10000 held-out queries, SqEuclidean, k=10, plus the 60000-point self kNN graph"
METRIC = "kNN queries/s: BF16+rerank vs FP32 at recall@10=1.0; learned-probe QPS@0.95"
IVF_N, IVF_Q, IVF_D, IVF_NLIST, IVF_TRAIN = 1_000_000, 10_000, 128, 4096, 200_000
IVF_WORKLOAD = ("anisotropic-clusters-128d: N=1,000,000 points from 1,024 Gaussian clusters (sigma per dim "
                "log-uniform in [0.05, 0.5]), Q=10,000 queries, SqEuclidean, k=10; IVF-Flat nlist=4,096 "
                "(KMeans: k-means++ + 25 Lloyd iterations); probe MLP 128-512-512-4096 (GELU) trained on the "
                "exact top-10 lists of 200,000 separate training queries")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--fp32-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU-baseline sample budget")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--ivf-epochs", type=int, default=30)
    ap.add_argument("--no-ivf", action="store_true", help="skip the learned-probe IVF leg")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched uneven graphs leg")
    ap.add_argument("--no-angular", action="store_true", help="skip the angular (cosine) leg")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain 64-d FP32 leg")
    ap.add_argument("--no-fp8", action="store_true", help="skip the FP8-form measurement")
    ap.add_argument("--case", choices=["full", "profile", "ivf", "batched", "batched-profile", "ivf-profile", "angular",
                                       "angular-profile", "plain"],
                    default="full",
                    help="profile: BF16 steps only (query batch + self graph, two k2_main "
                         "launches per step), for ncu captures")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi samples (200 ms) while the timed region runs."""

    def __init__(self, gpu_index: int):
        self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.tmp, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.tmp.flush()
        self.tmp.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.tmp.read().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.tmp.name)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def make_workload():
    from manifoldann_gb300 import synthetic

    base = synthetic.quantized_mixture(N_POINTS, DIM, seed=1)
    q = synthetic.quantized_mixture(N_QUERIES, DIM, seed=2)
    return base, q


CONFIG = {"workload": WORKLOAD, "metric": "SqEuclidean", "k": K, "queries_per_step": N_QUERIES + N_POINTS,
          "order": "FP64 near-tie order at the k-th distance (sets identical to the FP64 oracle)",
          "l2": "inputs larger than L2 (188 MB fp32 points)"}
# the CPU sample of one step: held-out queries as a batch, self-graph columns one at a time (1:6)
CPU_STEP_QUERIES, CPU_STEP_COLUMNS = 64, 384


def measured_peaks():
    """(bf16 burst TF/s, bf16 sustained TF/s, HBM GB/s, source).  The burst
    figure is the denominator for kernels timed over a short region (the
    timed steps here last well under a second)."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        j = json.loads(p.read_text())
        return (j.get("bf16_tflops", 1926.8), j.get("bf16_tflops_sustained", 1737.1), j.get("hbm_gbs", 6703.5),
                "measured")
    return 1900.0, 1700.0, 6800.0, "fallback"


_FP32_PEAK = None


def fp32_peak():
    """Measured FP32 FMA rate of this GPU (TF/s) from the library's FMA-chain
    kernel, timed with CUDA events; the SM clock seen during the measurement."""
    global _FP32_PEAK
    if _FP32_PEAK is None:
        from manifoldann_gb300 import _lib

        lib = _lib.load()
        sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
        best = 0.0
        for _ in range(3):
            tf, ms = C.c_double(), C.c_double()
            _lib.check(lib.mann_measure_fp32_peak(C.byref(tf), C.byref(ms)))
            best = max(best, tf.value)
        clk = sampler.stop()
        _FP32_PEAK = {"tflops": best, "sm_mhz": clk.get("sm_mhz"), "how": "mann_measure_fp32_peak: 16 "
                      "independent FMA chains per thread (f32x2 and scalar forms), 8 blocks x 256 threads per SM, "
                      "CUDA events, best of 3"}
    return _FP32_PEAK


def profiled_traffic():
    """DRAM bytes per k2_main main-pass launch from the committed ncu summary."""
    p = ROOT / "profiles" / "k2_main_bf16_knn_60k_784.md"
    if p.exists():
        for line in p.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1].split()[0])
    return None


def cpu_step(oracle, base, q, i, threads, nq=CPU_STEP_QUERIES, ncols=CPU_STEP_COLUMNS):
    """One CPU sample of the headline step (the reference's algorithm restated
    in C): `nq` held-out queries as one batch (threads over queries,
    src/ann_index.jl:91-98) and `ncols` self-graph columns, each one k+1
    query with threads inside it, the self id dropped
    (src/graphs/knn_graph.jl:63-67,105-130)."""
    s = (i * nq) % (N_QUERIES - nq)
    oracle.cpu_bruteforce_batch(base, q[s:s + nq], K, oracle.SQEUCLIDEAN, threads)
    c0 = (i * ncols) % (N_POINTS - ncols)
    for c in range(c0, c0 + ncols):
        ids, _ = oracle.cpu_bruteforce_batch(base, base[c:c + 1], K + 1, oracle.SQEUCLIDEAN, threads)
    return nq + ncols


def cpu_baseline(base, q, budget_s):
    """The reference algorithm (the oracle's OpenMP restatement) on a bounded sample of the step."""
    import oracle

    threads = os.cpu_count() or 1
    oracle.load()
    cpu_step(oracle, base, q, 0, threads, 16, 96)  # warm-up
    t0 = time.perf_counter()
    done, i = 0, 1
    while time.perf_counter() - t0 < budget_s:
        done += cpu_step(oracle, base, q, i, threads)
        i += 1
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"{i - 1} samples of {CPU_STEP_QUERIES} held-out queries (one batch) + {CPU_STEP_COLUMNS} "
                      f"self-graph columns (one k+1 query each) against all {N_POINTS} points (d={DIM}, k={K}), "
                      f"{dt:.1f} s wall on {threads} host threads"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    base, q = make_workload()
    import oracle

    oracle.load()
    threads = os.cpu_count() or 1
    for i in range(args.warmup):
        cpu_step(oracle, base, q, i, threads)
    t0 = time.perf_counter()
    done = 0
    for i in range(args.steps):
        done += cpu_step(oracle, base, q, args.warmup + i, threads)
    dt = time.perf_counter() - t0
    qps = done / dt
    line = {"metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference", "config": CONFIG,
            "step": f"{CPU_STEP_QUERIES} held-out queries (one batch) + {CPU_STEP_COLUMNS} self-graph columns "
                    "(one k+1 query each): a bounded sample of the 10,000 + 60,000 queries of the step, same mix",
            "parallelism": f"{threads} host threads",
            "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
                             "sample": f"{done // args.steps} queries per step x {args.steps} steps; the reference "
                                       "BruteForceIndex / build_knn_graph algorithm restated in C (Julia is not "
                                       "installed)"},
            "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_profile_case(args):
    """Case for ncu: BF16 steps only (the held-out queries, then the self graph)."""
    import torch

    from manifoldann_gb300 import _lib

    lib = _lib.load()
    base, q = make_workload()
    tb = torch.from_numpy(base).cuda()
    tq = torch.from_numpy(q).cuda()
    qi = torch.empty((N_QUERIES, K), dtype=torch.int32, device="cuda")
    qd = torch.empty((N_QUERIES, K), dtype=torch.float32, device="cuda")
    gi = torch.empty((N_POINTS, K), dtype=torch.int32, device="cuda")
    gd = torch.empty((N_POINTS, K), dtype=torch.float32, device="cuda")
    sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = _lib.params(_lib.METRIC_SQEUCLIDEAN, K, _lib.PREC_BF16, 0, _lib.FLAG_FP64_TIES)
    for _ in range(args.warmup + args.steps):
        _lib.check(lib.mann_knn_device(p, tb.data_ptr(), N_POINTS, tq.data_ptr(), N_QUERIES, DIM,
                                       qi.data_ptr(), qd.data_ptr(), None, sp))
        _lib.check(lib.mann_knn_graph_device(p, tb.data_ptr(), N_POINTS, DIM, 0, gi.data_ptr(),
                                             gd.data_ptr(), None, sp))
    torch.cuda.synchronize()
    print(json.dumps({"case": "profile", "steps": args.warmup + args.steps,
                      "k2_main_launches": 2 * (args.warmup + args.steps)}), flush=True)
    return 0


def run_angular_profile_case(args):
    """Case for ncu: the FP16-form cosine call on the angular set (290,000 x
    256 points, 10,000 queries, k = 20) only, warmup + steps calls."""
    import torch

    from manifoldann_gb300 import _lib, synthetic

    lib = _lib.load()
    n, nq, d, k = 290000, 10000, 256, 20
    base = torch.from_numpy(synthetic.angular_clusters(n, d, seed=1)).cuda()
    q = torch.from_numpy(synthetic.angular_clusters(nq, d, seed=2)).cuda()
    ids = torch.empty((nq, k), dtype=torch.int32, device="cuda")
    dd = torch.empty((nq, k), dtype=torch.float32, device="cuda")
    sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = _lib.params(_lib.METRIC_COSINE, k, _lib.PREC_FP16)
    for _ in range(args.warmup + args.steps):
        _lib.check(lib.mann_knn_device(p, base.data_ptr(), n, q.data_ptr(), nq, d, ids.data_ptr(), dd.data_ptr(),
                                       None, sp))
    torch.cuda.synchronize()
    print(json.dumps({"case": "angular-profile", "calls": args.warmup + args.steps}), flush=True)
    return 0


def run_ivf_leg(args, stream_ptr=0):
    """Learned-probe IVF beside the exact scan on the 1M x 128 set: build,
    train, sweep nprobe for the learned probe and for centroid routing, and
    time each at the smallest nprobe that reaches recall@10 >= 0.95."""
    import torch

    import manifoldann_gb300 as M
    from manifoldann_gb300 import _lib, synthetic
    from manifoldann_gb300.probe import neighbour_list_labels

    lib = _lib.load()
    X = synthetic.anisotropic_clusters(IVF_N, IVF_D, seed=1)
    TQ = synthetic.anisotropic_clusters(IVF_TRAIN, IVF_D, seed=2)
    Q = synthetic.anisotropic_clusters(IVF_Q, IVF_D, seed=3)
    t0 = time.perf_counter()
    idx = M.build_index(M.IVFFlatIndex, X.T, nlist=IVF_NLIST, distance=M.SqEuclidean(), seed=1)
    build_s = time.perf_counter() - t0
    dev = torch.device("cuda")
    Xd = torch.from_numpy(X).to(dev)
    Qd = torch.from_numpy(Q).to(dev)
    Cd = torch.from_numpy(np.ascontiguousarray(idx.centroids.T)).to(dev)
    od = torch.from_numpy(idx.list_offsets).to(dev)
    idd = torch.from_numpy(idx.list_ids).to(dev)
    oi = torch.empty((IVF_Q, K), dtype=torch.int32, device=dev)
    odist = torch.empty((IVF_Q, K), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    exact = {}
    answers = {}
    for name, prec in (("fp32", _lib.PREC_FP32), ("fp16", _lib.PREC_FP16), ("bf16", _lib.PREC_BF16)):
        pp = _lib.params(_lib.METRIC_SQEUCLIDEAN, K, prec)
        ms = timed(lambda: _lib.check(lib.mann_knn_device(pp, Xd.data_ptr(), IVF_N, Qd.data_ptr(), IVF_Q, IVF_D,
                                                          oi.data_ptr(), odist.data_ptr(), None, stream_ptr)),
                   2 if prec == _lib.PREC_FP32 else 5)
        exact[name] = {"ms": ms, "qps": IVF_Q / (ms / 1e3)}
        answers[name] = (oi.cpu().numpy().copy(), odist.cpu().numpy().copy())
    exact["fp16"]["equals_bf16_form"] = bool(np.array_equal(answers["fp16"][0], answers["bf16"][0]) and
                                             np.array_equal(answers["fp16"][1].view(np.uint32),
                                                            answers["bf16"][1].view(np.uint32)))
    truth = answers["bf16"][0]  # the BF16 form's certified exact top-10
    t0 = time.perf_counter()
    labels = neighbour_list_labels(idx, X.T, TQ.T, K)
    label_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    model = M.ProbeModel(IVF_D, IVF_NLIST, (512, 512), use_prior=False, batch=1024, lr=1e-3,
                         weight_decay=1e-4, seed=0)
    loss = model.train(TQ, labels, args.ivf_epochs)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    p = _lib.params(_lib.METRIC_SQEUCLIDEAN, K, _lib.PREC_FP32)

    def learned(npb):
        _lib.check(lib.mann_ivf_search_learned_device(model.handle, p, npb, Xd.data_ptr(), IVF_N, IVF_D, IVF_NLIST,
                                                      od.data_ptr(), idd.data_ptr(), Qd.data_ptr(), IVF_Q,
                                                      oi.data_ptr(), odist.data_ptr(), stream_ptr))

    def centroid(npb):
        _lib.check(lib.mann_ivf_search_device(p, npb, _lib.METRIC_SQEUCLIDEAN, Xd.data_ptr(), IVF_N, IVF_D,
                                              Cd.data_ptr(), IVF_NLIST, od.data_ptr(), idd.data_ptr(),
                                              Qd.data_ptr(), IVF_Q, oi.data_ptr(), odist.data_ptr(), stream_ptr))

    def recall():
        got = oi.cpu().numpy()
        return float(sum(len(set(got[i]) & set(truth[i])) for i in range(IVF_Q)) / (10.0 * IVF_Q))

    out = {}
    for name, fn in (("learned", learned), ("centroid", centroid)):
        sweep, chosen = [], None
        for npb in (1, 2, 3, 4, 5, 6, 8, 12, 16, 24, 32):
            fn(npb)
            torch.cuda.synchronize()
            r = recall()
            sweep.append([npb, r])
            if r >= 0.95:
                chosen = (npb, r)
                break
        res = {"sweep": sweep}
        if chosen:
            ms = timed(lambda: fn(chosen[0]), max(args.steps, 5))
            res.update({"nprobe": chosen[0], "recall_at_10": chosen[1], "ms": ms, "qps": IVF_Q / (ms / 1e3)})
        out[name] = res
    # e2e: host buffers through the C ABI (data, queries and lists copied every call)
    e2e = None
    if "qps" in out["learned"] and not args.no_e2e:
        hq = np.ascontiguousarray(Q)
        hi = np.empty((IVF_Q, K), np.int32)
        hd = np.empty((IVF_Q, K), np.float32)
        lib.mann_host_register(X.ctypes.data, X.nbytes)
        lib.mann_host_register(hq.ctypes.data, hq.nbytes)
        npb = out["learned"]["nprobe"]

        def host():
            _lib.check(lib.mann_ivf_search_learned(model.handle, p, npb, X.ctypes.data, IVF_N, IVF_D, IVF_NLIST,
                                                   idx.list_offsets.ctypes.data, idx.list_ids.ctypes.data,
                                                   hq.ctypes.data, IVF_Q, hi.ctypes.data, hd.ctypes.data))

        host()
        t0 = time.perf_counter()
        reps = max(3, min(args.steps, 10))
        for _ in range(reps):
            host()
        dt = (time.perf_counter() - t0) / reps
        lib.mann_host_unregister(X.ctypes.data)
        lib.mann_host_unregister(hq.ctypes.data)
        e2e = {"value": IVF_Q / dt, "unit": "queries/s",
               "h2d_bytes_per_step": int(X.nbytes + hq.nbytes + idx.list_offsets.nbytes + idx.list_ids.nbytes),
               "d2h_bytes_per_step": int(IVF_Q * K * 8)}
    # list-scan roofline: the scan of the learned probes alone (mann_ivf_scan_device,
    # routing excluded), bytes = every probed list's rows read once per query
    roof = None
    if "nprobe" in out["learned"]:
        npb = out["learned"]["nprobe"]
        probes = torch.empty((IVF_Q, npb), dtype=torch.int32, device=dev)
        model.route_device(Qd, npb, probes, stream=stream_ptr)
        torch.cuda.synchronize()
        sizes = np.diff(idx.list_offsets)
        pr = probes.cpu().numpy()
        rows_read = float(sizes[pr[pr >= 0]].sum())  # (query, probed list) pairs' points
        probed = np.unique(pr[pr >= 0])
        # algorithmic bytes: every probed list's points read once (its queries share the read),
        # plus the queries and the results
        scan_bytes = float(sizes[probed].sum()) * IVF_D * 4 + IVF_Q * IVF_D * 4 + IVF_Q * K * 8

        def scan_only():
            _lib.check(lib.mann_ivf_scan_device(p, probes.data_ptr(), npb, Xd.data_ptr(), IVF_N, IVF_D, IVF_NLIST,
                                                od.data_ptr(), idd.data_ptr(), Qd.data_ptr(), IVF_Q,
                                                oi.data_ptr(), odist.data_ptr(), stream_ptr))

        scan_ms = timed(scan_only, max(args.steps, 5))
        _, _, hbm, src = measured_peaks()
        ach = scan_bytes / (scan_ms / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": "ivf_scan_kernel + merge (learned probes given)", "achieved": ach,
                "peak": hbm, "unit": "GB/s", "frac": ach / hbm, "ms": scan_ms,
                "bytes": scan_bytes, "rows_scanned_per_query": rows_read / IVF_Q,
                "lists_probed": int(len(probed)),
                "peak_source": f"{src} HBM copy bandwidth",
                "work": "each probed list's rows x d x 4 B once (the queries of a list share its read), "
                        "+ queries and results"}
    # CPU baselines: the reference's exact batch and its IVF-Flat query (GEMV-form
    # centroid distances, partialsortperm, bounded-heap list scan) on query samples
    cpu = None
    if args.cpu_seconds > 0:
        import oracle

        oracle.load()
        threads = os.cpu_count() or 1
        m = 64
        t0 = time.perf_counter()
        oracle.cpu_bruteforce_batch(X, Q[:m], K, oracle.SQEUCLIDEAN, threads)
        ex_dt = time.perf_counter() - t0
        npc = out["centroid"].get("nprobe", 4)
        Cr = np.ascontiguousarray(idx.centroids.T)
        cn = np.array([np.float32(np.dot(c, c)) for c in Cr], np.float32)
        m2 = IVF_Q
        t0 = time.perf_counter()
        from manifoldann_gb300.distances import metric_code

        oracle.ivf_query_f32(X, Cr, cn, idx.list_offsets, idx.list_ids, Q[:m2], K, npc, oracle.SQEUCLIDEAN,
                             metric_code(idx.centroid_metric), threads)
        ivf_dt = time.perf_counter() - t0
        cpu = {"exact": {"value": m / ex_dt, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": f"{m} queries against all {IVF_N} points, {ex_dt:.1f} s"},
               "ivf_flat_centroid_routing": {"value": m2 / ivf_dt, "unit": "queries/s", "cores": threads,
                                             "kind": "port", "nprobe": npc,
                                             "sample": f"{m2} queries, nprobe {npc}, {ivf_dt:.1f} s "
                                                       "(reference IVF-Flat query restated in C)"}}
    best_exact = max(exact["fp32"]["qps"], exact["bf16"]["qps"], exact["fp16"]["qps"])
    res = {"workload": IVF_WORKLOAD, "build_s": build_s, "label_s": label_s, "train_s": train_s,
           "train_epochs": args.ivf_epochs, "final_loss": float(loss[-1]), "exact": exact,
           "learned": out["learned"], "centroid_routing": out["centroid"], "e2e_learned": e2e,
           "roofline_scan": roof, "cpu_baseline": cpu}
    if "qps" in out["learned"]:
        res["learned_over_exact"] = out["learned"]["qps"] / best_exact
        res["learned_over_exact_fp32"] = out["learned"]["qps"] / exact["fp32"]["qps"]
    return res


BATCH_WORKLOAD = ("manifold-clouds-32d: 64 point clouds, sizes log-uniform in [2,000, 50,000] (Swiss roll, "
                  "2-sphere, torus in R^3, zero-padded to 32-d, rotated, noise 0.01), SqEuclidean self-kNN k=15 "
                  "per cloud, one launch per step replayed from a CUDA graph")


def run_batched_leg(args, stream_ptr=0):
    """Config of uneven batched graphs: every step builds all 64 clouds' graphs."""
    import torch

    from manifoldann_gb300 import _lib, synthetic

    lib = _lib.load()
    clouds = synthetic.manifold_clouds(64, 2000, 50000, 32, seed=0)
    offs = np.zeros(65, np.int64)
    offs[1:] = np.cumsum([len(c) for c in clouds])
    N = int(offs[-1])
    pairs = float(sum(float(len(c)) ** 2 for c in clouds))
    X = torch.from_numpy(np.concatenate(clouds)).cuda()
    ids = torch.empty((N, 15), dtype=torch.int32, device="cuda")
    d = torch.empty((N, 15), dtype=torch.float32, device="cuda")
    p = _lib.params(_lib.METRIC_SQEUCLIDEAN, 15, _lib.PREC_FP32, 0, _lib.FLAG_TIME_KERNEL)
    r = _lib.KnnReport()

    def step():
        _lib.check(lib.mann_knn_graph_batched_device(p, X.data_ptr(), offs.ctypes.data, 64, 32, 0, ids.data_ptr(),
                                                     d.data_ptr(), r, stream_ptr))

    for _ in range(max(args.warmup, 2)):
        step()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(3, min(args.steps, 20))
    kernel_ms = 0.0
    e0.record(stream)
    for _ in range(reps):
        step()
        kernel_ms += r.kernel_ms
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    # the BF16 tensor-core form of the same graphs (one segmented pass, exact rerank)
    pb = _lib.params(_lib.METRIC_SQEUCLIDEAN, 15, _lib.PREC_BF16)
    rb = _lib.KnnReport()
    ids_b = torch.empty_like(ids)
    d_b = torch.empty_like(d)

    def step_bf16():
        _lib.check(lib.mann_knn_graph_batched_device(pb, X.data_ptr(), offs.ctypes.data, 64, 32, 0, ids_b.data_ptr(),
                                                     d_b.data_ptr(), rb, stream_ptr))

    for _ in range(2):
        step_bf16()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        step_bf16()
    e1.record(stream)
    torch.cuda.synchronize()
    bf16_ms = e0.elapsed_time(e1) / reps
    bf16_form = {"ms_per_step": bf16_ms, "points_per_s": N / (bf16_ms / 1e3),
                 "rows_fallback": rb.rows_fallback, "candidates_per_query": rb.candidates / N,
                 "equals_fp32_form": bool(torch.equal(ids_b, ids) and torch.equal(d_b, d))}
    # the graphs' consumer: a local PCA (intrinsic dimension 2) at every node
    offs_rows = np.repeat(offs[:-1], np.diff(offs)).astype(np.int32)
    glob = ids + torch.from_numpy(offs_rows).cuda()[:, None]
    cen = torch.arange(N, dtype=torch.int32, device="cuda")
    dims = torch.empty(N, dtype=torch.int32, device="cuda")
    eig = torch.empty((N, 2), dtype=torch.float32, device="cuda")  # slots for the 2 kept directions
    basis = torch.empty((N, 2, 32), dtype=torch.float32, device="cuda")
    pp = _lib.PcaParams(2, 0, 0.95)

    def pca():
        _lib.check(lib.mann_local_pca_device(pp, X.data_ptr(), N, 32, cen.data_ptr(), None, N, glob.data_ptr(), 15,
                                             2, dims.data_ptr(), eig.data_ptr(), basis.data_ptr(), stream_ptr))

    pca()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(3):
        pca()
    e1.record(stream)
    torch.cuda.synchronize()
    pca_ms = e0.elapsed_time(e1) / 3
    wts = torch.empty((N, 15), dtype=torch.float32, device="cuda")

    def weights():
        _lib.check(lib.mann_edge_weights_device(4, X.data_ptr(), N, 32, glob.data_ptr(), 15, dims.data_ptr(),
                                                basis.data_ptr(), 2, wts.data_ptr(), None, stream_ptr))

    weights()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(3):
        weights()
    e1.record(stream)
    torch.cuda.synchronize()
    wt_ms = e0.elapsed_time(e1) / 3
    pk = fp32_peak()
    achieved = 2.0 * 32 * pairs / (ms / 1e3) / 1e12
    cpu = None
    if args.cpu_seconds > 0:
        # the reference's build_knn_graph per cloud: a serial column loop, one
        # k+1 query per column with threads inside it (src/graphs/knn_graph.jl:63-67);
        # a sample of columns of three clouds gives the rate per (column, point) pair
        import oracle

        oracle.load()
        threads = os.cpu_count() or 1
        order = np.argsort([len(c) for c in clouds])
        picks = [order[0], order[len(order) // 2], order[-1]]
        col_pairs, t_all = 0.0, 0.0
        budget = min(6.0, args.cpu_seconds) / len(picks)
        for ci in picks:
            cl = clouds[ci]
            t0 = time.perf_counter()
            c = 0
            while time.perf_counter() - t0 < budget and c < len(cl):
                oracle.cpu_bruteforce_batch(cl, cl[c:c + 1], 16, oracle.SQEUCLIDEAN, threads)
                c += 1
            t_all += time.perf_counter() - t0
            col_pairs += c * float(len(cl))
        pair_rate = col_pairs / t_all
        cpu_step_s = pairs / pair_rate
        cpu = {"value": N / cpu_step_s, "unit": "points/s", "cores": threads, "kind": "port",
               "sample": f"columns (one k+1 query each) of the smallest, median and largest cloud for "
                         f"{t_all:.1f} s; whole-step time extrapolated by sum(n_i^2) pairs"}
    return {"workload": BATCH_WORKLOAD, "points": N, "pairs": pairs, "ms_per_step": ms,
            "graph_ms_per_step": kernel_ms / reps, "points_per_s": N / (ms / 1e3), "pairs_per_s": pairs / (ms / 1e3),
            "autotuned": {"tile_rows": r.margin_used // 100, "splits": r.margin_used % 100},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": pk["tflops"], "unit": "TFLOP/s",
                         "frac": achieved / pk["tflops"], "peak_source": "measured FP32 FMA rate (" + pk["how"] + ")",
                         "peak_sm_mhz": pk["sm_mhz"], "work": "2*d flops per ordered pair"},
            "cpu_baseline": cpu, "bf16_form": bf16_form,
            "launches_per_step": r.launches,
            "local_pca": {"ms": pca_ms, "nodes_per_s": N / (pca_ms / 1e3), "neighbours": 15, "intrinsic_dim": 2},
            "edge_weights": {"rule": "CurvatureFreeSymmetric", "ms": wt_ms, "edges_per_s": N * 15 / (wt_ms / 1e3)}}


def run_batched_profile_case(args):
    """Case for ncu: the BF16 form of the batched graphs only, on 16 manifold
    clouds (2,000-20,000 points, d = 32, k = 15; ~99k points): per call a
    segmented seed pass and a segmented main pass (k2_main), warmup + steps
    calls."""
    import torch

    from manifoldann_gb300 import _lib, synthetic

    lib = _lib.load()
    clouds = synthetic.manifold_clouds(16, 2000, 20000, 32, seed=2)
    X = torch.from_numpy(np.ascontiguousarray(np.concatenate(clouds))).cuda()
    offs = np.zeros(len(clouds) + 1, np.int64)
    offs[1:] = np.cumsum([len(c) for c in clouds])
    n = int(offs[-1])
    ids = torch.empty((n, 15), dtype=torch.int32, device="cuda")
    dd = torch.empty((n, 15), dtype=torch.float32, device="cuda")
    sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = _lib.params(_lib.METRIC_SQEUCLIDEAN, 15, _lib.PREC_BF16)
    for _ in range(args.warmup + args.steps):
        _lib.check(lib.mann_knn_graph_batched_device(p, X.data_ptr(), offs.ctypes.data, len(clouds), 32, 0,
                                                     ids.data_ptr(), dd.data_ptr(), None, sp))
    torch.cuda.synchronize()
    print(json.dumps({"case": "batched-profile", "points": n, "calls": args.warmup + args.steps,
                      "k2_main_launches": 2 * (args.warmup + args.steps)}), flush=True)
    return 0


def run_ivf_profile_case(args):
    """Case for ncu: IVF searches only (learned routing with an untrained
    network of the same shape -- same kernels and sizes -- then centroid
    routing), each at nprobe=4 on the 1M x 128 set."""
    import torch

    import manifoldann_gb300 as M
    from manifoldann_gb300 import _lib, synthetic

    lib = _lib.load()
    X = synthetic.anisotropic_clusters(IVF_N, IVF_D, seed=1)
    Q = synthetic.anisotropic_clusters(IVF_Q, IVF_D, seed=3)
    idx = M.build_index(M.IVFFlatIndex, X.T, nlist=IVF_NLIST, distance=M.SqEuclidean(), seed=1)
    model = M.ProbeModel(IVF_D, IVF_NLIST, (512, 512), use_prior=False, seed=0)
    dev = torch.device("cuda")
    Xd, Qd = torch.from_numpy(X).to(dev), torch.from_numpy(Q).to(dev)
    Cd = torch.from_numpy(np.ascontiguousarray(idx.centroids.T)).to(dev)
    od, idd = torch.from_numpy(idx.list_offsets).to(dev), torch.from_numpy(idx.list_ids).to(dev)
    oi = torch.empty((IVF_Q, K), dtype=torch.int32, device=dev)
    odist = torch.empty((IVF_Q, K), dtype=torch.float32, device=dev)
    p = _lib.params(_lib.METRIC_SQEUCLIDEAN, K, _lib.PREC_FP32)
    sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(args.warmup + args.steps):
        _lib.check(lib.mann_ivf_search_learned_device(model.handle, p, 4, Xd.data_ptr(), IVF_N, IVF_D, IVF_NLIST,
                                                      od.data_ptr(), idd.data_ptr(), Qd.data_ptr(), IVF_Q,
                                                      oi.data_ptr(), odist.data_ptr(), sp))
    for _ in range(args.warmup + args.steps):
        _lib.check(lib.mann_ivf_search_device(p, 4, _lib.METRIC_SQEUCLIDEAN, Xd.data_ptr(), IVF_N, IVF_D,
                                              Cd.data_ptr(), IVF_NLIST, od.data_ptr(), idd.data_ptr(),
                                              Qd.data_ptr(), IVF_Q, oi.data_ptr(), odist.data_ptr(), sp))
    torch.cuda.synchronize()
    print(json.dumps({"case": "ivf-profile", "searches": 2 * (args.warmup + args.steps)}), flush=True)
    return 0


ANG_WORKLOAD = ("angular-clusters-256d: N=290,000 points and Q=10,000 queries, Gaussian (sigma=0.3) around "
                "100 random unit centres then L2-normalised, CosineDist, k=20")


def run_angular_leg(args, stream_ptr=0):
    """Angular set: the cosine BF16 form (unit-normalised tensor-core pass,
    FP32-form cosine rerank), the FP16 and FP8 forms, beside the FP32 form on
    the same queries."""
    import torch

    from manifoldann_gb300 import _lib, synthetic

    lib = _lib.load()
    n, nq, d, k = 290000, 10000, 256, 20
    base = torch.from_numpy(synthetic.angular_clusters(n, d, seed=1)).cuda()
    q = torch.from_numpy(synthetic.angular_clusters(nq, d, seed=2)).cuda()
    ids = torch.empty((nq, k), dtype=torch.int32, device="cuda")
    dd = torch.empty((nq, k), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    out = {"workload": ANG_WORKLOAD}
    res = {}
    for name, prec, reps in (("bf16", _lib.PREC_BF16, max(3, min(args.steps, 10))),
                             ("fp16", _lib.PREC_FP16, max(3, min(args.steps, 10))), ("fp8", _lib.PREC_FP8, 3),
                             ("fp32", _lib.PREC_FP32, 2)):
        p = _lib.params(_lib.METRIC_COSINE, k, prec)
        r = _lib.KnnReport()

        def call():
            _lib.check(lib.mann_knn_device(p, base.data_ptr(), n, q.data_ptr(), nq, d, ids.data_ptr(),
                                           dd.data_ptr(), r, stream_ptr))

        for _ in range(2):
            call()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            call()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        res[name] = (ids.cpu().numpy().copy(), dd.cpu().numpy().copy())
        out[name] = {"ms": ms, "qps": nq / (ms / 1e3), "rows_fallback": r.rows_fallback,
                     "candidates_per_query": r.candidates / nq if prec != _lib.PREC_FP32 else None}
    out["bf16_over_fp32"] = out["bf16"]["qps"] / out["fp32"]["qps"]
    out["bf16_equals_fp32_form"] = bool(np.array_equal(res["bf16"][0], res["fp32"][0]) and
                                        np.array_equal(res["bf16"][1].view(np.uint32), res["fp32"][1].view(np.uint32)))
    out["fp8_equals_fp32_form"] = bool(np.array_equal(res["fp8"][0], res["fp32"][0]) and
                                       np.array_equal(res["fp8"][1].view(np.uint32), res["fp32"][1].view(np.uint32)))
    out["fp16_over_fp32"] = out["fp16"]["qps"] / out["fp32"]["qps"]
    out["fp16_equals_fp32_form"] = bool(np.array_equal(res["fp16"][0], res["fp32"][0]) and
                                        np.array_equal(res["fp16"][1].view(np.uint32), res["fp32"][1].view(np.uint32)))
    peak_tf, _, _, src = measured_peaks()
    flops = 2.0 * d * n * nq
    ach = flops / (out["bf16"]["ms"] / 1e3) / 1e12
    out["roofline_bf16"] = {"bound": "tensor", "achieved": ach, "peak": peak_tf, "unit": "TFLOP/s",
                            "frac": ach / peak_tf, "peak_source": f"{src} bf16 dense (burst)",
                            "work": "2*d flops per (query, point) pair", "note": "whole call (normalise, passes, rerank)"}
    ach16 = flops / (out["fp16"]["ms"] / 1e3) / 1e12
    out["roofline_fp16"] = {"bound": "tensor", "achieved": ach16, "peak": peak_tf, "unit": "TFLOP/s",
                            "frac": ach16 / peak_tf, "peak_source": f"{src} bf16 dense (burst; FP16 runs at the same rate)",
                            "work": "2*d flops per (query, point) pair", "note": "whole call (normalise, passes, rerank)"}
    if args.cpu_seconds > 0:
        import oracle

        oracle.load()
        threads = os.cpu_count() or 1
        bh, qh = base.cpu().numpy(), q.cpu().numpy()
        m = 64
        t0 = time.perf_counter()
        oracle.cpu_bruteforce_batch(bh, qh[:m], k, oracle.COSINE, threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": m / dt, "unit": "queries/s", "cores": threads, "kind": "port",
                               "sample": f"{m} queries against all {n} points, CosineDist, k={k}, {dt:.1f} s"}
    return out


PLAIN_WORKLOAD = ("iid-normal-64d: N=10,000 points and Q=1,000 queries, float32 N(0,1) from two seeds, "
                  "SqEuclidean, k=10, ties to the lower index (the plain FP32 form)")


def run_plain_leg(args, stream_ptr=0):
    """The plain exact kNN (the FP32 form): 10,000 x 64 points, 1,000 queries,
    k = 10.  The 2.8 MB of inputs fit in L2, so a 256 MB buffer is written
    between timed calls and only the calls are timed (CUDA events around each
    call on the launching stream).  The answer is checked against the FP32
    oracle (ids and distance bits)."""
    import torch

    import oracle
    from manifoldann_gb300 import _lib, synthetic

    lib = _lib.load()
    n, nq, d, k = 10000, 1000, 64, 10
    base = synthetic.iid_normal(n, d, seed=1)
    q = synthetic.iid_normal(nq, d, seed=2)
    tb, tq = torch.from_numpy(base).cuda(), torch.from_numpy(q).cuda()
    ids = torch.empty((nq, k), dtype=torch.int32, device="cuda")
    dd = torch.empty((nq, k), dtype=torch.float32, device="cuda")
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    p = _lib.params(_lib.METRIC_SQEUCLIDEAN, k, _lib.PREC_FP32)

    def call():
        _lib.check(lib.mann_knn_device(p, tb.data_ptr(), n, tq.data_ptr(), nq, d, ids.data_ptr(), dd.data_ptr(),
                                       None, stream_ptr))

    for _ in range(max(3, args.warmup)):
        call()
    torch.cuda.synchronize()
    reps = 50
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for e0, e1 in evs:
        flush.fill_(1.0)
        e0.record(stream)
        call()
        e1.record(stream)
    torch.cuda.synchronize()
    times = sorted(e0.elapsed_time(e1) for e0, e1 in evs)
    ms = float(np.median(times))
    oracle.load()
    ids_o, d_o = oracle.knn_f32(base, q, k, oracle.SQEUCLIDEAN)
    same = bool(np.array_equal(ids.cpu().numpy(), ids_o) and
                np.array_equal(dd.cpu().numpy().view(np.uint32), d_o.view(np.uint32)))
    pk = fp32_peak()
    flops = 2.0 * d * n * nq
    ach = flops / (ms / 1e3) / 1e12
    # e2e through the host-pointer C ABI (pinned inputs copied by every call)
    hb, hq = torch.from_numpy(base).pin_memory(), torch.from_numpy(q).pin_memory()
    hi = torch.empty((nq, k), dtype=torch.int32).pin_memory()
    hd = torch.empty((nq, k), dtype=torch.float32).pin_memory()

    def host():
        _lib.check(lib.mann_knn(p, hb.data_ptr(), n, hq.data_ptr(), nq, d, hi.data_ptr(), hd.data_ptr(), None))

    for _ in range(3):
        host()
    t0 = time.perf_counter()
    for _ in range(reps):
        host()
    e2e_s = (time.perf_counter() - t0) / reps
    cpu = None
    if args.cpu_seconds > 0:
        threads = os.cpu_count() or 1
        oracle.cpu_bruteforce_batch(base, q, k, oracle.SQEUCLIDEAN, threads)
        t0 = time.perf_counter()
        r = 0
        while time.perf_counter() - t0 < min(2.0, args.cpu_seconds):
            oracle.cpu_bruteforce_batch(base, q, k, oracle.SQEUCLIDEAN, threads)
            r += 1
        dt = time.perf_counter() - t0
        cpu = {"value": r * nq / dt, "unit": "queries/s", "cores": threads, "kind": "port",
               "sample": f"{r} x all {nq} queries, {dt:.1f} s"}
    return {"workload": PLAIN_WORKLOAD, "ms": ms, "ms_min": times[0], "qps": nq / (ms / 1e3),
            "l2": "256 MB buffer written between timed calls (inputs fit in L2)",
            "equals_fp32_oracle": same,
            "roofline": {"bound": "fp32", "kernel": "k1_tile_topk + merge (whole call)", "achieved": ach,
                         "peak": pk["tflops"], "unit": "TFLOP/s", "frac": ach / pk["tflops"],
                         "peak_source": "measured FP32 FMA rate (" + pk["how"] + ")", "peak_sm_mhz": pk["sm_mhz"],
                         "work": "2*d flops per (query, point) pair"},
            "e2e": {"value": nq / e2e_s, "unit": "queries/s", "h2d_bytes_per_step": int(base.nbytes + q.nbytes),
                    "d2h_bytes_per_step": int(nq * k * 8), "api": "mann_knn"},
            "cpu_baseline": cpu}


def fp64_oracle_check(base, q, qi, gi, nrows=1000, seed=5):
    """Sampled rows of the step's answers against the FP64 oracle (every host
    core, outside the timed region): held-out query rows with oracle.knn_f64,
    self-graph rows with oracle.knn_graph_rows(fp64=True)."""
    import oracle

    oracle.load()
    rng = np.random.default_rng(seed)
    qr = np.sort(rng.choice(N_QUERIES, nrows, replace=False)).astype(np.int32)
    gr = np.sort(rng.choice(N_POINTS, nrows, replace=False)).astype(np.int32)
    t0 = time.perf_counter()
    qo, _ = oracle.knn_f64(base, q[qr], K, oracle.SQEUCLIDEAN)
    go, _ = oracle.knn_graph_rows(base, gr, K, oracle.SQEUCLIDEAN, fp64=True)
    dt = time.perf_counter() - t0

    def recall(a, b):
        return float(sum(len(set(a[i]) & set(b[i])) for i in range(len(a))) / (K * len(a)))

    return {"recall_at_10_vs_fp64_oracle": min(recall(qi[qr], qo), recall(gi[gr], go)),
            "queries": {"rows": nrows, "recall_at_10": recall(qi[qr], qo),
                        "ids_identical_rows": int((qi[qr] == qo).all(axis=1).sum())},
            "graph": {"rows": nrows, "recall_at_10": recall(gi[gr], go),
                      "ids_identical_rows": int((gi[gr] == go).all(axis=1).sum())},
            "oracle_s": dt, "sample_seed": seed}


def run_ours(args):
    import torch

    import manifoldann_gb300 as M
    from manifoldann_gb300 import _lib

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    lib = _lib.load()
    base, q = make_workload()
    tb = torch.from_numpy(base).cuda()
    tq = torch.from_numpy(q).cuda()
    qi = torch.empty((N_QUERIES, K), dtype=torch.int32, device="cuda")
    qd = torch.empty((N_QUERIES, K), dtype=torch.float32, device="cuda")
    gi = torch.empty((N_POINTS, K), dtype=torch.int32, device="cuda")
    gd = torch.empty((N_POINTS, K), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)

    def step(prec, flags=0):
        p = _lib.params(_lib.METRIC_SQEUCLIDEAN, K, prec, 0, flags)
        r1, r2 = _lib.KnnReport(), _lib.KnnReport()
        _lib.check(lib.mann_knn_device(p, tb.data_ptr(), N_POINTS, tq.data_ptr(), N_QUERIES, DIM,
                                       qi.data_ptr(), qd.data_ptr(), r1, sp))
        _lib.check(lib.mann_knn_graph_device(p, tb.data_ptr(), N_POINTS, DIM, 0, gi.data_ptr(),
                                             gd.data_ptr(), r2, sp))
        return r1, r2

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- headline: BF16 form with FP64 near-tie order, inputs resident
    HEAD = _lib.FLAG_FP64_TIES
    for _ in range(args.warmup):
        step(_lib.PREC_BF16, HEAD)
    barrier()
    sampler = ClockSampler(local)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kernel_ms, launches, fallback, cands, ties, widened, unresolved = 0.0, 0, 0, 0, 0, 0, 0
    ev0.record(stream)
    for _ in range(args.steps):
        r1, r2 = step(_lib.PREC_BF16, HEAD | _lib.FLAG_TIME_KERNEL)
        kernel_ms += r1.kernel_ms + r2.kernel_ms
        launches += r1.launches + r2.launches
        fallback += r1.rows_fallback + r2.rows_fallback
        cands += r1.candidates + r2.candidates
        ties += r1.rows_fp64_ties + r2.rows_fp64_ties
        widened += r1.rows_ties_widened + r2.rows_ties_widened
        unresolved += r1.rows_unresolved + r2.rows_unresolved
    ev1.record(stream)
    barrier()
    clocks = sampler.stop()
    ms = ev0.elapsed_time(ev1)
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    qps_step = N_QUERIES + N_POINTS
    value = ws * qps_step * args.steps / (ms / 1e3)
    bf16_i = (qi.cpu().numpy().copy(), gi.cpu().numpy().copy())
    # the same step once more with the FP64 error report (untimed)
    e1r, e2r = step(_lib.PREC_BF16, HEAD | _lib.FLAG_FP64_ERR)
    same_again = bool(np.array_equal(bf16_i[0], qi.cpu().numpy()) and np.array_equal(bf16_i[1], gi.cpu().numpy()))

    # ---- the FP8 (e4m3) form on the held-out query batch (its certified window
    # is wide, so most rows fall back to the exact FP32 scan)
    fp8 = None
    if not args.no_fp8:
        pf = _lib.params(_lib.METRIC_SQEUCLIDEAN, K, _lib.PREC_FP8)
        rf = _lib.KnnReport()
        for _ in range(2):
            _lib.check(lib.mann_knn_device(pf, tb.data_ptr(), N_POINTS, tq.data_ptr(), N_QUERIES, DIM,
                                           qi.data_ptr(), qd.data_ptr(), rf, sp))
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(2):
            _lib.check(lib.mann_knn_device(pf, tb.data_ptr(), N_POINTS, tq.data_ptr(), N_QUERIES, DIM,
                                           qi.data_ptr(), qd.data_ptr(), rf, sp))
        e1.record(stream)
        barrier()
        fms = e0.elapsed_time(e1) / 2
        fp8 = {"workload": "the 10,000 held-out queries against the 60,000 points", "ms": fms,
               "qps": N_QUERIES / (fms / 1e3), "rows_fallback": rf.rows_fallback,
               "candidates_per_query": rf.candidates / N_QUERIES,
               "ids_equal_bf16_form": bool(np.array_equal(qi.cpu().numpy(), bf16_i[0]))}

    # ---- the plain FP32 form on the same step
    step(_lib.PREC_FP32)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.fp32_steps):
        step(_lib.PREC_FP32)
    e1.record(stream)
    barrier()
    fp32_ms = e0.elapsed_time(e1) / max(args.fp32_steps, 1)
    fp32_qps = qps_step / (fp32_ms / 1e3)
    fp32_i = (qi.cpu().numpy().copy(), gi.cpu().numpy().copy())

    # ---- e2e through the host-pointer C ABI (pinned host buffers): the
    # points uploaded once per step into a dataset handle that both calls
    # search (the headline e2e), and the plain host-pointer calls that copy
    # the points on each call
    e2e = None
    if not args.no_e2e:
        hb = torch.from_numpy(base).pin_memory()
        hq = torch.from_numpy(q).pin_memory()
        hqi = torch.empty((N_QUERIES, K), dtype=torch.int32).pin_memory()
        hqd = torch.empty((N_QUERIES, K), dtype=torch.float32).pin_memory()
        hgi = torch.empty((N_POINTS, K), dtype=torch.int32).pin_memory()
        hgd = torch.empty((N_POINTS, K), dtype=torch.float32).pin_memory()
        p = _lib.params(_lib.METRIC_SQEUCLIDEAN, K, _lib.PREC_BF16, 0, HEAD)

        def host_step():
            _lib.check(lib.mann_knn(p, hb.data_ptr(), N_POINTS, hq.data_ptr(), N_QUERIES, DIM,
                                    hqi.data_ptr(), hqd.data_ptr(), None))
            _lib.check(lib.mann_knn_graph(p, hb.data_ptr(), N_POINTS, DIM, 0, hgi.data_ptr(),
                                          hgd.data_ptr(), None))

        dsh = C.c_void_p()
        _lib.check(lib.mann_dataset_create(hb.data_ptr(), N_POINTS, DIM, C.byref(dsh)))

        def dataset_step():
            _lib.check(lib.mann_dataset_upload(dsh, hb.data_ptr(), N_POINTS))
            _lib.check(lib.mann_knn_dataset(p, dsh, hq.data_ptr(), N_QUERIES, hqi.data_ptr(), hqd.data_ptr(),
                                            None))
            _lib.check(lib.mann_knn_graph_dataset(p, dsh, 0, hgi.data_ptr(), hgd.data_ptr(), None))

        def timed(fn):
            for _ in range(max(1, args.warmup)):
                fn()
            barrier()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                fn()
            dt = time.perf_counter() - t0
            if dist is not None:
                t = torch.tensor([dt], device="cuda")
                dist.all_reduce(t, op=dist.ReduceOp.MAX)
                dt = float(t.item())
            return ws * qps_step * args.steps / dt

        d2h = int((N_QUERIES + N_POINTS) * K * 8)
        e2e = {"value": timed(dataset_step), "unit": "queries/s",
               "h2d_bytes_per_step": int(base.nbytes + q.nbytes), "d2h_bytes_per_step": d2h,
               "api": "mann_dataset_upload + mann_knn_dataset + mann_knn_graph_dataset (MANN_FLAG_FP64_TIES)"}
        e2e_ids_equal = bool(np.array_equal(hqi.numpy(), bf16_i[0]) and np.array_equal(hgi.numpy(), bf16_i[1]))
        e2e["host_pointer_calls"] = {"value": timed(host_step), "unit": "queries/s",
                                     "h2d_bytes_per_step": int(2 * base.nbytes + q.nbytes),
                                     "d2h_bytes_per_step": d2h, "api": "mann_knn + mann_knn_graph"}
        e2e["ids_equal_device_run"] = e2e_ids_equal
        lib.mann_dataset_destroy(dsh)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0

    peak_tf, peak_sus, hbm, peak_src = measured_peaks()
    traffic = profiled_traffic()
    flops_step = 2.0 * DIM * N_POINTS * (N_QUERIES + N_POINTS)
    launches_per_step_main = 2
    achieved_tf = flops_step * args.steps / (kernel_ms / 1e3) / 1e12 if kernel_ms > 0 else None
    roof = {"bound": "tensor", "achieved": achieved_tf, "peak": peak_tf, "unit": "TFLOP/s",
            "frac": (achieved_tf / peak_tf) if achieved_tf else None, "traffic": traffic,
            "peak_source": f"{peak_src} bf16 dense, burst (the timed region lasts well under a second); "
                           f"sustained {peak_sus}",
            "kernel": "k2_main (tcgen05 BF16 tiles + fused top-(k+m))",
            "kernel_ms_per_launch": kernel_ms / (args.steps * launches_per_step_main),
            "work": "2*d flops per (query, point) pair: 2*784*60000*(10000+60000) = 6.585 TFLOP per step"}
    t0 = time.perf_counter()
    oracle_check = fp64_oracle_check(base, q, bf16_i[0], bf16_i[1])
    oracle_check["max_abs_err_fp64"] = {"queries": e1r.max_abs_err_fp64, "graph": e2r.max_abs_err_fp64}
    oracle_check["fp32_form_recall_at_10_vs_fp64"] = fp64_oracle_check(base, q, fp32_i[0], fp32_i[1])[
        "recall_at_10_vs_fp64_oracle"]
    cpu = cpu_baseline(base, q, args.cpu_seconds) if args.cpu_seconds > 0 else None
    plain = None if args.no_plain else run_plain_leg(args, sp)
    ivf = None if args.no_ivf else run_ivf_leg(args, sp)
    batched = None if args.no_batched else run_batched_leg(args, sp)
    angular = None if args.no_angular else run_angular_leg(args, sp)
    line = {"metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": CONFIG, "parallelism": "replicas" if ws > 1 else "single GPU",
            "fp32_form": {"value": fp32_qps, "unit": "queries/s", "ms_per_step": fp32_ms,
                          "bf16_over_fp32": value / ws / fp32_qps},
            "recall_at_10_vs_fp64_oracle": oracle_check["recall_at_10_vs_fp64_oracle"],
            "max_abs_err_fp64": max(e1r.max_abs_err_fp64, e2r.max_abs_err_fp64),
            "fp64_oracle_check": oracle_check,
            "repeat_run_ids_equal": same_again,
            "rows_fallback_per_step": fallback / args.steps,
            "rows_fp64_ties_per_step": ties / args.steps,
            "rows_ties_widened_per_step": widened / args.steps,
            "rows_unresolved_total": unresolved,
            "candidates_per_query": cands / (args.steps * qps_step),
            "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clocks,
            "fp8_form": fp8, "gpu_launches": launches, "plain_fp32": plain, "ivf_learned_probe": ivf, "batched_graphs": batched,
            "angular_cosine": angular, "fp32_peak": fp32_peak() if (plain or batched) else None,
            "post_timing_s": time.perf_counter() - t0}
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.case == "profile":
        return run_profile_case(args)
    if args.case == "ivf-profile":
        return run_ivf_profile_case(args)
    if args.case == "angular":
        import torch

        print(json.dumps({"case": "angular", "angular_cosine": run_angular_leg(
            args, C.c_void_p(torch.cuda.current_stream().cuda_stream))}), flush=True)
        return 0
    if args.case == "angular-profile":
        return run_angular_profile_case(args)
    if args.case == "plain":
        import torch

        print(json.dumps({"case": "plain", "plain_fp32": run_plain_leg(
            args, C.c_void_p(torch.cuda.current_stream().cuda_stream))}), flush=True)
        return 0
    if args.case == "batched-profile":
        return run_batched_profile_case(args)
    if args.case == "batched":
        import torch

        print(json.dumps({"case": "batched", "batched_graphs": run_batched_leg(
            args, C.c_void_p(torch.cuda.current_stream().cuda_stream))}), flush=True)
        return 0
    if args.case == "ivf":
        import torch

        print(json.dumps({"case": "ivf", "ivf_learned_probe": run_ivf_leg(
            args, C.c_void_p(torch.cuda.current_stream().cuda_stream))}), flush=True)
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

#!/usr/bin/env python
"""Benchmark of the exact-kNN hot path on one GB300.

Workload (one step): the 784-d quantised Gaussian-mixture set -- N=60,000
points, Q=10,000 held-out queries, SqEuclidean, k=10 -- searched for the
held-out queries AND materialised as the self kNN graph of the 60,000 points
(build_knn_graph semantics).  A step therefore answers 70,000 queries.

Arms
  (default)          the BF16 tensor-core form with certified candidates and
                     exact FP32 rerank (recall@10 = 1.0 by construction); the
                     plain FP32 form is timed beside it.  `value` has the inputs
                     resident in HBM; `e2e` goes through the host-pointer C ABI
                     (pinned host buffers, copies inside the timed region).
  --impl reference   the reference's BruteForceIndex algorithm restated in C
                     (OpenMP over every host core), on a bounded sample of the
                     same workload per step.

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
    ap.add_argument("--case", choices=["full", "profile", "ivf", "batched", "ivf-profile", "angular"],
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


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        j = json.loads(p.read_text())
        return j.get("bf16_tflops_sustained", 1737.1), j.get("hbm_gbs", 6703.5), "measured"
    return 1700.0, 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per k2_main main-pass launch from the committed ncu summary."""
    p = ROOT / "profiles" / "k2_main_bf16_knn_60k_784.md"
    if p.exists():
        for line in p.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1].split()[0])
    return None


def cpu_baseline(base, q, budget_s):
    """The reference algorithm (oracle's OpenMP restatement) on a bounded query sample."""
    import oracle

    threads = os.cpu_count() or 1
    oracle.load()
    probe = 32
    t0 = time.perf_counter()
    oracle.cpu_bruteforce_batch(base, q[:probe], K, oracle.SQEUCLIDEAN, threads)
    dt = max(time.perf_counter() - t0, 1e-3)
    m = int(min(len(q), max(probe, probe * budget_s / dt)))
    t0 = time.perf_counter()
    oracle.cpu_bruteforce_batch(base, q[:m], K, oracle.SQEUCLIDEAN, threads)
    dt = time.perf_counter() - t0
    return {"value": m / dt, "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"{m} held-out queries against all {N_POINTS} points (d={DIM}, k={K}), "
                      f"{dt:.1f} s wall on {threads} host threads"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    base, q = make_workload()
    import oracle

    oracle.load()
    threads = os.cpu_count() or 1
    per_step = 64
    for i in range(args.warmup):
        oracle.cpu_bruteforce_batch(base, q[i * per_step % N_QUERIES:][:per_step], K, oracle.SQEUCLIDEAN, threads)
    t0 = time.perf_counter()
    for i in range(args.steps):
        s = (i * per_step) % (N_QUERIES - per_step)
        oracle.cpu_bruteforce_batch(base, q[s:s + per_step], K, oracle.SQEUCLIDEAN, threads)
    dt = time.perf_counter() - t0
    qps = per_step * args.steps / dt
    line = {"metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "step": f"{per_step} held-out queries against all points",
                       "parallelism": "host threads"},
            "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
                             "sample": f"{per_step} queries per step x {args.steps} steps; reference "
                                       "BruteForceIndex algorithm restated in C (Julia is not installed)"},
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
    p = _lib.params(_lib.METRIC_SQEUCLIDEAN, K, _lib.PREC_BF16)
    for _ in range(args.warmup + args.steps):
        _lib.check(lib.mann_knn_device(p, tb.data_ptr(), N_POINTS, tq.data_ptr(), N_QUERIES, DIM,
                                       qi.data_ptr(), qd.data_ptr(), None, sp))
        _lib.check(lib.mann_knn_graph_device(p, tb.data_ptr(), N_POINTS, DIM, 0, gi.data_ptr(),
                                             gd.data_ptr(), None, sp))
    torch.cuda.synchronize()
    print(json.dumps({"case": "profile", "steps": args.warmup + args.steps,
                      "k2_main_launches": 2 * (args.warmup + args.steps)}), flush=True)
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
    for name, prec in (("fp32", _lib.PREC_FP32), ("bf16", _lib.PREC_BF16)):
        pp = _lib.params(_lib.METRIC_SQEUCLIDEAN, K, prec)
        ms = timed(lambda: _lib.check(lib.mann_knn_device(pp, Xd.data_ptr(), IVF_N, Qd.data_ptr(), IVF_Q, IVF_D,
                                                          oi.data_ptr(), odist.data_ptr(), None, stream_ptr)),
                   2 if prec == _lib.PREC_FP32 else 5)
        exact[name] = {"ms": ms, "qps": IVF_Q / (ms / 1e3)}
    truth = oi.cpu().numpy().copy()  # the BF16 form's certified exact top-10
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
    best_exact = max(exact["fp32"]["qps"], exact["bf16"]["qps"])
    res = {"workload": IVF_WORKLOAD, "build_s": build_s, "label_s": label_s, "train_s": train_s,
           "train_epochs": args.ivf_epochs, "final_loss": float(loss[-1]), "exact": exact,
           "learned": out["learned"], "centroid_routing": out["centroid"], "e2e_learned": e2e}
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
    fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
    achieved = 2.0 * 32 * pairs / (ms / 1e3) / 1e12
    return {"workload": BATCH_WORKLOAD, "points": N, "pairs": pairs, "ms_per_step": ms,
            "graph_ms_per_step": kernel_ms / reps, "points_per_s": N / (ms / 1e3), "pairs_per_s": pairs / (ms / 1e3),
            "autotuned": {"tile_rows": r.margin_used // 100, "splits": r.margin_used % 100},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp32_peak, "peak_source": "nominal FP32 FMA rate (152 SMs x 128 lanes x 2.07 GHz)",
                         "work": "2*d flops per ordered pair"},
            "launches_per_step": r.launches,
            "local_pca": {"ms": pca_ms, "nodes_per_s": N / (pca_ms / 1e3), "neighbours": 15, "intrinsic_dim": 2},
            "edge_weights": {"rule": "CurvatureFreeSymmetric", "ms": wt_ms, "edges_per_s": N * 15 / (wt_ms / 1e3)}}


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
    FP32-form cosine rerank) beside the FP32 form on the same queries."""
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
    for name, prec, reps in (("bf16", _lib.PREC_BF16, max(3, min(args.steps, 10))), ("fp32", _lib.PREC_FP32, 2)):
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
                     "candidates_per_query": r.candidates / nq if prec == _lib.PREC_BF16 else None}
    out["bf16_over_fp32"] = out["bf16"]["qps"] / out["fp32"]["qps"]
    out["bf16_equals_fp32_form"] = bool(np.array_equal(res["bf16"][0], res["fp32"][0]) and
                                        np.array_equal(res["bf16"][1].view(np.uint32), res["fp32"][1].view(np.uint32)))
    peak_tf, _, _ = measured_peaks()
    flops = 2.0 * d * n * nq
    out["roofline_bf16"] = {"bound": "tensor", "achieved": flops / (out["bf16"]["ms"] / 1e3) / 1e12,
                            "peak": peak_tf, "unit": "TFLOP/s", "note": "whole call (normalise, passes, rerank)"}
    return out


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

    # ---- headline: BF16 form, inputs resident
    for _ in range(args.warmup):
        step(_lib.PREC_BF16)
    barrier()
    sampler = ClockSampler(local)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kernel_ms, launches, fallback, cands = 0.0, 0, 0, 0
    ev0.record(stream)
    for _ in range(args.steps):
        r1, r2 = step(_lib.PREC_BF16, _lib.FLAG_TIME_KERNEL)
        kernel_ms += r1.kernel_ms + r2.kernel_ms
        launches += r1.launches + r2.launches
        fallback += r1.rows_fallback + r2.rows_fallback
        cands += r1.candidates + r2.candidates
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
    same_as_fp32 = bool(np.array_equal(bf16_i[0], qi.cpu().numpy()) and np.array_equal(bf16_i[1], gi.cpu().numpy()))

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
        p = _lib.params(_lib.METRIC_SQEUCLIDEAN, K, _lib.PREC_BF16)

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
               "api": "mann_dataset_upload + mann_knn_dataset + mann_knn_graph_dataset"}
        e2e["host_pointer_calls"] = {"value": timed(host_step), "unit": "queries/s",
                                     "h2d_bytes_per_step": int(2 * base.nbytes + q.nbytes),
                                     "d2h_bytes_per_step": d2h, "api": "mann_knn + mann_knn_graph"}
        lib.mann_dataset_destroy(dsh)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0

    peak_tf, hbm, peak_src = measured_peaks()
    traffic = profiled_traffic()
    flops_step = 2.0 * DIM * N_POINTS * (N_QUERIES + N_POINTS)
    launches_per_step_main = 2
    achieved_tf = flops_step * args.steps / (kernel_ms / 1e3) / 1e12 if kernel_ms > 0 else None
    roof = {"bound": "tensor", "achieved": achieved_tf, "peak": peak_tf, "unit": "TFLOP/s",
            "frac": (achieved_tf / peak_tf) if achieved_tf else None, "traffic": traffic,
            "peak_source": f"{peak_src} bf16 dense (sustained)", "kernel": "k2_main (tcgen05 BF16 tiles + fused top-(k+m))",
            "kernel_ms_per_launch": kernel_ms / (args.steps * launches_per_step_main)}
    cpu = cpu_baseline(base, q, args.cpu_seconds) if args.cpu_seconds > 0 else None
    ivf = None if args.no_ivf else run_ivf_leg(args, sp)
    batched = None if args.no_batched else run_batched_leg(args, sp)
    angular = None if args.no_angular else run_angular_leg(args, sp)
    line = {"metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": WORKLOAD, "queries_per_step": qps_step, "l2": "inputs larger than L2 (188 MB fp32 points)",
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "fp32_form": {"value": fp32_qps, "unit": "queries/s", "ms_per_step": fp32_ms,
                          "bf16_over_fp32": value / ws / fp32_qps},
            "recall_at_10_vs_fp32_form": 1.0 if same_as_fp32 else 0.0,
            "rows_fallback_per_step": fallback / args.steps,
            "candidates_per_query": cands / (args.steps * qps_step),
            "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clocks,
            "gpu_launches": launches, "ivf_learned_probe": ivf, "batched_graphs": batched,
            "angular_cosine": angular}
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

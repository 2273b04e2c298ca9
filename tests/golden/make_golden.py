"""Generates the small golden fixtures under tests/golden/ from the CPU oracle.

The reference (Julia) cannot run here, so the fixtures pin the oracle's
restatement; the oracle itself is pinned by the reference's known-answer tests
(tests/test_oracle.py) and by an exact-arithmetic Python restatement of its
summation on small cases.  Each .npz holds the inputs (row-major [n][d]
float32) and the expected outputs (0-based int32 ids, float32 / float64
distances).

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from manifoldann_gb300 import synthetic  # noqa: E402


def knn_case(name, base, queries, k, metric):
    i32, d32 = oracle.knn_f32(base, queries, k, metric)
    i64, d64 = oracle.knn_f64(base, queries, k, metric)
    np.savez_compressed(HERE / f"{name}.npz", base=base, queries=queries, k=k, metric=metric,
                        ids_f32=i32, dists_f32=d32, ids_f64=i64, dists_f64=d64)


def graph_case(name, data, k, metric, include_self):
    i32, d32 = oracle.knn_graph_f32(data, k, metric, include_self)
    i64, d64 = oracle.knn_graph_f64(data, k, metric, include_self)
    np.savez_compressed(HERE / f"{name}.npz", data=data, k=k, metric=metric,
                        include_self=int(include_self), ids_f32=i32, dists_f32=d32, ids_f64=i64,
                        dists_f64=d64)


def main():
    # plain exact kNN, the shape family of the N=10k/Q=1k/d=64 workload, reduced
    base = synthetic.iid_normal(2000, 64, seed=11)
    q = synthetic.iid_normal(100, 64, seed=12)
    knn_case("knn_iid_sq_d64", base, q, 10, oracle.SQEUCLIDEAN)
    knn_case("knn_iid_euclid_d64", base, q, 10, oracle.EUCLIDEAN)
    # odd dimension (non-vector loads), cosine
    base = synthetic.iid_normal(1500, 37, seed=13)
    q = synthetic.iid_normal(64, 37, seed=14)
    knn_case("knn_iid_cos_d37", base, q, 20, oracle.COSINE)
    # quantised 784-d mixture (exact ties are common), reduced
    base = synthetic.quantized_mixture(1500, 784, seed=21)
    q = synthetic.quantized_mixture(50, 784, seed=22)
    knn_case("knn_mix_sq_d784", base, q, 10, oracle.SQEUCLIDEAN)
    graph_case("graph_mix_sq_d784", base[:800], 10, oracle.SQEUCLIDEAN, False)
    # angular blobs, reduced
    base = synthetic.angular_clusters(1500, 256, seed=31)
    q = synthetic.angular_clusters(50, 256, seed=32)
    knn_case("knn_ang_cos_d256", base, q, 20, oracle.COSINE)
    # one small manifold cloud, self graph k=15
    cloud = synthetic.manifold_clouds(count=1, lo=900, hi=900, seed=41)[0]
    graph_case("graph_cloud_sq_d32", cloud, 15, oracle.SQEUCLIDEAN, False)
    graph_case("graph_cloud_sq_d32_self", cloud, 15, oracle.SQEUCLIDEAN, True)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()

"""manifoldann_gb300 -- GB300 (sm_103a) implementation of ManifoldANN's exact
kNN / kNN-graph / KMeans-assignment hot path.

The compute lives in ``libmanngpu.so`` (C ABI: ``include/mann.h``); this
package mirrors the reference's Julia API on top of it (names follow
src/ManifoldANN.jl's exports; Julia's ``insert!``/``fit!`` are ``insert``/``fit``).
"""
from ._lib import ArgumentError, DimensionMismatch, MannError
from .distances import (CosineDist, Euclidean, SqEuclidean, cosine_distance, default_distance,
                        default_squared_distance, euclidean_distance)
from .eval_utils import recall_at_k
from .graphs import (KNNGraph, build_knn_graph, build_knn_graphs, graph_metadata, has_metadata,
                     knn_graph_arrays, knn_graph_batched_arrays, knn_graph_symmetrize_csr, node_metadata)
from .transforms import (KMeansAssignment, KMeansTransform, TransformResult, assign_arrays,
                         assign_clusters, fit, get_bucket_assignment, init_kmeans_plus_plus, lloyd,
                         pairwise_distances, take_pending_assignments, transform)
from .geometry import (CurvatureFreeSymmetric, EuclideanChord, PCAGeometry, PCAMethod,
                       TangentProjectedSourceOnly, TangentProjectedSymmetricMax,
                       TangentProjectedSymmetricMean, WeightedKNNGraph, build_weighted_graph,
                       candidate_neighbors, compute_edge_weights, fit_geometries, fit_geometry,
                       intrinsic_dimension, local_distance, project, reconstruct)
from .multilevel import (DisjointMerge, MultiLevelIndex, SimpleMerge, TerminalConfig, TransformedConfig,
                         TransformedIndex, build_multilevel_index, merge_results, multilevel_query)
from .ivf import IVFFlatIndex, TopKRouting, ivf_search_device, select_indices
from .probe import LearnedProbeRouting, ProbeModel, ivf_search_learned, neighbour_list_labels
from .indices import (AbstractANNIndex, BruteForceIndex, DeviceDataset, Neighbor, build_index, configured_k,
                      index_distance, insert, knn_arrays, neighbor_ids, query, supports_mutation)

__all__ = [
    "ArgumentError", "DimensionMismatch", "MannError", "DeviceDataset",
    "CosineDist", "Euclidean", "SqEuclidean", "cosine_distance", "default_distance",
    "default_squared_distance", "euclidean_distance",
    "recall_at_k",
    "KNNGraph", "build_knn_graph", "build_knn_graphs", "graph_metadata", "has_metadata", "knn_graph_arrays",
    "knn_graph_batched_arrays", "knn_graph_symmetrize_csr", "node_metadata",
    "AbstractANNIndex", "BruteForceIndex", "Neighbor", "build_index", "configured_k",
    "index_distance", "insert", "knn_arrays", "neighbor_ids", "query", "supports_mutation",
    "KMeansAssignment", "KMeansTransform", "TransformResult", "assign_arrays", "assign_clusters", "fit",
    "get_bucket_assignment", "init_kmeans_plus_plus", "lloyd", "pairwise_distances",
    "take_pending_assignments", "transform",
    "IVFFlatIndex", "TopKRouting", "ivf_search_device", "select_indices",
    "LearnedProbeRouting", "ProbeModel", "ivf_search_learned", "neighbour_list_labels",
    "PCAGeometry", "PCAMethod", "fit_geometries", "fit_geometry", "intrinsic_dimension", "local_distance",
    "project", "reconstruct", "CurvatureFreeSymmetric", "EuclideanChord", "TangentProjectedSourceOnly",
    "TangentProjectedSymmetricMax", "TangentProjectedSymmetricMean", "compute_edge_weights",
    "WeightedKNNGraph", "build_weighted_graph", "candidate_neighbors",
    "DisjointMerge", "MultiLevelIndex", "SimpleMerge", "TerminalConfig", "TransformedConfig", "TransformedIndex",
    "build_multilevel_index", "merge_results", "multilevel_query",
]

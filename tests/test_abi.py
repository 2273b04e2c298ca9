"""The C-ABI library loads, exports every symbol include/mann.h declares, and
rejects bad arguments before touching a GPU (no compute calls here)."""
import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    txt = "\n".join(p.read_text() for p in sorted((ROOT / "include").glob("*.h")))
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mann_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from manifoldann_gb300 import _lib

    lib = _lib.load()
    syms = declared_symbols()
    assert "mann_knn" in syms and "mann_knn_graph" in syms
    for s in syms:
        assert hasattr(lib, s), f"{s} declared in include/ but not exported"
    # the ctypes table covers every declared symbol too
    assert set(syms) <= set(_lib.SIGNATURES), set(syms) - set(_lib.SIGNATURES)


def test_python_constants_match_the_header():
    """Every MANN_METRIC_*, MANN_PREC_* and MANN_FLAG_* code the ctypes layer
    names has the value include/mann.h defines."""
    from manifoldann_gb300 import _lib

    txt = (ROOT / "include" / "mann.h").read_text()
    defs = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define MANN_([A-Z0-9_]+) (\d+)u?\b", txt)}
    pairs = {"PREC_FP32": _lib.PREC_FP32, "PREC_BF16": _lib.PREC_BF16, "PREC_FP8": _lib.PREC_FP8,
             "PREC_AUTO": _lib.PREC_AUTO, "PREC_FP16": _lib.PREC_FP16, "FLAG_FP64_TIES": _lib.FLAG_FP64_TIES,
             "FLAG_TIME_KERNEL": _lib.FLAG_TIME_KERNEL, "FLAG_FP64_ERR": _lib.FLAG_FP64_ERR,
             "METRIC_SQEUCLIDEAN": _lib.METRIC_SQEUCLIDEAN}
    for name, value in pairs.items():
        assert defs.get(name) == value, (name, defs.get(name), value)
    from manifoldann_gb300.indices import PRECISIONS

    assert PRECISIONS == {"fp32": 0, "bf16": 1, "fp8": 2, "auto": 3, "fp16": 4}


def test_version_and_errors_without_gpu():
    from manifoldann_gb300 import _lib

    lib = _lib.load()
    assert b"sm_103a" in lib.mann_version()
    p = _lib.params(_lib.METRIC_SQEUCLIDEAN, 5)
    x = np.zeros((4, 3), np.float32)
    ids = np.zeros((4, 5), np.int32)
    d = np.zeros((4, 5), np.float32)
    # d <= 0 and n <= 0 -> ArgumentError (src/indices/bruteforce.jl:32-33)
    assert lib.mann_knn(p, x.ctypes.data, 4, x.ctypes.data, 4, 0, ids.ctypes.data, d.ctypes.data, None) == 2
    assert b"dimension" in lib.mann_last_error()
    assert lib.mann_knn(p, x.ctypes.data, 0, x.ctypes.data, 4, 3, ids.ctypes.data, d.ctypes.data, None) == 2
    # unknown metric
    bad = _lib.params(9, 5)
    assert lib.mann_knn(bad, x.ctypes.data, 4, x.ctypes.data, 4, 3, ids.ctypes.data, d.ctypes.data, None) == 2
    # graph k out of range (src/graphs/knn_graph.jl:55-59)
    p0 = _lib.params(_lib.METRIC_SQEUCLIDEAN, 4)
    assert lib.mann_knn_graph(p0, x.ctypes.data, 4, 3, 0, ids.ctypes.data, d.ctypes.data, None) == 2
    assert b"0 < k <= 3" in lib.mann_last_error()
    # k <= 0 writes nothing and succeeds (src/indices/bruteforce.jl:55-56)
    pk = _lib.params(_lib.METRIC_SQEUCLIDEAN, 0)
    assert lib.mann_knn(pk, x.ctypes.data, 4, x.ctypes.data, 4, 3, ids.ctypes.data, d.ctypes.data, None) == 0
    n = C.c_int32(-1)
    assert lib.mann_device_count(C.byref(n)) == 0 and n.value >= 0


def test_python_api_validation_without_gpu():
    import manifoldann_gb300 as M

    data = np.array([[0.0, 1.0, 2.0], [0.0, 0.0, 0.0]])
    index = M.build_index(M.BruteForceIndex, data)
    assert index.dimension == 2 and index.n_points == 3
    with pytest.raises(M.ArgumentError):
        M.query(index, data[:, :2], np.array([0.25, 0.0]), 2)  # bruteforce_tests.jl:29-31
    with pytest.raises(M.DimensionMismatch):
        M.query(index, data, np.zeros(3), 1)  # bruteforce_tests.jl:33-34
    with pytest.raises(M.DimensionMismatch):
        M.query(index, data, np.zeros((3, 0)), 1)  # ann_index.jl:84-85, empty batch still checked
    assert M.query(index, data, np.zeros((2, 0)), 1) == []
    assert M.query(index, data, np.array([0.25, 0.0]), 0) == []
    with pytest.raises(M.ArgumentError):
        M.build_index(M.BruteForceIndex, np.zeros((0, 3)))
    with pytest.raises(M.ArgumentError):
        M.build_index(M.BruteForceIndex, np.zeros((3, 0)))


def test_insert_bookkeeping():
    # test/unit/indices/bruteforce_tests.jl:37-60
    import manifoldann_gb300 as M

    data = np.array([[1.0, 2.0], [3.0, 4.0]])
    index = M.build_index(M.BruteForceIndex, data)
    M.insert(index, np.array([10.0, 20.0]))
    assert index.n_points == 3
    M.insert(index, np.array([[30.0, 40.0, 50.0, 60.0], [11.0, 12.0, 13.0, 14.0]]))
    assert index.n_points == 7
    with pytest.raises(M.DimensionMismatch):
        M.insert(index, np.array([1.0, 2.0, 3.0]))
    with pytest.raises(M.DimensionMismatch):
        M.insert(index, np.arange(1.0, 4.0).reshape(3, 1))


def test_graph_host_logic_without_gpu():
    import manifoldann_gb300 as M
    from manifoldann_gb300.graphs import _create_graph_metadata, _symmetrize_adjacency

    adj = [[2, 3], [1, 3], [2, 4], [3, 2]]
    sym = _symmetrize_adjacency(adj, 4)
    assert sym == [[2, 3], [1, 3, 4], [1, 2, 4], [2, 3]]
    meta = _create_graph_metadata(2, True, ["a", "b", "c", "d"], 4)
    assert meta["original_k"] == 2 and meta["node_metadata"] == ["a", "b", "c", "d"]
    with pytest.raises(M.ArgumentError):
        _create_graph_metadata(2, True, ["oops"], 4)
    data = np.arange(1, 13, dtype=np.float64).reshape(4, 3).T
    index = M.build_index(M.BruteForceIndex, data)
    with pytest.raises(M.ArgumentError):
        M.build_knn_graph(index, data, k=0)
    with pytest.raises(M.ArgumentError):
        M.build_knn_graph(index, data, k=4, include_self=False)
    with pytest.raises(M.ArgumentError):
        M.build_knn_graph(index, data)  # BruteForce has no configured k


def test_recall_at_k():
    import manifoldann_gb300 as M

    assert M.recall_at_k([1, 2, 3], [3, 2, 9]) == pytest.approx(2 / 3)
    assert M.recall_at_k([[1, 2], [3, 4]], [[1, 2], [5, 6]]) == 0.5
    assert M.recall_at_k([1], []) == 0.0
    with pytest.raises(M.ArgumentError):
        M.recall_at_k([[1]], [[1], [2]])


def test_dataset_handle_rejects_bad_arguments_without_gpu():
    # argument checks run before any CUDA call
    from manifoldann_gb300 import _lib

    lib = _lib.load()
    h = C.c_void_p()
    x = np.zeros((4, 3), np.float32)
    assert lib.mann_dataset_create(x.ctypes.data, 0, 3, C.byref(h)) == _lib.MANN_EINVAL_ARG
    assert lib.mann_dataset_create(x.ctypes.data, 4, 0, C.byref(h)) == _lib.MANN_EINVAL_ARG
    assert lib.mann_dataset_create(None, 4, 3, C.byref(h)) == _lib.MANN_EINVAL_ARG
    assert lib.mann_dataset_create(x.ctypes.data, 4, 3, None) == _lib.MANN_EINVAL_ARG
    assert lib.mann_dataset_upload(None, x.ctypes.data, 4) == _lib.MANN_EINVAL_ARG
    assert lib.mann_dataset_destroy(None) == 0
    p = _lib.params(_lib.METRIC_SQEUCLIDEAN, 3, _lib.PREC_FP32)
    ids = np.zeros((4, 3), np.int32)
    d = np.zeros((4, 3), np.float32)
    assert lib.mann_knn_dataset(p, None, x.ctypes.data, 4, ids.ctypes.data, d.ctypes.data, None) == \
        _lib.MANN_EINVAL_ARG
    assert lib.mann_knn_graph_dataset(p, None, 0, ids.ctypes.data, d.ctypes.data, None) == _lib.MANN_EINVAL_ARG
    assert "dataset" in _lib.last_error()


def test_fault_injection_hook_arguments_without_gpu():
    from manifoldann_gb300 import _lib

    lib = _lib.load()
    assert lib.mann_debug_inject(99, 1) == _lib.MANN_EINVAL_ARG
    assert b"unknown injection kind" in lib.mann_last_error()
    assert lib.mann_debug_inject(_lib.INJECT_ALLOC, -1) == _lib.MANN_EINVAL_ARG
    # arming and clearing touch no device
    assert lib.mann_debug_inject(_lib.INJECT_ALLOC, 2) == _lib.MANN_OK
    assert lib.mann_debug_inject(_lib.INJECT_ALLOC, 0) == _lib.MANN_OK
    assert lib.mann_debug_inject(_lib.INJECT_LAUNCH, 0) == _lib.MANN_OK


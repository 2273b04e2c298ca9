"""ctypes binding of ``libmanngpu.so`` (the C ABI in ``include/mann.h``).

The library is loaded from the package directory.  There is no CPU fallback:
if the shared object is missing, or no GB300 is visible when a compute entry
point is called, the call raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libmanngpu.so"

MANN_OK = 0
MANN_EINVAL_DIM = 1
MANN_EINVAL_ARG = 2
MANN_ENOMEM = 3
MANN_ECUDA = 4
MANN_ETIMEOUT = 5
MANN_ENODEV = 6

METRIC_EUCLIDEAN = 0
METRIC_SQEUCLIDEAN = 1
METRIC_COSINE = 2

PREC_FP32 = 0
PREC_BF16 = 1
PREC_FP8 = 2
PREC_AUTO = 3
PREC_FP16 = 4

FLAG_FP64_TIES = 1
FLAG_TIME_KERNEL = 2
FLAG_FP64_ERR = 4
INJECT_ALLOC = 1
INJECT_LAUNCH = 2
INJECT_QUEUE = 3


class DimensionMismatch(ValueError):
    """Julia's ``DimensionMismatch`` (src/utils/validation.jl:8-12)."""


class ArgumentError(ValueError):
    """Julia's ``ArgumentError`` (src/utils/validation.jl:13-17)."""


class MannError(RuntimeError):
    """A CUDA / device error reported by the library."""


class KnnParams(C.Structure):
    _fields_ = [
        ("metric", C.c_int32),
        ("k", C.c_int32),
        ("precision", C.c_int32),
        ("margin", C.c_int32),
        ("flags", C.c_uint32),
        ("reserved", C.c_int32 * 3),
    ]


class KnnReport(C.Structure):
    _fields_ = [
        ("rows", C.c_int64),
        ("rows_fallback", C.c_int64),
        ("rows_fp64_ties", C.c_int64),
        ("candidates", C.c_int64),
        ("max_abs_err_fp64", C.c_double),
        ("precision_used", C.c_int32),
        ("margin_used", C.c_int32),
        ("kernel_ms", C.c_double),
        ("launches", C.c_int64),
        ("rows_ties_widened", C.c_int64),
        ("rows_unresolved", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class KmeansParams(C.Structure):
    _fields_ = [
        ("k", C.c_int32),
        ("metric", C.c_int32),
        ("init", C.c_int32),
        ("max_iters", C.c_int32),
        ("tol", C.c_double),
        ("subsample", C.c_int64),
        ("seed", C.c_uint64),
    ]


class IvfBuildParams(C.Structure):
    _fields_ = [
        ("nlist", C.c_int32),
        ("centroid_metric", C.c_int32),
        ("kmeans_max_iters", C.c_int32),
        ("reserved", C.c_int32),
        ("kmeans_tol", C.c_double),
        ("kmeans_subsample", C.c_int64),
        ("seed", C.c_uint64),
    ]


class ProbeParams(C.Structure):
    _fields_ = [
        ("din", C.c_int32),
        ("hidden1", C.c_int32),
        ("hidden2", C.c_int32),
        ("nout", C.c_int32),
        ("batch", C.c_int32),
        ("use_prior", C.c_int32),
        ("lr", C.c_float),
        ("beta1", C.c_float),
        ("beta2", C.c_float),
        ("eps", C.c_float),
        ("weight_decay", C.c_float),
        ("beta_init", C.c_float),
        ("seed", C.c_uint64),
    ]


class PcaParams(C.Structure):
    _fields_ = [("intrinsic_dim", C.c_int32), ("reserved", C.c_int32), ("min_variance_ratio", C.c_double)]


_P = C.c_void_p
_I64 = C.c_int64
_I32 = C.c_int32

# name -> (restype, argtypes); every symbol declared in include/mann.h
SIGNATURES = {
    "mann_version": (C.c_char_p, []),
    "mann_last_error": (C.c_char_p, []),
    "mann_device_count": (_I32, [C.POINTER(_I32)]),
    "mann_host_register": (_I32, [_P, _I64]),
    "mann_host_unregister": (_I32, [_P]),
    "mann_knn": (_I32, [C.POINTER(KnnParams), _P, _I64, _P, _I64, _I32, _P, _P, C.POINTER(KnnReport)]),
    "mann_knn_device": (_I32, [C.POINTER(KnnParams), _P, _I64, _P, _I64, _I32, _P, _P,
                               C.POINTER(KnnReport), _P]),
    "mann_knn_graph": (_I32, [C.POINTER(KnnParams), _P, _I64, _I32, _I32, _P, _P, C.POINTER(KnnReport)]),
    "mann_knn_graph_device": (_I32, [C.POINTER(KnnParams), _P, _I64, _I32, _I32, _P, _P,
                                     C.POINTER(KnnReport), _P]),
    "mann_dataset_create": (_I32, [_P, _I64, _I32, C.POINTER(_P)]),
    "mann_dataset_upload": (_I32, [_P, _P, _I64]),
    "mann_dataset_destroy": (_I32, [_P]),
    "mann_knn_dataset": (_I32, [C.POINTER(KnnParams), _P, _P, _I64, _P, _P, C.POINTER(KnnReport)]),
    "mann_knn_graph_dataset": (_I32, [C.POINTER(KnnParams), _P, _I32, _P, _P, C.POINTER(KnnReport)]),
    "mann_knn_device_noalloc": (_I32, [C.POINTER(KnnParams), _P, _I64, _P, _I64, _I32, _P, _P, _P]),
    "mann_pairwise_distances": (_I32, [_P, _I64, _P, _I32, _I32, _I32, _P]),
    "mann_kmeans_assign": (_I32, [_P, _I64, _P, _I32, _I32, _I32, _P, _P]),
    "mann_kmeanspp": (_I32, [_P, _I64, _I32, _I32, _I64, _P, _P]),
    "mann_kmeans_lloyd": (_I32, [_P, _I64, _I32, _I32, _P, _I32, C.c_double, _I32, _P, _P]),
    "mann_kmeans_fit": (_I32, [C.POINTER(KmeansParams), _P, _I64, _I32, _P, _P, _P]),
    "mann_ivf_build": (_I32, [C.POINTER(IvfBuildParams), _P, _I64, _I32, _P, _P, _P, _P]),
    "mann_ivf_search": (_I32, [C.POINTER(KnnParams), _I32, _I32, _P, _I64, _I32, _P, _I32, _P, _P, _P,
                               _I64, _P, _P]),
    "mann_ivf_search_device": (_I32, [C.POINTER(KnnParams), _I32, _I32, _P, _I64, _I32, _P, _I32, _P,
                                      _P, _P, _I64, _P, _P, _P]),
    "mann_probe_param_count": (_I64, [C.POINTER(ProbeParams)]),
    "mann_probe_init": (_I32, [C.POINTER(ProbeParams), _P]),
    "mann_probe_create": (_I32, [C.POINTER(ProbeParams), _P, _P, C.POINTER(_P)]),
    "mann_probe_destroy": (_I32, [_P]),
    "mann_probe_get_params": (_I32, [_P, _P]),
    "mann_probe_train": (_I32, [_P, _P, _I64, _P, _I32, _I32, _P]),
    "mann_probe_grad": (_I32, [_P, _P, _I64, _P, _I32, _P, _P]),
    "mann_probe_scores": (_I32, [_P, _P, _I64, _P]),
    "mann_probe_route_device": (_I32, [_P, _P, _I64, _I32, _P, _P, _P]),
    "mann_ivf_search_learned_device": (_I32, [_P, C.POINTER(KnnParams), _I32, _P, _I64, _I32, _I32, _P, _P,
                                              _P, _I64, _P, _P, _P]),
    "mann_ivf_search_learned": (_I32, [_P, C.POINTER(KnnParams), _I32, _P, _I64, _I32, _I32, _P, _P, _P,
                                       _I64, _P, _P]),
    "mann_knn_graph_batched": (_I32, [C.POINTER(KnnParams), _P, _P, _I32, _I32, _I32, _P, _P,
                                      C.POINTER(KnnReport)]),
    "mann_knn_graph_batched_device": (_I32, [C.POINTER(KnnParams), _P, _P, _I32, _I32, _I32, _P, _P,
                                             C.POINTER(KnnReport), _P]),
    "mann_local_pca": (_I32, [C.POINTER(PcaParams), _P, _I64, _I32, _P, _P, _I64, _P, _I32, _I32, _P, _P, _P]),
    "mann_local_pca_device": (_I32, [C.POINTER(PcaParams), _P, _I64, _I32, _P, _P, _I64, _P, _I32, _I32, _P, _P,
                                     _P, _P]),
    "mann_edge_weights": (_I32, [_I32, _P, _I64, _I32, _P, _I32, _P, _P, _I32, _P, _P]),
    "mann_edge_weights_device": (_I32, [_I32, _P, _I64, _I32, _P, _I32, _P, _P, _I32, _P, _P, _P]),
    "mann_knn_graph_symmetrize": (_I32, [_P, _I64, _I32, _P, _P, _P]),
    "mann_knn_graph_symmetrize_device": (_I32, [_P, _I64, _I32, _P, _P, _P, _P]),
    "mann_ivf_scan_device": (_I32, [C.POINTER(KnnParams), _P, _I32, _P, _I64, _I32, _I32, _P, _P, _P,
                                    _I64, _P, _P, _P]),
    "mann_measure_fp32_peak": (_I32, [C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "mann_debug_inject": (_I32, [_I32, _I32]),
}

_lib = None
_lock = threading.Lock()


def load() -> C.CDLL:
    """Load libmanngpu.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise MannError(
                    f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
            lib = C.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def last_error() -> str:
    return load().mann_last_error().decode()


def check(status: int) -> None:
    if status == MANN_OK:
        return
    msg = last_error()
    if status == MANN_EINVAL_DIM:
        raise DimensionMismatch(msg)
    if status == MANN_EINVAL_ARG:
        raise ArgumentError(msg)
    raise MannError(f"libmanngpu status {status}: {msg}")


def params(metric: int, k: int, precision: int = PREC_FP32, margin: int = 0, flags: int = 0) -> KnnParams:
    p = KnnParams()
    p.metric = metric
    p.k = k
    p.precision = precision
    p.margin = margin
    p.flags = flags
    return p

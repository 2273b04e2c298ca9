"""Metric objects mirroring the Distances.jl aliases of the reference
(src/utils/distances.jl:15-18).

``Euclidean()`` is the reference default (``default_distance``).  Calling a
metric on two vectors evaluates it on the GPU through the library (one
1-point search), so even this convenience has no CPU arithmetic path.
"""
from __future__ import annotations

import numpy as np

from . import _lib


class Metric:
    code: int = -1
    name: str = "?"

    def __call__(self, x, y) -> float:
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float32).ravel())
        y = np.ascontiguousarray(np.asarray(y, dtype=np.float32).ravel())
        if x.shape != y.shape:
            raise _lib.DimensionMismatch(f"vectors of length {x.size} and {y.size}")
        lib = _lib.load()
        ids = np.empty(1, np.int32)
        d = np.empty(1, np.float32)
        p = _lib.params(self.code, 1)
        _lib.check(lib.mann_knn(p, y.ctypes.data, 1, x.ctypes.data, 1, x.size, ids.ctypes.data,
                                d.ctypes.data, None))
        return float(d[0])

    def __eq__(self, other) -> bool:
        return type(self) is type(other)

    def __hash__(self) -> int:
        return hash(type(self))

    def __repr__(self) -> str:
        return f"{self.name}()"


class Euclidean(Metric):
    """sqrt(sum((x - y)^2))"""
    code = _lib.METRIC_EUCLIDEAN
    name = "Euclidean"


class SqEuclidean(Metric):
    """sum((x - y)^2)"""
    code = _lib.METRIC_SQEUCLIDEAN
    name = "SqEuclidean"


class CosineDist(Metric):
    """max(1 - x.y / (|x| |y|), 0); NaN when a norm is zero."""
    code = _lib.METRIC_COSINE
    name = "CosineDist"


default_distance = Euclidean()
default_squared_distance = SqEuclidean()
euclidean_distance = Euclidean()
cosine_distance = CosineDist()


def metric_code(distance) -> int:
    if isinstance(distance, Metric):
        return distance.code
    raise _lib.ArgumentError(
        f"metric {distance!r} has no GPU form; supported: Euclidean(), SqEuclidean(), CosineDist()")

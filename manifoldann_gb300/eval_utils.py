"""``recall_at_k`` (src/utils/eval_utils.jl:7-36)."""
from __future__ import annotations

from ._lib import ArgumentError


def recall_at_k(found, ground_truth) -> float:
    """Single query: |found ∩ truth| / |truth|.  Batches (lists of lists): the mean."""
    if len(found) and hasattr(found[0], "__len__") and not isinstance(found[0], (str, bytes)):
        if len(found) != len(ground_truth):
            raise ArgumentError("found and ground truth batches must match in length")
        if len(found) == 0:
            return 0.0
        return sum(recall_at_k(f, g) for f, g in zip(found, ground_truth)) / len(found)
    k = len(ground_truth)
    if k == 0:
        return 0.0
    gt = set(int(g) for g in ground_truth)
    return sum(1 for f in found if int(f) in gt) / k

"""Failure handling on the host side: an out-of-memory scratch request, a
failed kernel launch and an unpublished device work queue, all injected
through mann_debug_inject (nothing on the GPU faults, traps or hangs: the
queue's consumers run out a short bounded wait with no other work in flight).  Each call returns its status with a
message, and the next call on the same context succeeds with the same
answer -- the library never aborts (error rules of the reference's Julia
API: src/utils/validation.jl:8-35)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(lib, base, q, k, precision):
    from manifoldann_gb300 import _lib

    ids = np.full((len(q), k), -7, np.int32)
    d = np.full((len(q), k), 7.0, np.float32)
    p = _lib.params(_lib.METRIC_SQEUCLIDEAN, k, precision)
    st = lib.mann_knn(p, base.ctypes.data, len(base), q.ctypes.data, len(q), base.shape[1], ids.ctypes.data,
                      d.ctypes.data, None)
    return st, ids, d


@pytest.mark.parametrize("precision", [0, 1])
def test_injected_out_of_memory_then_recovery(gpu_lib, precision):
    from manifoldann_gb300 import _lib

    rng = np.random.default_rng(31)
    base = rng.standard_normal((5000, 128)).astype(np.float32)
    q = rng.standard_normal((200, 128)).astype(np.float32)
    st, ids0, d0 = _call(gpu_lib, base, q, 10, precision)
    assert st == _lib.MANN_OK
    try:
        _lib.check(gpu_lib.mann_debug_inject(_lib.INJECT_ALLOC, 1))
        st, _, _ = _call(gpu_lib, base, q, 10, precision)
        assert st == _lib.MANN_ENOMEM
        assert b"out of memory" in gpu_lib.mann_last_error()
    finally:
        gpu_lib.mann_debug_inject(_lib.INJECT_ALLOC, 0)
    st, ids1, d1 = _call(gpu_lib, base, q, 10, precision)
    assert st == _lib.MANN_OK
    assert np.array_equal(ids0, ids1) and np.array_equal(d0.view(np.uint32), d1.view(np.uint32))


def test_injected_out_of_memory_raises_in_python(gpu_lib):
    import manifoldann_gb300 as M
    from manifoldann_gb300 import _lib

    rng = np.random.default_rng(32)
    data = rng.standard_normal((64, 3000)).astype(np.float32)
    index = M.build_index(M.BruteForceIndex, data, distance=M.SqEuclidean())
    try:
        _lib.check(gpu_lib.mann_debug_inject(_lib.INJECT_ALLOC, 1))
        with pytest.raises(M.MannError, match="out of memory"):
            M.knn_arrays(index, data, data[:, :10], 5)
    finally:
        gpu_lib.mann_debug_inject(_lib.INJECT_ALLOC, 0)
    ids, _ = M.knn_arrays(index, data, data[:, :10], 5)
    assert (ids[:, 0] == np.arange(10)).all()


@pytest.mark.parametrize("precision", [0, 1])
def test_injected_launch_error_then_recovery(gpu_lib, precision):
    from manifoldann_gb300 import _lib

    rng = np.random.default_rng(33)
    base = rng.standard_normal((4000, 256)).astype(np.float32)
    q = rng.standard_normal((300, 256)).astype(np.float32)
    st, ids0, d0 = _call(gpu_lib, base, q, 12, precision)
    assert st == _lib.MANN_OK
    for nth in (1, 2):  # the first or the second checked launch of the call fails
        try:
            _lib.check(gpu_lib.mann_debug_inject(_lib.INJECT_LAUNCH, nth))
            st, _, _ = _call(gpu_lib, base, q, 12, precision)
            assert st == _lib.MANN_ECUDA
            assert b"injected" in gpu_lib.mann_last_error()
        finally:
            gpu_lib.mann_debug_inject(_lib.INJECT_LAUNCH, 0)
        st, ids1, d1 = _call(gpu_lib, base, q, 12, precision)
        assert st == _lib.MANN_OK
        assert np.array_equal(ids0, ids1) and np.array_equal(d0.view(np.uint32), d1.view(np.uint32))


def test_unpublished_work_queue_times_out_then_recovers(gpu_lib):
    """The batched graphs' persistent kernel waits (bounded) for its work
    queue to be published; with the publish dropped it returns MANN_ETIMEOUT
    and the next call -- the captured graph replay -- is correct."""
    from manifoldann_gb300 import _lib, synthetic

    clouds = synthetic.manifold_clouds(5, 300, 2000, 16, seed=9)
    offs = np.zeros(6, np.int64)
    offs[1:] = np.cumsum([len(c) for c in clouds])
    pts = np.ascontiguousarray(np.concatenate(clouds))
    N = int(offs[-1])
    p = _lib.params(_lib.METRIC_SQEUCLIDEAN, 10, _lib.PREC_FP32)

    def call():
        ids = np.full((N, 10), -7, np.int32)
        d = np.full((N, 10), 7.0, np.float32)
        st = gpu_lib.mann_knn_graph_batched(p, pts.ctypes.data, offs.ctypes.data, 5, 16, 0, ids.ctypes.data,
                                            d.ctypes.data, None)
        return st, ids, d

    st, ids0, d0 = call()
    assert st == _lib.MANN_OK
    try:
        _lib.check(gpu_lib.mann_debug_inject(_lib.INJECT_QUEUE, 1))
        st, _, _ = call()
        assert st == _lib.MANN_ETIMEOUT
        assert b"work queue" in gpu_lib.mann_last_error()
    finally:
        gpu_lib.mann_debug_inject(_lib.INJECT_QUEUE, 0)
    for _ in range(2):
        st, ids1, d1 = call()
        assert st == _lib.MANN_OK
        assert np.array_equal(ids0, ids1) and np.array_equal(d0.view(np.uint32), d1.view(np.uint32))


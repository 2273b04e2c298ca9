"""The allocation-free entry point (mann_knn_device_noalloc) against the
regular device entry point: the same FP32 kernels, so the same ids and the
same distance bits, on consecutive calls that share its scratch array.

Callers that own all device memory through their own pool, or that must not
stall the device with cudaMalloc, use this entry point; it reuses one fixed
array of scratch and rejects searches that do not fit in it."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(lib, fn_name, base_t, q_t, k, metric, stream, noalloc):
    import torch

    from manifoldann_gb300 import _lib

    nq, d = q_t.shape
    ids = torch.full((nq, k), -7, dtype=torch.int32, device="cuda")
    dists = torch.full((nq, k), 7.0, dtype=torch.float32, device="cuda")
    p = _lib.params(metric, k, _lib.PREC_FP32)
    if noalloc:
        st = lib.mann_knn_device_noalloc(p, base_t.data_ptr(), base_t.shape[0], q_t.data_ptr(), nq, d,
                                         ids.data_ptr(), dists.data_ptr(), C.c_void_p(stream))
    else:
        st = lib.mann_knn_device(p, base_t.data_ptr(), base_t.shape[0], q_t.data_ptr(), nq, d,
                                 ids.data_ptr(), dists.data_ptr(), None, C.c_void_p(stream))
    _lib.check(st)
    torch.cuda.synchronize()
    return ids.cpu().numpy(), dists.cpu().numpy()


@pytest.mark.parametrize("metric", [0, 1, 2])
def test_noalloc_matches_regular_entry_point(gpu_lib, metric):
    import torch

    rng = np.random.default_rng(100 + metric)
    stream = torch.cuda.current_stream().cuda_stream
    # calls in a row with different shapes: a later call must not see an earlier one's
    # scratch; the last two are few-row batches (q <= 32), which run the few-row kernel
    for n, nq, d, k in [(20000, 700, 64, 10), (5003, 41, 37, 33), (70000, 5, 64, 10), (3001, 32, 19, 64)]:
        base = torch.from_numpy(rng.standard_normal((n, d)).astype(np.float32)).cuda()
        q = torch.from_numpy(rng.standard_normal((nq, d)).astype(np.float32)).cuda()
        ids_r, d_r = _run(gpu_lib, "regular", base, q, k, metric, stream, noalloc=False)
        ids_n, d_n = _run(gpu_lib, "noalloc", base, q, k, metric, stream, noalloc=True)
        assert np.array_equal(ids_n, ids_r)
        assert np.array_equal(d_n.view(np.uint32), d_r.view(np.uint32))


def test_noalloc_rejects_what_does_not_fit(gpu_lib):
    import torch

    from manifoldann_gb300 import _lib

    # 300,000 queries x k=64 lists are far beyond the fixed scratch: rejected, nothing launched
    base = torch.zeros((1000, 8), dtype=torch.float32, device="cuda")
    p = _lib.params(1, 64, _lib.PREC_FP32)
    st = gpu_lib.mann_knn_device_noalloc(p, base.data_ptr(), 1000, base.data_ptr(), 300000, 8,
                                         base.data_ptr(), base.data_ptr(), None)
    assert st == _lib.MANN_EINVAL_ARG
    assert b"scratch" in gpu_lib.mann_last_error()
    p = _lib.params(1, 5, _lib.PREC_BF16)
    st = gpu_lib.mann_knn_device_noalloc(p, base.data_ptr(), 1000, base.data_ptr(), 10, 8,
                                         base.data_ptr(), base.data_ptr(), None)
    assert st == _lib.MANN_EINVAL_ARG

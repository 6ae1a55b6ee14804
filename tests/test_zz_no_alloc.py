"""The allocation-free direct sum, through the C ABI.

tc_direct_device_noalloc serves callers that cannot call cudaMalloc (a stream
being captured into a CUDA graph, a framework that owns all device memory, a
loop that must not block in the allocator): its scratch is a fixed static
device array.  This checks it against tc_direct_device on two calls in a row
(the shared scratch keeps the previous call's contents, which must not leak
into the next result) and that oversized requests are refused.  The file is
named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from masterthesislucas_gb300 import _lib, datasets

pytestmark = pytest.mark.gpu


def test_noalloc_direct_matches_allocating_entry_point():
    import torch

    L = _lib.lib()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    cases = [("gravity", 1, 1e-3, datasets.gaussian_mixture(20000, seed=41), 3000),
             ("tsne", 0, 0.0, np.random.default_rng(42).normal(0, 4, (30000, 2)), 4096)]
    for name, kernel, eps, pos, m in cases:
        pos_d = torch.from_numpy(np.ascontiguousarray(pos, np.float64)).to(dev)
        n = pos_d.shape[0]
        rows = torch.from_numpy(np.random.default_rng(5).choice(n, m, replace=False).astype(np.int64)).to(dev)
        # FP64: the same sums up to rounding; FP32: the same pairs summed over a
        # different slice partition (the fixed scratch holds fewer slices)
        for precision, tol_max, tol_med in ((_lib.TC_PREC_FP64, 1e-12, 1e-13), (_lib.TC_PREC_FP32, 1e-4, 2e-6)):
            g_ref = torch.zeros((m, 2), dtype=torch.float64, device=dev)
            z_ref = torch.zeros(1, dtype=torch.float64, device=dev)
            torch.cuda.synchronize()
            _lib.check(L.tc_direct_device(kernel, eps, precision, _lib.ptr(pos_d), n, _lib.ptr(rows), m,
                                          _lib.ptr(g_ref), _lib.ptr(z_ref), ctypes.c_void_p(stream.cuda_stream)))
            for call in range(2):
                g = torch.full((m, 2), float("nan"), dtype=torch.float64, device=dev)
                z = torch.zeros(1, dtype=torch.float64, device=dev)
                torch.cuda.synchronize()
                _lib.check(L.tc_direct_device_noalloc(kernel, eps, precision, _lib.ptr(pos_d), n, _lib.ptr(rows), m,
                                                      _lib.ptr(g), _lib.ptr(z), ctypes.c_void_p(stream.cuda_stream)))
                stream.synchronize()
                a, b = g.cpu().numpy(), g_ref.cpu().numpy()
                assert np.isfinite(a).all(), (name, call)
                err = np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)
                assert err.max() < tol_max and np.median(err) < tol_med, (name, precision, call, err.max())
                assert float(z.item()) == pytest.approx(float(z_ref.item()), rel=tol_max / 10)


def test_noalloc_direct_rejects_oversized_requests():
    import torch

    L = _lib.lib()
    dev = torch.device("cuda", 0)
    m = (1 << 19) // 4 + 1  # one row beyond the maximum
    pos_d = torch.zeros((m, 2), dtype=torch.float64, device=dev)
    g = torch.zeros((m, 2), dtype=torch.float64, device=dev)
    rc = L.tc_direct_device_noalloc(0, 0.0, _lib.TC_PREC_FP64, _lib.ptr(pos_d), m, None, m, _lib.ptr(g), None,
                                    None)
    assert rc == _lib.TC_ERR_INVALID
    assert b"exceeds the maximum" in L.tc_last_error()

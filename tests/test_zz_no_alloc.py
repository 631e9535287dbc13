"""The allocation-free H_eff . A entry point (ptn_heff_apply_noalloc).

Callers that cannot allocate device memory (an FFI host without a CUDA
allocator, a process whose memory belongs to another framework's pool) get an
H_eff . A whose scratch is a fixed device array inside the library. This test
calls it through the C ABI twice in a row, with different inputs, and checks
each result against ptn_heff_apply with a caller-provided workspace, at the
1e-12 relative tolerance of the FP64 contraction tests. It also checks that a
size beyond the array is refused. Collected last on purpose."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _crandn(shape, rng):
    return (rng.normal(size=shape) + 1j * rng.normal(size=shape)) / np.sqrt(2)


def _case(rng, Dl, d, Dr, cl, cr):
    a = _crandn((Dl, d, Dr), rng)
    w = rng.normal(size=(cl, d, d, cr))
    w[np.abs(w) < 0.7] = 0.0
    l = _crandn((Dl, cl, Dl), rng)
    r = _crandn((Dr, cr, Dr), rng)
    return a, w, l, r


def test_heff_noalloc_matches_workspace_entry():
    import torch
    from pytenet_gb300 import _lib
    from pytenet_gb300.device import to_dev, to_host, ptr, stream_ptr, empty
    L = _lib.load()
    rng = np.random.default_rng(2027)
    for dims in [(64, 2, 96, 5, 4), (130, 2, 97, 4, 5)]:   # two calls in a row, different inputs
        Dl, d, Dr, cl, cr = dims
        a, w, l, r = (to_dev(x) for x in _case(rng, *dims))
        ref = empty((Dl, d, Dr))
        wsb = L.ptn_heff_workspace_bytes(Dl, d, Dr, cl, cr, 0)
        ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
        _lib.check(L.ptn_heff_apply(ptr(a), ptr(w), ptr(l), ptr(r), ptr(ref), Dl, d, Dr, cl, cr, 0,
                                    ptr(ws), wsb, stream_ptr()))
        out = empty((Dl, d, Dr))
        _lib.check(L.ptn_heff_apply_noalloc(ptr(a), ptr(w), ptr(l), ptr(r), ptr(out), Dl, d, Dr,
                                            cl, cr, stream_ptr()))
        x, y = to_host(out), to_host(ref)
        assert np.linalg.norm(x - y) <= RTOL * np.linalg.norm(y)


def test_heff_noalloc_rejects_oversize():
    from pytenet_gb300 import _lib
    L = _lib.load()
    cap = L.ptn_heff_noalloc_capacity_bytes()
    D = 1024                      # 2 * 1024 * 10 * 1024 * 16 bytes = 320 MiB > capacity
    assert 2 * D * 10 * D * 16 > cap
    st = L.ptn_heff_apply_noalloc(None, None, None, None, None, D, 2, D, 5, 5, None)
    assert st == _lib.PTN_BAD_SHAPE
    assert b"scratch" in L.ptn_last_error()

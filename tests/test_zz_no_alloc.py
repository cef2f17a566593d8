"""The entry point that allocates nothing (pfast_fsm3d_noalloc), called through the
C ABI: it serves callers that cannot allocate device memory (code under CUDA
stream capture, hosts whose own allocator owns the device), taking its work
memory from a fixed static device array instead.  Its field must equal the
allocating entry point's (pfast_fsm3d) bit for bit -- the tolerance of the plain
FP64 tests -- on two calls in a row, which share the static array.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(vp_dev, U_dev, src, maxswp, h, shape, stream=None):
    from pfast_gb300 import _capi
    nz, nr, nc = shape
    return _capi.lib().pfast_fsm3d_noalloc(C.c_void_p(vp_dev.data_ptr()), C.c_void_p(U_dev.data_ptr()),
                                           int(src[0]), int(src[1]), int(src[2]), maxswp, h[0], h[1], h[2],
                                           nr, nc, nz, stream)


def test_noalloc_matches_allocating_entry_point_twice():
    import torch
    import pfast_gb300 as pg
    shape, h = (20, 24, 40), (10.0, 12.5, 8.0)
    rng = np.random.default_rng(21)
    vp = 1500.0 + 2000.0 * rng.random(shape)
    srcs = np.array([[5, 7, 3], [23, 39, 19]], np.int32)   # (row, col, z)
    d_vp = torch.from_numpy(vp).cuda()
    for s in range(2):   # two calls in a row on the shared static array
        U_ref = np.empty(shape)
        pg.fsm3d(vp, U_ref, srcs, s, 100, h[0], h[1], h[2], shape[1], shape[2], shape[0])
        d_U = torch.full(shape, -1.0, dtype=torch.float64, device="cuda")
        st = _noalloc(d_vp, d_U, srcs[s], 100, h, shape)
        assert st == 0, pg._capi.lib().pfast_last_error()
        torch.cuda.synchronize()
        U = d_U.cpu().numpy()
        assert np.array_equal(U.view(np.int64), U_ref.view(np.int64))


def test_noalloc_rejects_grids_beyond_its_limit():
    import torch
    from pfast_gb300 import _capi
    shape = (65, 128, 128)   # 1,064,960 nodes > PFAST_NOALLOC_MAX_NODES
    assert shape[0] * shape[1] * shape[2] > _capi.PFAST_NOALLOC_MAX_NODES
    d_vp = torch.full((8,), 2000.0, dtype=torch.float64, device="cuda")   # never read: the size check comes first
    d_U = torch.empty((8,), dtype=torch.float64, device="cuda")
    st = _noalloc(d_vp, d_U, (0, 0, 0), 100, (10.0, 10.0, 10.0), shape)
    assert st == _capi.PFAST_ERR_INVALID
    assert b"no-allocation limit" in _capi.lib().pfast_last_error()

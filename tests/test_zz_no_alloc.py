"""The entry point that allocates nothing (pfast_fsm3d_noalloc), called through the
C ABI.  It serves callers that cannot allocate device memory -- a host whose own pool
allocator or memory budget owns the device and forbids libraries to call cudaMalloc --
by taking its work memory from a fixed static device array instead.  Its field must
equal the allocating entry point's (pfast_fsm3d) bit for bit -- the tolerance of the
plain FP64 tests -- on two calls in a row, which share the static array; the same holds
on a caller's own stream, with an iteration cap, and for the rejection of a velocity
model that is not positive.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE, H = (20, 24, 40), (10.0, 12.5, 8.0)   # (nz, nrows, ncols), (dx, dy, dz)


def _noalloc(vp_dev, U_dev, src, maxswp, h, shape, stream=None):
    from pfast_gb300 import _capi
    nz, nr, nc = shape
    return _capi.lib().pfast_fsm3d_noalloc(C.c_void_p(vp_dev.data_ptr()), C.c_void_p(U_dev.data_ptr()),
                                           int(src[0]), int(src[1]), int(src[2]), maxswp, h[0], h[1], h[2],
                                           nr, nc, nz, stream)


def _reference_field(vp, srcs, s, maxswp):
    import pfast_gb300 as pg
    U = np.empty(SHAPE)
    pg.fsm3d(vp, U, srcs, s, maxswp, H[0], H[1], H[2], SHAPE[1], SHAPE[2], SHAPE[0])
    return U


def _model(seed=21):
    rng = np.random.default_rng(seed)
    return 1500.0 + 2000.0 * rng.random(SHAPE)


SRCS = np.array([[5, 7, 3], [23, 39, 19]], np.int32)   # (row, col, z)


def test_noalloc_matches_allocating_entry_point_twice():
    import torch
    import pfast_gb300 as pg
    vp = _model()
    d_vp = torch.from_numpy(vp).cuda()
    for s in range(2):   # two calls in a row on the shared static array
        U_ref = _reference_field(vp, SRCS, s, 100)
        d_U = torch.full(SHAPE, -1.0, dtype=torch.float64, device="cuda")
        st = _noalloc(d_vp, d_U, SRCS[s], 100, H, SHAPE)
        assert st == 0, pg._capi.lib().pfast_last_error()
        torch.cuda.synchronize()
        U = d_U.cpu().numpy()
        assert np.array_equal(U.view(np.int64), U_ref.view(np.int64))


def test_noalloc_on_a_caller_stream_with_an_iteration_cap():
    """On a stream of the caller's (not the default stream), with MAXSwp = 1 (one outer
    iteration: the field is not converged) and then the full cap, still bit-equal."""
    import torch
    import pfast_gb300 as pg
    vp = _model(22)
    side = torch.cuda.Stream()
    d_vp = torch.from_numpy(vp).cuda()
    torch.cuda.synchronize()
    for maxswp in (1, 100):
        U_ref = _reference_field(vp, SRCS, 1, maxswp)
        with torch.cuda.stream(side):
            d_U = torch.full(SHAPE, -1.0, dtype=torch.float64, device="cuda")
            st = _noalloc(d_vp, d_U, SRCS[1], maxswp, H, SHAPE, stream=C.c_void_p(side.cuda_stream))
        assert st == 0, pg._capi.lib().pfast_last_error()
        side.synchronize()
        U = d_U.cpu().numpy()
        assert np.array_equal(U.view(np.int64), U_ref.view(np.int64)), f"MAXSwp={maxswp}"
    U1 = _reference_field(vp, SRCS, 1, 1)
    assert not np.array_equal(U1, U_ref), "one iteration should leave the field unconverged"


def test_noalloc_rejects_a_non_positive_velocity_like_the_allocating_entry_point():
    import torch
    import pfast_gb300 as pg
    from pfast_gb300 import _capi
    vp = _model(23)
    vp[4, 5, 6] = 0.0
    with pytest.raises(pg.PfastError) as ei:
        _reference_field(vp, SRCS, 0, 100)
    assert ei.value.status == _capi.PFAST_ERR_INVALID
    d_vp = torch.from_numpy(vp).cuda()
    d_U = torch.zeros(SHAPE, dtype=torch.float64, device="cuda")
    st = _noalloc(d_vp, d_U, SRCS[0], 100, H, SHAPE)
    assert st == _capi.PFAST_ERR_INVALID
    assert b"positive finite" in _capi.lib().pfast_last_error()
    # the array keeps no state that spoils the next call
    vp[4, 5, 6] = 2000.0
    d_vp = torch.from_numpy(vp).cuda()
    st = _noalloc(d_vp, d_U, SRCS[0], 100, H, SHAPE)
    assert st == 0, _capi.lib().pfast_last_error()
    torch.cuda.synchronize()
    U_ref = _reference_field(vp, SRCS, 0, 100)
    assert np.array_equal(d_U.cpu().numpy().view(np.int64), U_ref.view(np.int64))


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

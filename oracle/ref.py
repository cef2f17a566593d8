"""ctypes wrapper of the reference's own solvers built into oracle/_ref by
oracle/build_ref.py.  TEST INFRASTRUCTURE ONLY; available only where the
reference tree was present at build time (`available()` says so).

The reference functions exit the process on malformed input (for example
src/RT_pfsm2d.h:232), so only well-formed cases are passed here.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
_libs = {}
_d, _i, _p = C.c_double, C.c_int, C.c_void_p


def available():
    return all(os.path.exists(os.path.join(REF, f"libpfast_ref{d}.so")) for d in ("2d", "3d"))


def _lib(dim):
    if dim not in _libs:
        L = C.CDLL(os.path.join(REF, f"libpfast_ref{dim}.so"))
        if dim == "3d":
            L.ref_fsm3d.restype = None
            L.ref_fsm3d.argtypes = [_p, _p, _p, _i, _i, _d, _d, _d, _i, _i, _i]
            L.ref_adjoint3d.restype = _d
            L.ref_adjoint3d.argtypes = [_p, _p, _p, _p, _p, _p, _p, _i, _i, _d, _d, _d, _i, _i, _i]
        else:
            L.ref_rt_fsm2d.restype = None
            L.ref_rt_fsm2d.argtypes = [_p, _p, _p, _p, _p, _p, _p, _p, _i, _i, _i, _d, _d, _i, _i]
            L.ref_tadjoint2d.restype = _d
            L.ref_tadjoint2d.argtypes = [_p, _p, _p, _p, _p, _p, _p, _i, _i, _d, _d, _i, _i]
            L.ref_radjoint2d.restype = _d
            L.ref_radjoint2d.argtypes = [_p, _p, _p, _p, _p, _p, _p, _p, _i, _i, _i, _d, _d, _i, _i]
        _libs[dim] = L
    return _libs[dim]


def _c(a, dt):
    return np.array(a, dtype=dt, order="C", copy=True)   # the reference takes non-const pointers


def fsm3d(vp, src, srcid, maxswp=100, dx=1.0, dy=1.0, dz=1.0):
    vp = _c(vp, np.float64)
    nz, nr, nc = vp.shape
    src = _c(src, np.int32)
    U = np.empty_like(vp)
    _lib("3d").ref_fsm3d(vp.ctypes.data, U.ctypes.data, src.ctypes.data, srcid, maxswp, dx, dy, dz, nr, nc, nz)
    return U


def adjoint3d(T, Tobs, rec, nxyz, src, srnum, srcid, maxswp=100, dx=1.0, dy=1.0, dz=1.0):
    T = _c(T, np.float64)
    nz, nr, nc = T.shape
    a = [_c(Tobs, np.float64), _c(rec, np.int32), _c(nxyz, np.float64), _c(src, np.int32), _c(srnum, np.int32)]
    L = np.empty_like(T)
    E = _lib("3d").ref_adjoint3d(L.ctypes.data, T.ctypes.data, *[x.ctypes.data for x in a], srcid, maxswp,
                                 dx, dy, dz, nr, nc, nz)
    return L, E


def rt_fsm2d(vp, Z, src, srcid, numofr, maxswp=500, dx=1.0, dz=1.0):
    vp = _c(vp, np.float64)
    nr, nc = vp.shape
    Z = _c(Z if numofr > 0 else np.zeros((1, 3)), np.float64)
    src = _c(src, np.int32)
    U = np.empty_like(vp)
    TTd = np.empty((max(numofr, 1), nr, nc))
    TTu = np.empty((max(numofr, 1), nr, nc))
    dummy = np.zeros(4, np.int32)
    _lib("2d").ref_rt_fsm2d(vp.ctypes.data, U.ctypes.data, TTd.ctypes.data, TTu.ctypes.data, Z.ctypes.data,
                            src.ctypes.data, dummy.ctypes.data, dummy.ctypes.data, srcid, numofr, maxswp, dx, dz,
                            nr, nc)
    return U, TTd[:numofr], TTu[:numofr]


def tadjoint2d(T, Tobs, rec, nxy, src, srnum, srcid, maxswp=500, dx=1.0, dz=1.0):
    T = _c(T, np.float64)
    nr, nc = T.shape
    a = [_c(Tobs, np.float64), _c(rec, np.int32), _c(nxy, np.float64), _c(src, np.int32), _c(srnum, np.int32)]
    L = np.empty_like(T)
    E = _lib("2d").ref_tadjoint2d(L.ctypes.data, T.ctypes.data, *[x.ctypes.data for x in a], srcid, maxswp,
                                  dx, dz, nr, nc)
    return L, E


def radjoint2d(Td, Tu, TRobs, rec, nxy, src, srnum, srcid, numofr, maxswp=500, dx=1.0, dz=1.0):
    Td, Tu = _c(Td, np.float64), _c(Tu, np.float64)
    nr, nc = Tu.shape[1:]
    a = [_c(TRobs, np.float64), _c(rec, np.int32), _c(nxy, np.float64), _c(src, np.int32), _c(srnum, np.int32)]
    UR = np.empty((nr, nc))
    E = _lib("2d").ref_radjoint2d(UR.ctypes.data, Td.ctypes.data, Tu.ctypes.data, *[x.ctypes.data for x in a],
                                  srcid, numofr, maxswp, dx, dz, nr, nc)
    return UR, E

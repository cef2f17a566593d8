"""ctypes wrapper of the oracle restatement (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: the checker that the CUDA library is compared with.
Array conventions follow the reference (see oracle/pfast_oracle.cpp): fields are
float64 in row-major reference layout; 3D src/rec are int32 [n, 3] (row, col, z),
2D src/rec are int32 [n, 2] (row, col) and 2D normals [n, 2] (n_z, n_x).
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None

_d = C.c_double
_i = C.c_int
_p = C.c_void_p


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            from . import build_oracle
            build_oracle.build()
        L = C.CDLL(path)
        L.oracle_fsm3d.restype = _i
        L.oracle_fsm3d.argtypes = [_p, _p, _p, _i, _i, _d, _d, _d, _i, _i, _i]
        L.oracle_adjoint3d.restype = _d
        L.oracle_adjoint3d.argtypes = [_p, _p, _p, _p, _p, _p, _p, _i, _i, _d, _d, _d, _i, _i, _i, _p]
        L.oracle_eval3d.restype = _i
        L.oracle_eval3d.argtypes = [_p, _p, _p, _p, _p, _p, _i, _i, _i, _d, _d, _d, _i, _i, _i,
                                    _p, _p, _i, _p, _p]
        L.oracle_forward3d.restype = _i
        L.oracle_forward3d.argtypes = [_p, _p, _p, _p, _i, _i, _i, _d, _d, _d, _i, _i, _i, _p, _i]
        L.oracle_rt_fsm2d.restype = _i
        L.oracle_rt_fsm2d.argtypes = [_p, _p, _p, _p, _p, _p, _i, _i, _i, _d, _d, _i, _i, _p]
        L.oracle_tadjoint2d.restype = _d
        L.oracle_tadjoint2d.argtypes = [_p, _p, _p, _p, _p, _p, _p, _i, _i, _d, _d, _i, _i, _p]
        L.oracle_radjoint2d.restype = _d
        L.oracle_radjoint2d.argtypes = [_p, _p, _p, _p, _p, _p, _p, _i, _i, _i, _d, _d, _i, _i, _p]
        L.oracle_forward2d.restype = _i
        L.oracle_forward2d.argtypes = [_p, _p, _p, _p, _p, _i, _i, _i, _i, _d, _d, _i, _i, _p, _i]
        L.oracle_eval2d.restype = _i
        L.oracle_eval2d.argtypes = [_p, _p, _p, _p, _p, _p, _p, _p, _p, _i, _i, _i, _i, _d, _d, _i, _i,
                                    _p, _p, _p, _p, _p, _i]
        _lib = L
    return _lib


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a):
    return None if a is None else a.ctypes.data


# ------------------------------------------------------------------ 3D
def fsm3d(vp, src, srcid, maxswp=100, dx=1.0, dy=1.0, dz=1.0):
    """fsm3d (src/T_pfsm3d.h:131).  vp: [nz, nrows, ncols].  Returns (U, iterations)."""
    vp = _f64(vp)
    nz, nr, nc = vp.shape
    src = _i32(src)
    U = np.empty_like(vp)
    it = lib().oracle_fsm3d(_ptr(vp), _ptr(U), _ptr(src), srcid, maxswp, dx, dy, dz, nr, nc, nz)
    return U, it


def adjoint3d(T, Tobs, rec, nxyz, src, srnum, srcid, maxswp=100, dx=1.0, dy=1.0, dz=1.0):
    """adjoint_fsm3d (src/T_padjoint3d.h:73).  Returns (lambda, EE, iterations)."""
    T = _f64(T)
    nz, nr, nc = T.shape
    Tobs, nxyz = _f64(Tobs), _f64(nxyz)
    rec, src, srnum = _i32(rec), _i32(src), _i32(srnum)
    L = np.empty_like(T)
    it = C.c_int(0)
    E = lib().oracle_adjoint3d(_ptr(L), _ptr(T), _ptr(Tobs), _ptr(rec), _ptr(nxyz), _ptr(src),
                               _ptr(srnum), srcid, maxswp, dx, dy, dz, nr, nc, nz, C.addressof(it))
    return L, E, it.value


def eval3d(vp, src, srnum, rec, nxyz, Tobs, maxswp=100, dx=1.0, dy=1.0, dz=1.0, s_begin=0, s_end=None,
           nthreads=1):
    """Misfit + gradient over sources [s_begin, s_end) (src/T_PFAST3D.cpp:387-399, np=1).
    Returns (grad, misfit, fwd_iters, adj_iters)."""
    vp = _f64(vp)
    nz, nr, nc = vp.shape
    src, srnum, rec = _i32(src), _i32(srnum), _i32(rec)
    nxyz, Tobs = _f64(nxyz), _f64(Tobs)
    if s_end is None:
        s_end = len(srnum)
    g = np.empty_like(vp)
    E = C.c_double(0)
    fi = np.zeros(s_end - s_begin, np.int32)
    ai = np.zeros(s_end - s_begin, np.int32)
    lib().oracle_eval3d(_ptr(vp), _ptr(src), _ptr(srnum), _ptr(rec), _ptr(nxyz), _ptr(Tobs), s_begin,
                        s_end, maxswp, dx, dy, dz, nr, nc, nz, _ptr(g), C.addressof(E), nthreads,
                        _ptr(fi), _ptr(ai))
    return g, E.value, fi, ai


def forward3d(vp, src, srnum, rec, maxswp=100, dx=1.0, dy=1.0, dz=1.0, s_begin=0, s_end=None, nthreads=1):
    """Picks T_s[rec] for the receiver rows of sources [s_begin, s_end)."""
    vp = _f64(vp)
    nz, nr, nc = vp.shape
    src, srnum, rec = _i32(src), _i32(srnum), _i32(rec)
    if s_end is None:
        s_end = len(srnum)
    out = np.empty(int(srnum[s_begin:s_end].sum()), np.float64)
    lib().oracle_forward3d(_ptr(vp), _ptr(src), _ptr(srnum), _ptr(rec), s_begin, s_end, maxswp, dx, dy, dz,
                           nr, nc, nz, _ptr(out), nthreads)
    return out


# ------------------------------------------------------------------ 2D
def rt_fsm2d(vp, Z, src, srcid, numofr, maxswp=500, dx=1.0, dz=1.0):
    """RT_fsm2d (src/RT_pfsm2d.h:116).  vp: [nrows, ncols]; Z: [numofr*ncols, 3].
    Returns (U, TTd, TTu, status, iters[2*numofr+1])."""
    vp = _f64(vp)
    nr, nc = vp.shape
    Z = _f64(Z) if numofr > 0 else np.zeros((1, 3))
    src = _i32(src)
    U = np.empty_like(vp)
    TTd = np.empty((max(numofr, 1), nr, nc))
    TTu = np.empty((max(numofr, 1), nr, nc))
    its = np.zeros(2 * numofr + 1, np.int32)
    st = lib().oracle_rt_fsm2d(_ptr(vp), _ptr(U), _ptr(TTd), _ptr(TTu), _ptr(Z), _ptr(src), srcid, numofr,
                               maxswp, dx, dz, nr, nc, _ptr(its))
    return U, TTd[:numofr], TTu[:numofr], st, its


def tadjoint2d(T, Tobs, rec, nxy, src, srnum, srcid, maxswp=500, dx=1.0, dz=1.0):
    """Tadjoint_fsm2d, Cr=1 (src/RT_padjoint2d.h:288).  Returns (lambda, EE, iterations)."""
    T = _f64(T)
    nr, nc = T.shape
    L = np.empty_like(T)
    it = C.c_int(0)
    Tobs, nxy = _f64(Tobs), _f64(nxy)
    rec, src, srnum = _i32(rec), _i32(src), _i32(srnum)
    E = lib().oracle_tadjoint2d(_ptr(L), _ptr(T), _ptr(Tobs), _ptr(rec), _ptr(nxy), _ptr(src), _ptr(srnum),
                                srcid, maxswp, dx, dz, nr, nc, C.addressof(it))
    return L, E, it.value


def radjoint2d(Tu, TRobs, rec, nxy, src, srnum, srcid, numofr, maxswp=500, dx=1.0, dz=1.0):
    """Radjoint_fsm2d, Cr=1 (src/RT_padjoint2d.h:382).  TRobs: [Nrec, numofr].
    Returns (lambda_R, EE, iters[numofr])."""
    Tu = _f64(Tu)
    nr, nc = Tu.shape[1:]
    UR = np.empty((nr, nc))
    its = np.zeros(max(numofr, 1), np.int32)
    TRobs, nxy = _f64(TRobs), _f64(nxy)
    rec, src, srnum = _i32(rec), _i32(src), _i32(srnum)
    E = lib().oracle_radjoint2d(_ptr(UR), _ptr(Tu), _ptr(TRobs), _ptr(rec), _ptr(nxy), _ptr(src), _ptr(srnum),
                                srcid, numofr, maxswp, dx, dz, nr, nc, _ptr(its))
    return UR, E, its[:numofr]


def forward2d(vp, Z, src, srnum, rec, numofr, maxswp=500, dx=1.0, dz=1.0, s_begin=0, s_end=None, nthreads=1):
    """2D picks [rows, numofr+1] for sources [s_begin, s_end) (src/RT_PFAST2D.cpp:832-852).
    Returns (Tr, status)."""
    vp = _f64(vp)
    nr, nc = vp.shape
    Z = _f64(Z) if numofr > 0 else np.zeros((1, 3))
    src, srnum, rec = _i32(src), _i32(srnum), _i32(rec)
    if s_end is None:
        s_end = len(srnum)
    Tr = np.empty((int(srnum[s_begin:s_end].sum()), numofr + 1))
    st = lib().oracle_forward2d(_ptr(vp), _ptr(Z), _ptr(src), _ptr(srnum), _ptr(rec), s_begin, s_end, numofr,
                                maxswp, dx, dz, nr, nc, _ptr(Tr), nthreads)
    return Tr, st


def eval2d(vp, WR, Z, src, srnum, rec, nxy, TTobs, TRobs, numofr, maxswp=500, dx=1.0, dz=1.0,
           s_begin=0, s_end=None, nthreads=1):
    """2D joint gradient (src/RT_PFAST2D.cpp:420-436, np=1).
    Returns dict(gT, gR, gRT, Et, Er, status)."""
    vp, WR = _f64(vp), _f64(WR)
    nr, nc = vp.shape
    Z = _f64(Z) if numofr > 0 else np.zeros((1, 3))
    TRobs = _f64(TRobs) if numofr > 0 else np.zeros((1,))
    src, srnum, rec = _i32(src), _i32(srnum), _i32(rec)
    nxy, TTobs = _f64(nxy), _f64(TTobs)
    if s_end is None:
        s_end = len(srnum)
    gT, gR, gRT = (np.empty_like(vp) for _ in range(3))
    Et, Er = C.c_double(0), C.c_double(0)
    st = lib().oracle_eval2d(_ptr(vp), _ptr(WR), _ptr(Z), _ptr(src), _ptr(srnum), _ptr(rec), _ptr(nxy),
                             _ptr(TTobs), _ptr(TRobs), s_begin, s_end, numofr, maxswp, dx, dz, nr, nc,
                             _ptr(gT), _ptr(gR), _ptr(gRT), C.addressof(Et), C.addressof(Er), nthreads)
    return dict(gT=gT, gR=gR, gRT=gRT, Et=Et.value, Er=Er.value, status=st)

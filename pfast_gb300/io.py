"""Reference file formats: raw little-endian float64 arrays (.vp, .src, .rec, .ref,
.wr, outputs) and the positional .inp parameter files.

readmod / writemod follow src/T_pfsm3d.h:39-57 and src/RT_pfsm2d.h; the .inp
layout follows src/RT_PFAST2D.cpp:137-172 and src/T_PFAST3D.cpp:105-134 (every
line not starting with '#' is a parameter line, read by position); metres are
converted to node indices with ceil(x/h)-1 (src/T_PFAST3D.cpp:250-252,
src/RT_PFAST2D.cpp:300-301).
"""
import math

import numpy as np


def readmod(path, count):
    a = np.fromfile(path, dtype="<f8", count=count)
    if a.size != count:
        raise ValueError(f"{path}: expected {count} doubles, found {a.size}")
    return a


def writemod(path, arr):
    np.ascontiguousarray(arr, dtype="<f8").tofile(path)


def _param_lines(path):
    out = []
    with open(path) as f:
        for line in f:
            if not line.startswith("#"):
                out.append(line.strip())
    return out


def parse_inp2d(path):
    """RT_PFAST2D .inp (src/RT_PFAST2D.cpp:148-172)."""
    L = _param_lines(path)
    f = lambda i: L[i].split()
    p = dict(vp=f(0)[0], src=f(1)[0], sNX=int(f(2)[0]), sNY=int(f(2)[1]), rec=f(3)[0], rNX=int(f(4)[0]),
             rNY=int(f(4)[1]), ref=f(5)[0], gmNX=int(f(6)[0]), gmNY=int(f(6)[1]), NX=int(float(f(7)[0])),
             NY=int(float(f(7)[1])), dx=float(f(7)[2]), dz=float(f(7)[3]), out_vp=f(8)[0])
    if len(L) > 9:
        p.update(nux=float(f(9)[0]), nuz=float(f(9)[1]))
    if len(L) > 10:
        p["wr"] = f(10)[0]
    if len(L) > 11:
        p.update(schemetag=int(f(11)[0]), lsrc=int(f(11)[1]))
    p["NumofR"] = int(math.ceil(p["gmNX"] / p["NY"]))   # src/RT_PFAST2D.cpp:230
    return p


def parse_inp3d(path):
    """T_PFAST3D .inp (src/T_PFAST3D.cpp:116-134)."""
    L = _param_lines(path)
    f = lambda i: L[i].split()
    p = dict(vp=f(0)[0], src=f(1)[0], sNX=int(f(2)[0]), sNY=int(f(2)[1]), rec=f(3)[0], rNX=int(f(4)[0]),
             rNY=int(f(4)[1]), NX=int(float(f(5)[0])), NY=int(float(f(5)[1])), NZ=int(float(f(5)[2])),
             dx=float(f(5)[3]), dy=float(f(5)[4]), dz=float(f(5)[5]), out_vp=f(6)[0])
    if len(L) > 7:
        p.update(nux=float(f(7)[0]), nuy=float(f(7)[1]), nuz=float(f(7)[2]))
    if len(L) > 8:
        p.update(schemetag=int(f(8)[0]), lsrc=int(f(8)[1]))
    return p


def to_index(metres, h):
    """(int)ceil(x/h)-1, elementwise."""
    return (np.ceil(np.asarray(metres, np.float64) / h) - 1).astype(np.int32)


def load_survey2d(src_arr, rec_arr, dx, dz, numofr):
    """Convert the 2D .src [nsrc,3] = (z, x, nrec) and .rec [nrec, 4+NumofR+...] = (z, x, n_z, n_x, TT, TR...)
    arrays to index form.  Returns src, srnum, rec, nxy, tt_obs, tr_obs (src/RT_PFAST2D.cpp:299-343)."""
    src = np.stack([to_index(src_arr[:, 0], dz), to_index(src_arr[:, 1], dx)], axis=1).astype(np.int32)
    srnum = src_arr[:, 2].astype(np.int32)
    rec = np.stack([to_index(rec_arr[:, 0], dz), to_index(rec_arr[:, 1], dx)], axis=1).astype(np.int32)
    nxy = np.ascontiguousarray(rec_arr[:, 2:4], np.float64)
    tt = rec_arr[:, 4].copy() if rec_arr.shape[1] > 4 else None
    tr = np.ascontiguousarray(rec_arr[:, 5:5 + numofr]) if rec_arr.shape[1] >= 5 + numofr and numofr else None
    return np.ascontiguousarray(src), srnum, np.ascontiguousarray(rec), nxy, tt, tr


def load_survey3d(src_arr, rec_arr, dx, dy, dz):
    """3D .src [nsrc,4] = (y, x, z, nrec) and .rec [nrec,7] = (y, x, z, n_y, n_x, n_z, T) to index form
    (src/T_PFAST3D.cpp:249-302).  Returns src, srnum, rec, nxyz, t_obs."""
    src = np.stack([to_index(src_arr[:, 0], dy), to_index(src_arr[:, 1], dx), to_index(src_arr[:, 2], dz)],
                   axis=1).astype(np.int32)
    srnum = np.ceil(src_arr[:, 3]).astype(np.int32)
    rec = np.stack([to_index(rec_arr[:, 0], dy), to_index(rec_arr[:, 1], dx), to_index(rec_arr[:, 2], dz)],
                   axis=1).astype(np.int32)
    nxyz = np.ascontiguousarray(rec_arr[:, 3:6], np.float64) if rec_arr.shape[1] >= 6 else None
    tobs = rec_arr[:, 6].copy() if rec_arr.shape[1] >= 7 else None
    return np.ascontiguousarray(src), srnum, np.ascontiguousarray(rec), nxyz, tobs

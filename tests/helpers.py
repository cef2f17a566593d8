"""Shared inputs of the parity tests (no CUDA calls here)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


def load_fw():
    z = np.load(os.path.join(GOLDEN, "rt2d_fw_golden.npz"))
    return {k: z[k] for k in z.files}


def load_inv():
    z = np.load(os.path.join(GOLDEN, "rt2d_inv_golden.npz"))
    return {k: z[k] for k in z.files}


def case3d(shape, h, seed, nsrc_extra=0):
    """Small 3D survey: random model, 3 sources (interior + two corners), receivers on k=0
    every 2nd row / 3rd column, noisy picks, one unpicked row per source (same recipe as
    tests/golden/make_golden.py)."""
    rng = np.random.default_rng(seed)
    nz, nr, nc = shape
    vp = 1500.0 + 2000.0 * rng.random((nz, nr, nc))
    src = np.array([[nr // 2, nc // 3, nz // 3], [0, 0, 0], [nr - 1, nc - 1, nz - 1]], np.int32)
    r1 = np.array([(i, j, 0) for i in range(0, nr, 2) for j in range(0, nc, 3)], np.int32)
    rec = np.concatenate([r1, r1, r1])
    srnum = np.full(3, len(r1), np.int32)
    nxyz = np.tile([0.0, 0.0, -1.0], (len(rec), 1))
    noise = 0.002 * (rng.random(len(rec)) - 0.5)
    return vp, src, srnum, rec, nxyz, noise


def picks_from(Ts, src, srnum, rec, noise, unpicked_offset=3):
    """Observed picks per source from that source's traveltime field Ts[s]."""
    ch0 = np.concatenate([[0], np.cumsum(srnum)])
    tobs = np.zeros(len(rec))
    for s in range(len(srnum)):
        rows = np.arange(ch0[s], ch0[s + 1])
        U = Ts[s]
        tobs[rows] = U[rec[rows, 2], rec[rows, 0], rec[rows, 1]] + noise[rows]
        if len(rows) > unpicked_offset:
            tobs[rows[unpicked_offset]] = 1000.0
    return tobs


def load_trace():
    """Noisy picks of all 56 sources of the shipped inversion case and the reference's
    printed iteration lines (tests/golden/rt2d_inv_trace.npz)."""
    z = np.load(os.path.join(GOLDEN, "rt2d_inv_trace.npz"))
    return {k: z[k] for k in z.files}

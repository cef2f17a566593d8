"""Seeded synthetic surveys in the shapes of the benchmark workloads.

The reference ships no data for these workloads; everything here is generated
from a seed (numpy PCG64).  Index conventions are the reference's: 3D src/rec
rows are (row, col, z), 2D rows (row, col); a node at index i sits at (i+1)*h
(the drivers convert metres with ceil(x/h)-1).
"""
import numpy as np


def _rng(seed):
    return np.random.default_rng(seed)


# ------------------------------------------------------------------ 3D
def gradient_model3d(nz, nrows, ncols, h, v0=2000.0, grad=0.6):
    """1D gradient model v = v0 + grad*z, z = (k+1)*h (the starting model of the 3D workload)."""
    z = (np.arange(nz, dtype=np.float64) + 1.0) * h
    v = v0 + grad * z
    return np.ascontiguousarray(np.broadcast_to(v[:, None, None], (nz, nrows, ncols)))


def random_field3d(shape, h, corr_len, seed):
    """White noise Gaussian-filtered to `corr_len` metres, normalised to unit std."""
    from scipy.ndimage import gaussian_filter
    r = _rng(seed).standard_normal(shape)
    r = gaussian_filter(r, sigma=corr_len / h, mode="reflect")
    r -= r.mean()
    r /= r.std()
    return r


def true_model3d(nz, nrows, ncols, h, seed, amp=0.05, corr_len=200.0):
    """vp = (2000 + 0.6 z)(1 + amp*r), r = filtered noise with `corr_len` correlation length."""
    return gradient_model3d(nz, nrows, ncols, h) * (1.0 + amp * random_field3d((nz, nrows, ncols), h, corr_len, seed))


def surface_survey3d(nrows, ncols, n_src_side, n_rec_side):
    """Sources on an n_src_side^2 surface grid, receivers on an n_rec_side^2 surface grid (k = 0);
    every source records every receiver; normals (n_y, n_x, n_z) = (0, 0, -1).
    Returns src [nsrc,3], srnum [nsrc], rec [nsrc*nrec,3], nxyz [nsrc*nrec,3]."""
    si = (np.arange(n_src_side) * nrows) // n_src_side + nrows // (2 * n_src_side)
    sj = (np.arange(n_src_side) * ncols) // n_src_side + ncols // (2 * n_src_side)
    ri = (np.arange(n_rec_side) * nrows) // n_rec_side + nrows // (2 * n_rec_side)
    rj = (np.arange(n_rec_side) * ncols) // n_rec_side + ncols // (2 * n_rec_side)
    src = np.array([(i, j, 0) for i in si for j in sj], np.int32)
    rec1 = np.array([(i, j, 0) for i in ri for j in rj], np.int32)
    nsrc, nrec = len(src), len(rec1)
    rec = np.ascontiguousarray(np.tile(rec1, (nsrc, 1)))
    nxyz = np.ascontiguousarray(np.tile(np.array([[0.0, 0.0, -1.0]]), (nsrc * nrec, 1)))
    srnum = np.full(nsrc, nrec, np.int32)
    return src, srnum, rec, nxyz


def random_small3d(shape, seed, vmin=1500.0, vmax=3500.0):
    """Uniform random model (bit-reproducible on every platform: no transcendental functions)."""
    return vmin + (vmax - vmin) * _rng(seed).random(shape)


def add_noise(picks, sigma, seed):
    return picks + _rng(seed).normal(0.0, sigma, picks.shape)


# ------------------------------------------------------------------ 2D
def first_arrival2d_model(nrows=101, ncols=301, h=10.0, seed=11):
    """2D first-arrival workload: vp = 1500 + 0.8 z plus a +15% and a -15% Gaussian anomaly
    (sigma = 150 m) at seeded positions."""
    rng = _rng(seed)
    z = (np.arange(nrows) + 1.0) * h
    x = (np.arange(ncols) + 1.0) * h
    Zg, Xg = np.meshgrid(z, x, indexing="ij")
    vp = 1500.0 + 0.8 * Zg
    for amp in (0.15, -0.15):
        cz = rng.uniform(0.25, 0.75) * nrows * h
        cx = rng.uniform(0.2, 0.8) * ncols * h
        vp = vp * (1.0 + amp * np.exp(-((Zg - cz) ** 2 + (Xg - cx) ** 2) / (2 * 150.0 ** 2)))
    return np.ascontiguousarray(vp)


def surface_survey2d(nrows, ncols, src_cols, rec_cols):
    """Sources and receivers on the surface row 0; every source records every receiver;
    normals (n_z, n_x) = (-1, 0).  Returns src [nsrc,2], srnum, rec [nsrc*nrec,2], nxy."""
    src = np.array([(0, j) for j in src_cols], np.int32)
    rec1 = np.array([(0, j) for j in rec_cols], np.int32)
    rec = np.ascontiguousarray(np.tile(rec1, (len(src), 1)))
    nxy = np.ascontiguousarray(np.tile(np.array([[-1.0, 0.0]]), (len(rec), 1)))
    srnum = np.full(len(src), len(rec1), np.int32)
    return src, srnum, rec, nxy


def joint2d_models(nrows=201, ncols=601, h=5.0, seed=12):
    """2D joint-inversion workload: true model (linear 1800->4000 m/s with depth plus three
    elliptical -20% lenses with 60-200 m semi-axes), starting model (the linear trend), and the
    reflector table Z [ncols, 3] = (depth, n_z, n_x) for z(x) = 600 + 40 sin(2 pi x / 1200) + N(0, 5^2)."""
    rng = _rng(seed)
    z = (np.arange(nrows) + 1.0) * h
    x = (np.arange(ncols) + 1.0) * h
    Zg, Xg = np.meshgrid(z, x, indexing="ij")
    v0 = 1800.0 + (4000.0 - 1800.0) * (Zg - z[0]) / (z[-1] - z[0])
    vt = v0.copy()
    for _ in range(3):
        cz = rng.uniform(0.15, 0.5) * nrows * h
        cx = rng.uniform(0.15, 0.85) * ncols * h
        az, ax = rng.uniform(60, 200, 2)
        inside = ((Zg - cz) / az) ** 2 + ((Xg - cx) / ax) ** 2 <= 1.0
        vt[inside] *= 0.8
    depth = 600.0 + 40.0 * np.sin(2 * np.pi * x / 1200.0) + rng.normal(0.0, 5.0, ncols)
    slope = np.gradient(depth, h)
    nrm = np.sqrt(1.0 + slope ** 2)
    Z = np.stack([depth, -1.0 / nrm, slope / nrm], axis=1)   # unit normal pointing up (toward the sources)
    return np.ascontiguousarray(vt), np.ascontiguousarray(v0), np.ascontiguousarray(Z)

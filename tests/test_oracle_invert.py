"""The oracle's inversion loop (oracle/invert.py) pinned to the reference's printed traces,
and host-side pieces of the inversion API.  CPU only.

The reference's 2D example was run three times (par/RT_SynMod2D_Inv_{RT,Trans,Ref}.out:
RTtag 3 joint, 1 transmission, 2 reflection; L-BFGS with LM = 50, secant strong-Wolfe line
search, nux = 60, nuz = 20, WR = 0.5).  The oracle, started from the same model and picks,
must print the same lines (6 significant digits).  The full 4-iteration traces are checked
against the GPU loop in test_gpu_invert.py; here the oracle runs the first iterations.
"""
import numpy as np
import pytest

from helpers import load_fw, load_inv, load_trace


def _lines(rep, nrec):
    ms = lambda e: 1000 * np.sqrt(2 * e / nrec)
    out = ["Average Time Residual (TR): %g ms\t(T): %g ms\t(R): %g ms" % (ms(rep["E"]), ms(rep["Et"]), ms(rep["Er"]))]
    out += ["(alpha0,alpha1,phi0,phi1,dphi0,dphi1)=(%g %g %g %g %g %g" % tuple(t) for t in rep["trials"]]
    return out


@pytest.mark.parametrize("rttag,iters", [(3, 2), (1, 1), (2, 1)])
def test_oracle_loop_prints_the_reference_trace(rttag, iters):
    from oracle import invert
    fw, inv, tr = load_fw(), load_inv(), load_trace()
    rec = fw["rec"].astype(np.int32)
    L = invert.loop2d(inv["vp"], np.full(inv["vp"].size, 0.5), fw["Z"], fw["src"], fw["srnum"], rec, tr["nxy"],
                      tr["tt"], tr["tr"], 2, float(fw["dx"]), float(fw["dz"]), float(tr["nux"]), float(tr["nuz"]),
                      rttag=rttag, LM=int(tr["LM"]), nthreads=8)
    got = []
    for _ in range(iters):
        got += _lines(L.step(), len(rec))
    want = [str(s) for s in tr[f"log_rttag{rttag}"]]
    assert got == want[:len(got)]


def test_regu_matches_a_direct_dft():
    """regu on a small odd/even grid equals the filter applied through an explicit DFT matrix,
    with the reference's swapped wavenumber vector (odd sizes keep its half-sample offset)."""
    from oracle import invert
    rng = np.random.default_rng(3)
    nr, nc, dx, dz, nux, nuz = 5, 6, 12.5, 8.0, 30.0, 10.0
    D = rng.standard_normal((nr, nc))
    vp = np.full((nr, nc), 2000.0)
    vp[0, 1] = 330.0
    Fr = np.exp(-2j * np.pi * np.outer(np.arange(nr), np.arange(nr)) / nr)
    Fc = np.exp(-2j * np.pi * np.outer(np.arange(nc), np.arange(nc)) / nc)
    F = Fr @ D @ Fc.T
    kx, kz = invert._kvec(nc, dx), invert._kvec(nr, dz)
    F = F / (1 + nux * nux * kx[None, :] ** 2 + nuz * nuz * kz[:, None] ** 2)
    R = (np.conj(Fr) @ F @ np.conj(Fc).T).real / (nr * nc)
    R[0, 1] = 0.0
    got = invert.regu(D, vp, (nux, nuz), (dx, dz))
    assert np.allclose(got, R, rtol=1e-12, atol=1e-14)
    # even sizes: the swapped vector is the usual FFT frequency order
    k = invert._kvec(8, 2.0)
    assert np.allclose(k, 2 * np.pi * np.fft.fftfreq(8, 2.0))


def test_cubic_interp_branches():
    from oracle import invert
    # a cubic with a minimiser between the points
    a = invert.cubic_interp(0.0, 1.0, 1.0, 0.5, -1.0, 0.2)
    assert 0.0 < a < 1.0
    with pytest.raises(RuntimeError):
        invert.cubic_interp(0.0, 1.0, 0.0, 0.0, 0.0, 0.0)


def test_lbfgs_two_loop_with_one_pair_is_the_bfgs_update():
    """With one stored pair the two-loop recursion equals H g for the BFGS inverse-Hessian
    update of gamma*I (the quantity src/RT_PFAST2D.cpp:520-546 computes)."""
    from oracle import invert
    rng = np.random.default_rng(5)
    n = 7
    g0, g1, d0 = rng.standard_normal((3, n))
    L = invert.Loop(np.ones(n), None, (1.0,), (1.0,), 2, LM=3)
    L.it, L.alpha1, L.dk, L.Djk1 = 2, 0.7, d0.copy(), g1.copy()
    d = L._lbfgs(g0)
    s, y = 0.7 * d0, -g1 + g0
    rho, gamma = 1 / (s @ y), (s @ y) / (y @ y)
    V = np.eye(n) - rho * np.outer(y, s)
    H = V.T @ (gamma * np.eye(n)) @ V + rho * np.outer(s, s)
    assert np.allclose(d, H @ g1, rtol=1e-12)


def test_invert_default_options_are_the_drivers():
    from pfast_gb300 import api
    o2, o3 = api.invert_options(2), api.invert_options(3)
    assert (o2.schemetag, o2.lsrc, o2.LM, o2.max_linesearch, o2.rttag) == (3, 2, 5, 5, 3)
    assert (o2.minv, o2.maxv, o2.conv_tol, o2.eval.maxswp) == (1600.0, 4500.0, 1e-3, 500)
    assert (o3.max_linesearch, o3.minv, o3.maxv, o3.conv_tol, o3.eval.maxswp) == (2, 1400.0, 8000.0, 1e-2, 100)
    o = api.invert_options(2, LM=50, nux=60.0, precision=1)
    assert (o.LM, o.nux, o.eval.precision) == (50, 60.0, 1)
    with pytest.raises(TypeError):
        api.invert_options(2, bogus=1)

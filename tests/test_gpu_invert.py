"""The inversion loop on the GPU (pfast_inversion*) through the C ABI.

* The reference's shipped 2D inversion (all 56 sources, 33600 traces, 2 reflectors,
  L-BFGS LM = 50, secant strong-Wolfe search), plain FP64 gradients: the lines the loop
  prints for iterations 1-4 must equal the reference's logs (par/RT_SynMod2D_Inv_*.out,
  committed in tests/golden/rt2d_inv_trace.npz) for RTtag 3, 1 and 2.
* Small 2D and 3D cases against the oracle loop (oracle/invert.py) for every search
  scheme and line search: misfits, line-search rows, step sizes and the final model within
  1e-9 relative (the FFT and the inner-product order differ from the oracle's by rounding).
"""
import numpy as np
import pytest

from helpers import load_fw, load_inv, load_trace

pytestmark = pytest.mark.gpu


def _pg():
    import pfast_gb300 as pg
    return pg


def _lines(rep, nrec):
    ms = lambda e: 1000 * np.sqrt(2 * e / nrec)
    out = ["Average Time Residual (TR): %g ms\t(T): %g ms\t(R): %g ms" % (ms(rep["E"]), ms(rep["Et"]), ms(rep["Er"]))]
    out += ["(alpha0,alpha1,phi0,phi1,dphi0,dphi1)=(%g %g %g %g %g %g" % tuple(t) for t in rep["trials"]]
    return out


def _full_survey(ctx):
    pg = _pg()
    fw, tr = load_fw(), load_trace()
    return pg.Survey2D(ctx, 160, 600, float(fw["dx"]), float(fw["dz"]), fw["src"], fw["srnum"],
                       fw["rec"].astype(np.int32), numofr=2, Z=fw["Z"], nxy=tr["nxy"], tt_obs=tr["tt"],
                       tr_obs=tr["tr"])


@pytest.mark.parametrize("rttag", [3, 1, 2])
def test_shipped_inversion_prints_the_reference_trace(ctx, rttag):
    pg = _pg()
    tr = load_trace()
    sv = _full_survey(ctx)
    inv = pg.Inversion(sv, load_inv()["vp"], WR=0.5, LM=int(tr["LM"]), rttag=rttag, nux=float(tr["nux"]),
                       nuz=float(tr["nuz"]))
    got = []
    for _ in range(int(tr["iters"])):
        got += _lines(inv.step(), 33600)
    assert got == [str(s) for s in tr[f"log_rttag{rttag}"]]
    vp, vp0 = inv.get("vp"), load_inv()["vp"]
    water = np.abs(vp0 - 330) < 1e-9
    assert np.array_equal(vp[water], vp0[water])          # updatevp leaves water alone
    assert vp[~water].min() >= 1600.0 and vp[~water].max() <= 4500.0
    inv.close()
    sv.close()


def test_shipped_inversion_mixed_precision_tracks_the_trace(ctx):
    """FP32-bulk gradients: the first two iterations' misfits within 1e-4 of the printed ones."""
    pg = _pg()
    tr = load_trace()
    sv = _full_survey(ctx)
    inv = pg.Inversion(sv, load_inv()["vp"], WR=0.5, LM=int(tr["LM"]), nux=float(tr["nux"]), nuz=float(tr["nuz"]),
                       precision=pg.PFAST_MIXED)
    want = [float(s.split()[4]) for s in tr["log_rttag3"] if s.startswith("Average")]
    for k in range(2):
        r = inv.step()
        got = 1000 * np.sqrt(2 * r["E"] / 33600)
        assert abs(got - want[k]) <= 1e-4 * want[k], (k, got, want[k])
    inv.close()
    sv.close()


# ------------------------------------------------------------------ small cases vs the oracle
def _case2d():
    """50 x 120 grid, 2 reflectors, 3 sources, a patch of water (vp = 330) away from the sources;
    picks from a model with a slow anomaly, inversion from the background."""
    from oracle import port
    nr, nc, h = 50, 120, 10.0
    bg = 1700.0 + 30.0 * np.arange(nr)[:, None] + np.zeros((1, nc))
    ii, jj = np.meshgrid(np.arange(nr), np.arange(nc), indexing="ij")
    true = bg - 250.0 * np.exp(-((ii - 20) ** 2 + (jj - 60) ** 2) / 60.0)
    for v in (bg, true):
        v[0:2, 90:100] = 330.0
    Z = np.concatenate([np.stack([np.full(nc, 230.0 + 10 * np.sin(np.arange(nc) / 9.0)), -np.ones(nc),
                                  np.zeros(nc)], 1),
                        np.stack([np.full(nc, 420.0), -np.ones(nc), np.zeros(nc)], 1)])
    src = np.array([[0, 15], [0, 60], [0, 110]], np.int32)
    rec = np.array([(0, j) for j in range(0, nc, 2)] * 3, np.int32)
    srnum = np.full(3, nc // 2, np.int32)
    nxy = np.tile([-1.0, 0.0], (len(rec), 1))
    Tr, _ = port.forward2d(true, Z, src, srnum, rec, 2, 500, h, h)
    rng = np.random.default_rng(11)
    tt = Tr[:, 0] + rng.normal(0, 5e-4, len(rec))
    trr = Tr[:, 1:] + rng.normal(0, 5e-4, (len(rec), 2))
    WR = np.full((nr, nc), 0.4)
    return dict(vp=bg, Z=Z, src=src, srnum=srnum, rec=rec, nxy=nxy, tt=tt, tr=trr, WR=WR, h=h, nr=nr, nc=nc)


def _close(a, b, rtol):
    return abs(a - b) <= rtol * max(abs(a), abs(b), 1e-300)


def _compare(rg, ro, rtol=1e-9):
    for k in ("E", "Et", "Er", "alpha_start", "stepsize"):
        a, b = rg[k], ro.get(k)
        if b is None:
            continue
        assert _close(a, b, rtol), (k, a, b)
    assert rg["count"] == ro["count"] and bool(rg["stopped"]) == bool(ro["stopped"])
    assert bool(rg["converged"]) == bool(ro["converged"])
    assert len(rg["trials"]) == len(ro["trials"])
    for tg, to in zip(rg["trials"], ro["trials"]):
        for a, b in zip(tg[:4], to[:4]):
            assert _close(a, b, rtol) or abs(a - b) < 1e-300, (tg, to)
        # dphi = sum(-dk * Dj) cancels: compare on the scale of the larger directional derivative
        scale = max(abs(to[4]), abs(to[5]))
        assert abs(tg[4] - to[4]) <= rtol * scale and abs(tg[5] - to[5]) <= rtol * scale, (tg, to)


def _run_pair(inv, loop, iters, rtol=1e-9):
    """Step the GPU loop and the oracle loop together; both must stop the same way (check_conv's
    convergence, its "Over corrected" abort after the model update, or a cubic step without a
    minimiser)."""
    from oracle import invert as oinv
    pg = _pg()
    for _ in range(iters):
        err_o = err_g = None
        try:
            ro = loop.step()
        except oinv.OverCorrected:
            err_o = pg._capi.PFAST_ERR_OVER_CORRECTED
        except RuntimeError:
            err_o = pg._capi.PFAST_ERR_LINE_SEARCH
        try:
            rg = inv.step()
        except pg.PfastError as e:
            err_g = e.status
        assert err_g == err_o
        if err_o is not None:
            return
        _compare(rg, ro, rtol)
        if ro["converged"]:
            return


SCHEMES = [
    dict(schemetag=3, lsrc=2, LM=2, iters=5),     # L-BFGS with the pair ring wrapping (LM = 2)
    dict(schemetag=1, lsrc=2, LM=5, iters=3),     # HS
    dict(schemetag=2, lsrc=2, LM=5, iters=3),     # CG_DESCENT
    dict(schemetag=3, lsrc=3, LM=5, iters=3),     # cubic, strong-Wolfe loop
    dict(schemetag=1, lsrc=3, LM=5, iters=2),     # cubic, single interpolation
    dict(schemetag=3, lsrc=1, LM=5, iters=1),     # secant 'exact' (always ends at step 0, then 0/0 pairs)
    dict(schemetag=1, lsrc=0, LM=5, iters=2),     # no line search
]


@pytest.mark.parametrize("cfg", SCHEMES, ids=lambda c: f"scheme{c['schemetag']}_ls{c['lsrc']}")
@pytest.mark.parametrize("rttag", [3, 1])
def test_loop2d_matches_oracle(ctx, cfg, rttag):
    from oracle import invert as oinv
    pg = _pg()
    c = _case2d()
    kw = dict(schemetag=cfg["schemetag"], lsrc=cfg["lsrc"], LM=cfg["LM"], rttag=rttag)
    loop = oinv.loop2d(c["vp"], c["WR"], c["Z"], c["src"], c["srnum"], c["rec"], c["nxy"], c["tt"], c["tr"], 2,
                       c["h"], c["h"], 40.0, 15.0, nthreads=8, **kw)
    sv = pg.Survey2D(ctx, c["nr"], c["nc"], c["h"], c["h"], c["src"], c["srnum"], c["rec"], numofr=2, Z=c["Z"],
                     nxy=c["nxy"], tt_obs=c["tt"], tr_obs=c["tr"])
    inv = pg.Inversion(sv, c["vp"], WR=c["WR"], nux=40.0, nuz=15.0, keep_components=1, **kw)
    _run_pair(inv, loop, cfg["iters"])
    vg = inv.get("vp")
    assert np.allclose(vg, loop.vp, rtol=1e-8, atol=0), np.max(np.abs(vg - loop.vp))
    assert np.allclose(inv.get("direction"), loop.dk.reshape(vg.shape), rtol=1e-6,
                       atol=1e-8 * np.max(np.abs(loop.dk)))
    # water stays water; the raw and regularised components are readable
    assert np.all(vg[0:2, 90:100] == 330.0)
    for f in ("grad_raw", "grad", "gR_raw", "gR", "gT_raw", "gT"):
        assert np.isfinite(inv.get(f)).all()
    assert np.all(inv.get("grad")[0:2, 90:100] == 0.0)
    inv.close()
    sv.close()


def _case3d(nz=12, nr=16, nc=20, h=10.0):
    """Depth-gradient background with a slow Gaussian anomaly; 5 surface sources, receivers on
    every 2nd surface node; picks from the anomaly model with 2e-5 s noise."""
    from oracle import port
    k, i, j = np.meshgrid(np.arange(nz), np.arange(nr), np.arange(nc), indexing="ij")
    bg = 1800.0 + 60.0 * k
    true = bg - 600.0 * np.exp(-((k - 6) ** 2 + (i - 8) ** 2 + (j - 10) ** 2) / 8.0)
    src = np.array([[1, 1, 0], [1, nc - 2, 0], [nr - 2, 1, 0], [nr - 2, nc - 2, 0], [nr // 2, nc // 2, 0]], np.int32)
    r1 = np.array([(a, b, 0) for a in range(0, nr, 2) for b in range(0, nc, 2)], np.int32)
    rec = np.concatenate([r1] * len(src))
    srnum = np.full(len(src), len(r1), np.int32)
    nxyz = np.tile([0.0, 0.0, -1.0], (len(rec), 1))
    ch0 = np.concatenate([[0], np.cumsum(srnum)])
    tobs = np.zeros(len(rec))
    rng = np.random.default_rng(7)
    for s in range(len(src)):
        U = port.fsm3d(true, src, s, 100, h, h, h)[0]
        rows = np.arange(ch0[s], ch0[s + 1])
        tobs[rows] = U[rec[rows, 2], rec[rows, 0], rec[rows, 1]] + rng.normal(0, 2e-5, len(rows))
    return bg, src, srnum, rec, nxyz, tobs, (nz, nr, nc), h


@pytest.mark.parametrize("lsrc", [2, 3])
def test_loop3d_matches_oracle(ctx, lsrc):
    """T_PFAST3D's loop (L-BFGS, MAXLineSch 2) on a small survey: 3-4 iterations until check_conv
    stops it, the pair ring (LM = 2) in use from the third."""
    from oracle import invert as oinv
    pg = _pg()
    bg, src, srnum, rec, nxyz, tobs, (nz, nr, nc), h = _case3d()
    loop = oinv.loop3d(bg, src, srnum, rec, nxyz, tobs, h, h, h, 30.0, 30.0, 20.0, lsrc=lsrc, LM=2, nthreads=8)
    sv = pg.Survey3D(ctx, nr, nc, nz, h, h, h, src, srnum, rec, nxyz, tobs)
    inv = pg.Inversion(sv, bg, lsrc=lsrc, LM=2, nux=30.0, nuy=30.0, nuz=20.0)
    # The cubic step is built from phi1 - phi0; after the tiny third step here the two misfits
    # agree to 1e-5, so rounding of 1e-12 in each becomes ~1e-8 in the interpolated step.
    _run_pair(inv, loop, 6, rtol=1e-9 if lsrc == 2 else 1e-6)
    assert len(inv.history) == loop.it >= 3
    assert np.allclose(inv.get("vp"), loop.vp, rtol=1e-8, atol=0)
    inv.close()
    sv.close()


def test_invalid_options_are_rejected(ctx):
    pg = _pg()
    c = _case2d()
    sv = pg.Survey2D(ctx, c["nr"], c["nc"], c["h"], c["h"], c["src"], c["srnum"], c["rec"], numofr=2, Z=c["Z"],
                     nxy=c["nxy"], tt_obs=c["tt"], tr_obs=c["tr"])
    for bad in (dict(schemetag=4), dict(lsrc=7), dict(LM=0), dict(max_linesearch=17), dict(rttag=0)):
        with pytest.raises(pg.PfastError) as e:
            pg.Inversion(sv, c["vp"], WR=c["WR"], **bad)
        assert e.value.status == 1
    nopicks = pg.Survey2D(ctx, c["nr"], c["nc"], c["h"], c["h"], c["src"], c["srnum"], c["rec"], numofr=2, Z=c["Z"])
    with pytest.raises(pg.PfastError):
        pg.Inversion(nopicks, c["vp"], WR=c["WR"])
    sv.close()
    nopicks.close()

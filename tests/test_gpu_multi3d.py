"""Many 3D models in one evaluation (pfast_surveys3d_eval): every sweep phase of all the
(model, source) instances runs as one dataflow launch.  Each model's gradient and misfit must
equal its own evaluation bit for bit, in plain FP64 (which equals the oracle) and in the mixed
mode; a model without sources gives a zero gradient; a non-positive velocity is rejected."""
import numpy as np
import pytest

from helpers import bits_equal

pytestmark = pytest.mark.gpu

# (nz, nrows, ncols), spacings, sources
MODELS = [((9, 11, 13), (10.0, 10.0, 10.0), 3), ((22, 40, 100), (20.0, 20.0, 20.0), 5),
          ((13, 17, 70), (10.0, 12.5, 8.0), 2), ((5, 3, 33), (5.0, 7.0, 3.0), 1),
          ((16, 24, 64), (15.0, 15.0, 15.0), 4), ((8, 8, 8), (10.0, 10.0, 10.0), 0)]


def _surveys(ctx, seed=61):
    import torch
    import pfast_gb300 as pg
    rng = np.random.default_rng(seed)
    out = []
    for shape, h, ns in MODELS:
        nz, nr, nc = shape
        vp = 1500.0 + 2000.0 * rng.random(shape)
        src = np.stack([rng.integers(0, nr, ns), rng.integers(0, nc, ns), rng.integers(0, nz, ns)], 1).astype(np.int32)
        r1 = np.array([(i, j, 0) for i in range(0, nr, 2) for j in range(0, nc, 3)], np.int32)
        rec = np.concatenate([r1] * ns) if ns else np.zeros((0, 3), np.int32)
        srnum = np.full(ns, len(r1), np.int32)
        nxyz = np.tile([0.0, 0.0, -1.0], (len(rec), 1))
        tobs = 0.05 + 0.3 * rng.random(len(rec))
        if ns:
            tobs[2] = 1000.0   # one unpicked row
        sv = pg.Survey3D(ctx, nr, nc, nz, *h, src, srnum, rec, nxyz, tobs)
        out.append((sv, torch.from_numpy(vp).cuda()))
    return out


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_many_models_match_their_own_evaluations(ctx, precision):
    import pfast_gb300 as pg
    prec = pg.PFAST_PLAIN_FP64 if precision == "plain" else pg.PFAST_MIXED
    pairs = _surveys(ctx)
    svs, vps = [p[0] for p in pairs], [p[1] for p in pairs]
    grads, misfits, st = pg.eval3d_many(ctx, svs, vps, precision=prec)
    assert st["not_converged"] == 0
    launches_alone = 0
    for k, (sv, vp) in enumerate(pairs):
        if sv.nsrc == 0:
            assert misfits[k] == 0.0 and not grads[k].any()
            continue
        g, e, s1 = sv.eval(vp, precision=prec)
        launches_alone += s1["launches"]
        assert bits_equal(g.cpu().numpy(), grads[k].cpu().numpy()), k
        assert e == misfits[k], k
    # the sweeps of all models: four (mixed) or two (plain) dataflow launches
    assert st["launches"] < launches_alone
    for sv, _ in pairs:
        sv.close()


def test_many_models_reject_a_non_positive_velocity(ctx):
    import pfast_gb300 as pg
    pairs = _surveys(ctx, 62)
    vps = [p[1].clone() for p in pairs]
    vps[2][1, 2, 3] = -1.0
    with pytest.raises(pg.PfastError) as ei:
        pg.eval3d_many(ctx, [p[0] for p in pairs], vps, precision=pg.PFAST_MIXED)
    assert ei.value.status == pg._capi.PFAST_ERR_INVALID
    for sv, _ in pairs:
        sv.close()

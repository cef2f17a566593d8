"""2D joint transmission + reflection inversion benchmark (L-BFGS iterations per second).

    python -m pfast_gb300.inv_bench --iters 15

Workload: 601 x 201 grid (x by z), h = 5 m; true model linear 1800 -> 4000 m/s with depth
plus three seeded elliptical -20% lenses; one reflector z(x) = 600 + 40 sin(2 pi x / 1200)
plus seeded 5 m jitter; 40 surface sources, 400 surface receivers; first-arrival and
reflection picks from the plain FP64 solver on the true model plus 1 ms Gaussian noise;
inversion from the 1D linear model with the drivers' loop (L-BFGS, secant strong-Wolfe
line search, the reference's FFT regularisation with nux = 60, nuz = 20, WR = 0.5) for a
fixed number of iterations.  Runs the loop with mixed-precision and with plain FP64
gradients and reports iterations/s, gradient evaluations, misfits and the difference of
the two final models.
"""
import argparse
import json
import time

import numpy as np

from . import synth

H = 5.0


def workload(seed=12):
    vt, v0, Z = synth.joint2d_models(201, 601, H, seed=seed)
    nr, nc = vt.shape
    src_cols = np.round(np.linspace(7, nc - 8, 40)).astype(int)
    rec_cols = np.round(np.linspace(0, nc - 1, 400)).astype(int)
    src, srnum, rec, nxy = synth.surface_survey2d(nr, nc, src_cols, rec_cols)
    return vt, v0, Z, src, srnum, rec, nxy


def picks(ctx, vt, Z, src, srnum, rec, seed=3):
    import torch
    import pfast_gb300 as pg
    nr, nc = vt.shape
    sv = pg.Survey2D(ctx, nr, nc, H, H, src, srnum, rec, numofr=1, Z=Z)
    Tr, _ = sv.forward(torch.from_numpy(vt).cuda(), precision=pg.PFAST_PLAIN_FP64)
    sv.close()
    Tr = Tr.cpu().numpy()
    rng = np.random.default_rng(seed)
    return Tr[:, 0] + rng.normal(0.0, 0.001, len(rec)), Tr[:, 1:] + rng.normal(0.0, 0.001, (len(rec), 1))


def run(iters=15, LM=5):
    import pfast_gb300 as pg
    vt, v0, Z, src, srnum, rec, nxy = workload()
    ctx = pg.Context(0)
    tt, tr = picks(ctx, vt, Z, src, srnum, rec)
    nr, nc = vt.shape
    sv = pg.Survey2D(ctx, nr, nc, H, H, src, srnum, rec, numofr=1, Z=Z, nxy=nxy, tt_obs=tt, tr_obs=tr)
    out = {}
    models = {}
    for name, prec in (("mixed", pg.PFAST_MIXED), ("plain", pg.PFAST_PLAIN_FP64)):
        inv = pg.Inversion(sv, v0, WR=0.5, LM=LM, nux=60.0, nuz=20.0, precision=prec, conv_tol=-1.0)
        t0 = time.perf_counter()
        reps = [inv.step() for _ in range(iters)]
        wall = time.perf_counter() - t0
        models[name] = inv.get("vp")
        inv.close()
        out[name] = {"iters": iters, "wall_s": wall, "lbfgs_iters_per_s": iters / wall,
                     "gradient_evals": int(sum(r["evals"] for r in reps)),
                     "misfit_first": reps[0]["E"], "misfit_last": reps[-1]["E"],
                     "ms_per_iter_p50": float(np.median([r["ms_total"] for r in reps]))}
    sv.close()
    ctx.close()
    d = models["mixed"] - models["plain"]
    out["model_rel_l2_mixed_vs_plain"] = float(np.linalg.norm(d) / np.linalg.norm(models["plain"]))
    out["model_rel_l2_start_vs_true"] = float(np.linalg.norm(v0 - vt) / np.linalg.norm(vt))
    out["model_rel_l2_final_vs_true"] = float(np.linalg.norm(models["mixed"] - vt) / np.linalg.norm(vt))
    out["speedup"] = out["mixed"]["lbfgs_iters_per_s"] / out["plain"]["lbfgs_iters_per_s"]
    return out


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--iters", type=int, default=15)
    p.add_argument("--lm", type=int, default=5)
    a = p.parse_args()
    print(json.dumps(run(a.iters, a.lm)), flush=True)


if __name__ == "__main__":
    main()

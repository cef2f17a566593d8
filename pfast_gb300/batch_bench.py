"""Batched uneven 3D gradients: many independent models of different grid sizes evaluated
together on one GPU.

    python -m pfast_gb300.batch_bench --models 48 --slots 8

Instances: `models` models with node counts log-uniform between 64^3 and 224x224x112
(nrows = ncols = 2 nz, h = 20 m), velocity (2000 + 0.6 z)(1 + 0.05 r) with r the seeded
Gaussian-filtered noise field of the 3D gradient workload (cropped from one field at the
largest size), 4-128 surface sources each (uniform integer), receivers on every 4th surface
node, picks from the true model plus 2 ms noise; every instance evaluates misfit + gradient
on the 1D starting model once.

Batched: all models in one evaluation (pfast_surveys3d_eval): every sweep phase runs as one
dataflow launch over all (model, source) instances, largest grid first, each retiring as it
converges; in mixed precision and in plain FP64, so that the gains of batching and of precision
show separately.  Baseline: the same evaluations one model after another with the plain FP64
path.  Also the request-server path (`slots` models at a time on their own streams).  Reports
wall times, models/s, and the largest gradient difference between mixed and plain.
"""
import argparse
import json
import math
import time

import numpy as np

from . import synth

H = 20.0
NMIN, NMAX = 64 * 64 * 64, 224 * 224 * 112


def instances(n_models, seed=48):
    rng = np.random.default_rng(seed)
    field = synth.random_field3d((112, 224, 224), H, 200.0, seed)
    out = []
    for m in range(n_models):
        n = math.exp(rng.uniform(math.log(NMIN), math.log(NMAX)))
        nz = int(round((n / 4.0) ** (1.0 / 3.0)))
        nz = max(40, min(nz, 112))
        side = max(80, min(224, int(round(math.sqrt(n / nz)))))
        shape = (nz, side, side)
        true = synth.gradient_model3d(nz, side, side, H) * (1.0 + 0.05 * field[:nz, :side, :side])
        start = synth.gradient_model3d(nz, side, side, H)
        nsrc = int(rng.integers(4, 129))
        src = np.stack([rng.integers(0, side, nsrc), rng.integers(0, side, nsrc), np.zeros(nsrc, int)], 1).astype(np.int32)
        ri, rj = np.meshgrid(np.arange(0, side, 4), np.arange(0, side, 4), indexing="ij")
        rec1 = np.stack([ri.ravel(), rj.ravel(), np.zeros(ri.size, int)], 1).astype(np.int32)
        rec = np.ascontiguousarray(np.tile(rec1, (nsrc, 1)))
        srnum = np.full(nsrc, len(rec1), np.int32)
        nxyz = np.tile([0.0, 0.0, -1.0], (len(rec), 1))
        out.append(dict(shape=shape, true=np.ascontiguousarray(true), start=start, src=src, srnum=srnum, rec=rec,
                        nxyz=nxyz, seed=int(rng.integers(0, 2 ** 31))))
    return out


def observed(ctx, inst):
    """Picks on the true model (mixed precision) plus 2 ms noise."""
    import torch
    import pfast_gb300 as pg
    nz, nr, nc = inst["shape"]
    sv = pg.Survey3D(ctx, nr, nc, nz, H, H, H, inst["src"], inst["srnum"], inst["rec"])
    pk, _ = sv.forward(torch.from_numpy(inst["true"]).cuda(), precision=pg.PFAST_MIXED)
    sv.close()
    return synth.add_noise(pk.cpu().numpy(), 0.002, inst["seed"])


def run(n_models=48, slots=8, budget_gb=150.0, plain_models=None, server=True):
    """Batched (one dataflow launch per sweep phase over all models' sources, pfast_surveys3d_eval)
    in mixed precision and in plain FP64, the sequential per-model plain FP64 baseline, and the
    request-server path (slots models at a time on their own streams)."""
    import torch
    import pfast_gb300 as pg
    insts = instances(n_models)
    ctx = pg.Context(0)
    for inst in insts:
        inst["tobs"] = observed(ctx, inst)
    node_src = sum(int(np.prod(i["shape"])) * len(i["srnum"]) for i in insts)
    svs = [pg.Survey3D(ctx, i["shape"][1], i["shape"][2], i["shape"][0], H, H, H, i["src"], i["srnum"], i["rec"],
                       i["nxyz"], i["tobs"]) for i in insts]
    vps = [torch.from_numpy(i["start"]).cuda() for i in insts]
    out = {"models": n_models, "node_sources": node_src}

    def timed(fn):
        torch.cuda.synchronize()
        a = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - a

    # batched: all models in one evaluation (a warm-up call first: kernel attributes, buffers)
    pg.eval3d_many(ctx, svs[:2], vps[:2], precision=pg.PFAST_MIXED)
    (gm, em, stm), t_bm = timed(lambda: pg.eval3d_many(ctx, svs, vps, precision=pg.PFAST_MIXED))
    gm = [g.cpu().numpy() for g in gm]
    (gp, ep, stp), t_bp = timed(lambda: pg.eval3d_many(ctx, svs, vps, precision=pg.PFAST_PLAIN_FP64))
    gp = [g.cpu().numpy() for g in gp]
    out.update({"batched_mixed_s": t_bm, "batched_mixed_models_per_s": n_models / t_bm,
                "batched_mixed_launches": stm["launches"], "batched_mixed_not_converged": stm["not_converged"],
                "batched_plain_s": t_bp, "batched_plain_models_per_s": n_models / t_bp,
                "grad_rel_l2_max_mixed_vs_plain": max(float(np.linalg.norm(a - b) / np.linalg.norm(b))
                                                      for a, b in zip(gm, gp))})
    # sequential plain FP64, one model after another (direct survey API, inputs resident)
    m_plain = n_models if plain_models is None else min(plain_models, n_models)
    t_plain = 0.0
    max_diff = 0.0
    for k in range(m_plain):
        (g, e, _), t = timed(lambda: svs[k].eval(vps[k], precision=pg.PFAST_PLAIN_FP64))
        t_plain += t
        max_diff = max(max_diff, float(np.abs(g.cpu().numpy() - gp[k]).max()))
    plain_scaled = t_plain * n_models / m_plain
    out.update({"sequential_plain_s": plain_scaled, "sequential_plain_models_per_s": n_models / plain_scaled,
                "plain_sample_models": m_plain, "batched_plain_equals_sequential": max_diff == 0.0,
                "speedup_batched_mixed_vs_sequential_plain": plain_scaled / t_bm,
                "speedup_batching_plain": plain_scaled / t_bp, "speedup_precision_batched": t_bp / t_bm})
    for sv in svs:
        sv.close()
    if server:
        srv = pg.Server(slots=slots, hbm_budget_gb=budget_gb)
        for k, inst in enumerate(insts):
            srv.put_model(k, inst["start"], (H, H, H))
            srv.put_survey3d(k, inst["shape"], (H, H, H), inst["src"], inst["srnum"], inst["rec"], inst["nxyz"],
                             inst["tobs"])
        small = min(range(n_models), key=lambda k: np.prod(insts[k]["shape"]))
        srv.submit_gradient(small, small).result()
        t0 = time.perf_counter()
        tickets = [srv.submit_gradient(k, k, pg.PFAST_MIXED) for k in range(n_models)]
        for t in tickets:
            t.result()
        out["server_mixed_s"] = time.perf_counter() - t0
        out["server_slots"] = slots
        out["server_peak_gb"] = srv.stats()["peak_bytes"] / 1e9
        srv.close()
    ctx.close()
    out["shapes"] = [list(i["shape"]) for i in insts]
    out["sources"] = [len(i["srnum"]) for i in insts]
    return out


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--models", type=int, default=48)
    p.add_argument("--slots", type=int, default=8)
    p.add_argument("--plain-models", type=int, default=None, help="time the plain baseline on the first N models")
    a = p.parse_args()
    out = run(a.models, a.slots, plain_models=a.plain_models)
    print(json.dumps({k: v for k, v in out.items() if k not in ("shapes", "sources")}), flush=True)


if __name__ == "__main__":
    main()

"""Serving benchmark: a Poisson stream of mixed requests through the request server.

    python -m pfast_gb300.serve_bench --rates 4 8 16 --duration 15 --precision mixed

Each request is a forward traveltime (70%) or a misfit + gradient (30%) evaluation on a 2D
grid (201x201 to 1001x401, one reflector) or a 3D grid (64^3 to 256x256x128), sizes
log-uniform, 1-64 surface sources, receivers on every 4th surface node (3D) / every 2nd
column (2D).  Half of the requests reuse a model already resident under its ID (an
inversion loop); the others bring a new model, which is registered on arrival.  Every
request brings its own survey.  Latency runs from arrival (before registration) to the
result on the host.  The offered load is swept over the given arrival rates; each rate
reports p50/p99 latency and completed solves per second (one solve = one source's
forward, or forward + adjoint for a gradient request).
"""
import argparse
import json
import math
import threading
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import synth

H3 = 20.0
H2 = 10.0
SIZES3 = (64 * 64 * 64, 256 * 256 * 128)
SIZES2 = (201 * 201, 1001 * 401)


def _shape3(n, rng):
    """A 3D grid of about n nodes with nrows = ncols = 2 nz (64^3 .. 256x256x128 range)."""
    nz = int(round((n / 4.0) ** (1.0 / 3.0)))
    nz = max(32, min(nz, 128))
    side = int(round(math.sqrt(n / nz)))
    side = max(64, min(side, 256))
    return nz, side, side


def _shape2(n, rng):
    nr = int(rng.integers(201, 402))
    nc = max(201, min(1001, int(round(n / nr))))
    return nr, nc


def model_pool(rng, n3=6, n2=6, seed=90):
    """Velocity models of log-uniform sizes: 3D (2000 + 0.6 z)(1 + 0.05 r) as the 3D gradient
    workload, 2D linear 1800 -> 4000 m/s with depth."""
    pool3, pool2 = [], []
    for k in range(n3):
        n = math.exp(rng.uniform(math.log(SIZES3[0]), math.log(SIZES3[1])))
        nz, nr, nc = _shape3(n, rng)
        pool3.append(synth.true_model3d(nz, nr, nc, H3, seed=seed + k))
    for k in range(n2):
        n = math.exp(rng.uniform(math.log(SIZES2[0]), math.log(SIZES2[1])))
        nr, nc = _shape2(n, rng)
        z = (np.arange(nr) + 1.0) * H2
        v = 1800.0 + (4000.0 - 1800.0) * (z - z[0]) / (z[-1] - z[0])
        pool2.append(np.ascontiguousarray(np.broadcast_to(v[:, None], (nr, nc))))
    return pool3, pool2


def survey3d(shape, nsrc, rng, noise=0.002):
    nz, nr, nc = shape
    ri, rj = np.meshgrid(np.arange(0, nr, 4), np.arange(0, nc, 4), indexing="ij")
    rec1 = np.stack([ri.ravel(), rj.ravel(), np.zeros(ri.size, int)], 1).astype(np.int32)
    src = np.stack([rng.integers(0, nr, nsrc), rng.integers(0, nc, nsrc), np.zeros(nsrc, int)], 1).astype(np.int32)
    rec = np.ascontiguousarray(np.tile(rec1, (nsrc, 1)))
    srnum = np.full(nsrc, len(rec1), np.int32)
    nxyz = np.tile([0.0, 0.0, -1.0], (len(rec), 1))
    s = np.repeat(src, len(rec1), axis=0)
    dist = H3 * np.sqrt(((rec[:, :2] - s[:, :2]) ** 2).sum(1))
    tobs = dist / 2000.0 + rng.normal(0.0, noise, len(rec))
    return src, srnum, rec, nxyz, tobs


def survey2d(shape, nsrc, rng, noise=0.002):
    nr, nc = shape
    depth = 0.7 * nr * H2
    Z = np.stack([np.full(nc, depth), -np.ones(nc), np.zeros(nc)], 1)
    cols = np.arange(0, nc, 2)
    src = np.stack([np.zeros(nsrc, int), rng.integers(0, nc, nsrc)], 1).astype(np.int32)
    rec = np.ascontiguousarray(np.tile(np.stack([np.zeros(len(cols), int), cols], 1), (nsrc, 1))).astype(np.int32)
    srnum = np.full(nsrc, len(cols), np.int32)
    nxy = np.tile([-1.0, 0.0], (len(rec), 1))
    off = H2 * np.abs(rec[:, 1] - np.repeat(src[:, 1], len(cols)))
    tt = off / 1800.0 + rng.normal(0.0, noise, len(rec))
    tr = np.sqrt(off ** 2 + (2 * depth) ** 2) / 2500.0 + rng.normal(0.0, noise, len(rec))
    return src, srnum, rec, nxy, tt, tr[:, None], Z


def run_stream(srv, pool3, pool2, rate, duration, precision, rng, max_inflight=256):
    """Offer a Poisson stream at `rate` requests/s for `duration` s.  Returns per-request records."""
    import pfast_gb300 as pg
    arrivals = np.cumsum(rng.exponential(1.0 / rate, int(rate * duration * 1.5) + 8))
    arrivals = arrivals[arrivals < duration]
    plans = []
    resident = {2: [], 3: []}
    next_id = [1000]
    for t in arrivals:
        dim = 3 if rng.random() < 0.5 else 2
        kind = "grad" if rng.random() < 0.3 else "fwd"
        nsrc = int(rng.integers(1, 65))
        reuse = bool(resident[dim]) and rng.random() < 0.5
        if reuse:
            mid, vp = resident[dim][int(rng.integers(0, len(resident[dim])))]
        else:
            vp = (pool3 if dim == 3 else pool2)[int(rng.integers(0, len(pool3 if dim == 3 else pool2)))]
            mid = next_id[0]
            next_id[0] += 1
            resident[dim].append((mid, vp))
        plans.append(dict(t=t, dim=dim, kind=kind, nsrc=nsrc, mid=mid, vp=vp, reuse=reuse,
                          seed=int(rng.integers(0, 2 ** 31))))
    records = []
    lock = threading.Lock()
    done_models = set()
    sem = threading.Semaphore(max_inflight)

    def finish(plan, ticket, t_arr):
        try:
            _, _, info = ticket.result()
            ok = True
        except pg.PfastError:
            info, ok = {}, False
        t_done = time.perf_counter()
        with lock:
            records.append(dict(dim=plan["dim"], kind=plan["kind"], nsrc=plan["nsrc"], ok=ok, lag_ms=plan["lag_ms"],
                                latency_ms=(t_done - t_arr) * 1e3, queue_ms=info.get("queue_ms", 0.0),
                                run_ms=info.get("run_ms", 0.0), t_done=t_done))
        srv.drop_survey(plan["sid"])
        sem.release()

    pool = ThreadPoolExecutor(max_workers=64)
    t0 = time.perf_counter()
    for k, plan in enumerate(plans):
        delay = t0 + plan["t"] - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        sem.acquire()
        t_arr = time.perf_counter()
        plan["lag_ms"] = (t_arr - t0 - plan["t"]) * 1e3   # > 0: the client offered it late
        prng = np.random.default_rng(plan["seed"])
        shape = plan["vp"].shape
        if plan["mid"] not in done_models:
            srv.put_model(plan["mid"], plan["vp"], (H3, H3, H3) if plan["dim"] == 3 else (H2, H2),
                          WR=None if plan["dim"] == 3 else 0.5)
            done_models.add(plan["mid"])
        sid = 10 ** 6 + k
        plan["sid"] = sid
        if plan["dim"] == 3:
            src, srnum, rec, nxyz, tobs = survey3d(shape, plan["nsrc"], prng)
            srv.put_survey3d(sid, shape, (H3, H3, H3), src, srnum, rec, nxyz, tobs)
        else:
            src, srnum, rec, nxy, tt, tr, Z = survey2d(shape, plan["nsrc"], prng)
            srv.put_survey2d(sid, shape, (H2, H2), src, srnum, rec, numofr=1, Z=Z, nxy=nxy, tt_obs=tt, tr_obs=tr)
        def submit():
            return (srv.submit_gradient(plan["mid"], sid, precision) if plan["kind"] == "grad"
                    else srv.submit_forward(plan["mid"], sid, precision))
        try:
            ticket = submit()
        except pg.PfastError:
            # the model was evicted to make room (least recently used): bring it back
            srv.put_model(plan["mid"], plan["vp"], (H3, H3, H3) if plan["dim"] == 3 else (H2, H2),
                          WR=None if plan["dim"] == 3 else 0.5)
            ticket = submit()
        pool.submit(finish, plan, ticket, t_arr)
    pool.shutdown(wait=True)
    t_end = max(r["t_done"] for r in records) if records else time.perf_counter()
    return records, t_end - t0


def summarize(records, wall_s, rate, duration):
    ok = [r for r in records if r["ok"]]
    lat = np.array([r["latency_ms"] for r in ok]) if ok else np.zeros(1)
    solves = sum(r["nsrc"] * (2 if r["kind"] == "grad" else 1) for r in ok)
    return {"offered_rate": rate, "requests": len(records), "failed": len(records) - len(ok),
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_queue_ms": float(np.mean([r["queue_ms"] for r in ok])) if ok else 0.0,
            "requests_per_s": len(ok) / wall_s, "solves_per_s": solves / wall_s, "wall_s": wall_s,
            "arrival_lag_ms_p99": float(np.percentile([r["lag_ms"] for r in records], 99)) if records else 0.0,
            "arrival_rate": len(records) / duration}


def knee(results, factor=3.0):
    """The lowest offered rate at which p99 latency exceeds `factor` times the p99 at the lowest
    rate, or the completion rate falls below 90% of the stream's actual arrival rate (None: not
    reached)."""
    if not results:
        return None
    base = results[0]["p99_ms"]
    for r in results:
        if r["p99_ms"] > factor * base or r["requests_per_s"] < 0.9 * r["arrival_rate"]:
            return r["offered_rate"]
    return None


def sweep(rates, duration, precision, slots=8, budget_gb=150.0, seed=5, pool=None):
    import pfast_gb300 as pg
    rng = np.random.default_rng(seed)
    pool3, pool2 = pool if pool is not None else model_pool(rng)
    out = []
    for rate in rates:
        srv = pg.Server(slots=slots, hbm_budget_gb=budget_gb)
        recs, wall = run_stream(srv, pool3, pool2, rate, duration, precision, np.random.default_rng(seed + int(rate)))
        st = srv.stats()
        srv.close()
        s = summarize(recs, wall, rate, duration)
        s["peak_gb"] = st["peak_bytes"] / 1e9
        out.append(s)
    return out


def main():
    import pfast_gb300 as pg
    p = argparse.ArgumentParser()
    p.add_argument("--rates", type=float, nargs="+", default=[2.0, 4.0, 8.0])
    p.add_argument("--duration", type=float, default=15.0)
    p.add_argument("--precision", choices=["mixed", "plain", "both"], default="both")
    p.add_argument("--slots", type=int, default=8)
    p.add_argument("--budget-gb", type=float, default=150.0)
    a = p.parse_args()
    rng = np.random.default_rng(5)
    pool = model_pool(rng)
    precs = {"mixed": [pg.PFAST_MIXED], "plain": [pg.PFAST_PLAIN_FP64], "both": [pg.PFAST_MIXED, pg.PFAST_PLAIN_FP64]}
    for prec in precs[a.precision]:
        for s in sweep(a.rates, a.duration, prec, a.slots, a.budget_gb, pool=pool):
            s["precision"] = "mixed" if prec == pg.PFAST_MIXED else "plain"
            print(json.dumps(s), flush=True)


if __name__ == "__main__":
    main()

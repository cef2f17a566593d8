"""Benchmark: 3D traveltime + adjoint-state gradient evaluations per second on one
GB300 (the 256 x 256 x 128, 256-source, 4096-receiver workload), batched FP32-bulk +
FP64-polish sweeps, with the plain FP64 path and the CPU restatement beside it.

A step = one misfit + gradient evaluation over all 256 sources (forward FSM,
receiver boundary conditions, adjoint FSM and the source-ordered gradient sum).
Inputs are seeded synthetic data (the workload has no public data set): the true
model is vp = (2000 + 0.6 z)(1 + 0.05 r) with r filtered white noise (200 m
correlation, unit std), observed picks = traveltimes on the true model + 2 ms
Gaussian noise, starting model = the 1D gradient.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  Under torchrun each rank evaluates its own copy
of the workload (independent replicas, weak scaling; the path has no collective).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NZ, NR, NC, H = 128, 256, 256, 20.0
NSRC_SIDE, NREC_SIDE = 16, 64
METRIC = "3D traveltime+adjoint grads/s vs plain FP64 GPU FSM at <=1e-5 rel; p50/p99 lat"
WORKLOAD = "3D first-arrival forward + adjoint gradient, 256x256x128 grid h=20 m, 256 surface sources (16x16), 4096 surface receivers (64x64), one misfit+gradient evaluation over all sources"
# identical in both arms (the CPU reference arm and the GPU arm)
CONFIG = {"workload": WORKLOAD, "grid": [256, 256, 128], "h_m": 20.0, "sources": 256, "receivers_per_source": 4096,
          "picks": "plain FP64 traveltimes on the true model + 2 ms Gaussian noise (seed 7)"}
DATA = ("synthetic (seeded generator, no public data set): vp = (2000 + 0.6 z)(1 + 0.05 r), r filtered noise with "
        "200 m correlation; starting model the 1D gradient")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--e2e-steps", type=int, default=None)
    p.add_argument("--cpu-sample", type=int, default=0, help="sources per CPU sample (0 = one per host thread)")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the secondary workloads (2D inversion, batched uneven 3D models, serving stream)")
    return p.parse_args()


def workload(seed=2024):
    from pfast_gb300.workloads import c3_inputs
    return c3_inputs(NZ, NR, NC, NSRC_SIDE, NREC_SIDE, seed=seed)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows if r[3].replace(".", "").isdigit()), default=None)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def fp64_peak_gflops(n=4096, reps=3):
    """Dense FP64 rate of this GPU: a cuBLAS DGEMM (torch.matmul on float64 n^3, 2 n^3 flops),
    best of `reps` after a warm-up, timed with CUDA events.  The polish kernels' FP64 roof."""
    import torch
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = None
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / (best / 1e3) / 1e9


PICK_NOISE_S, PICK_NOISE_SEED = 0.002, 7


def cpu_picks_sample(vt, src, srnum, rec, nsample, nthreads):
    """Observed picks of the first `nsample` sources, made the way the GPU arm makes them for all
    sources: plain FP64 traveltimes on the true model (the oracle port, bit-identical to the
    library's plain FP64 path) plus 2 ms Gaussian noise drawn in row order from one seeded
    stream, so the rows of the sample carry the same noise as in the full array."""
    from oracle import port
    from pfast_gb300 import synth
    ch = int(srnum[:nsample].sum())
    picks = port.forward3d(vt, src, srnum, rec, 100, H, H, H, s_begin=0, s_end=nsample, nthreads=nthreads)
    tobs = np.full(len(rec), 1000.0)
    tobs[:ch] = synth.add_noise(picks[:ch], PICK_NOISE_S, PICK_NOISE_SEED)
    return tobs


def cpu_eval_sample(v0, src, srnum, rec, nxyz, tobs, nsample, nthreads):
    """One misfit+gradient evaluation of the first `nsample` sources with the oracle port
    (the CPU restatement of the reference, `nthreads` threads).  Returns seconds."""
    from oracle import port
    t = time.perf_counter()
    port.eval3d(v0, src, srnum, rec, nxyz, tobs, 100, H, H, H, s_begin=0, s_end=nsample, nthreads=nthreads)
    return time.perf_counter() - t


def run_reference(args, rank):
    """--impl reference: the CPU restatement of the reference (oracle port, all host threads)
    on a bounded sample of the workload: each step evaluates the first `ns` sources (one per
    host thread), and `value` scales the step time to all 256 sources.  Nothing here loads the
    CUDA library: the generators in pfast_gb300.synth / workloads are numpy only."""
    if rank != 0:
        return
    vt, v0, src, srnum, rec, nxyz = workload()
    nthreads = os.cpu_count() or 1
    ns = args.cpu_sample or nthreads
    tobs = cpu_picks_sample(vt, src, srnum, rec, ns, nthreads)   # untimed, as on the GPU arm
    times = []
    for k in range(args.warmup + args.steps):
        dt = cpu_eval_sample(v0, src, srnum, rec, nxyz, tobs, ns, nthreads)
        if k >= args.warmup:
            times.append(dt)
    t_step = float(np.mean(times))             # seconds per step (ns sources)
    value = (ns / len(srnum)) / t_step         # full 256-source evaluations per second
    sample = (f"{ns} of 256 sources x 1 misfit+gradient evaluation per step on {nthreads} threads "
              f"({t_step:.2f} s); value scales the step time to 256 sources")
    line = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": DATA, "impl": "reference", "config": CONFIG,
            "precision": "plain FP64 (the reference's arithmetic)", "sample": sample,
            "cpu_baseline": {"value": value, "unit": "evals/s", "cores": nthreads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def extras():
    """Secondary workloads, each reported beside the headline (bounded: about two minutes in all):
    the 2D joint inversion (15 L-BFGS iterations, mixed vs plain FP64), 48 uneven 3D models
    in one batched evaluation (mixed and plain) vs sequential plain FP64 and vs the request
    server, and a Poisson serving stream swept over offered loads until p99 latency degrades
    (mixed 4-128 requests/s, plain 1-4 requests/s)."""
    out = {}
    jobs = (("inversion_2d", lambda: __import__("pfast_gb300.inv_bench", fromlist=["run"]).run(15)),
            ("batched_uneven_3d", lambda: {k: v for k, v in __import__("pfast_gb300.batch_bench", fromlist=["run"])
                                           .run(48, 8).items() if k not in ("shapes", "sources")}),
            ("serving", serving))
    for key, fn in jobs:
        try:
            out[key] = fn()
        except Exception as e:   # a secondary workload must not cost the headline line
            out[key] = {"error": repr(e)[:400]}
    return out


def serving():
    import pfast_gb300 as pg
    from pfast_gb300 import serve_bench
    rng = np.random.default_rng(5)
    pool = serve_bench.model_pool(rng)
    mixed = serve_bench.sweep([4.0, 16.0, 32.0, 64.0, 128.0], 6.0, pg.PFAST_MIXED, pool=pool)
    plain = serve_bench.sweep([1.0, 2.0, 4.0], 6.0, pg.PFAST_PLAIN_FP64, pool=pool)
    res = {"mixed": mixed, "plain": plain,
           "saturation_requests_per_s": {"mixed": max(r["requests_per_s"] for r in mixed),
                                         "plain": max(r["requests_per_s"] for r in plain)},
           "knee_rate": {"mixed": serve_bench.knee(mixed), "plain": serve_bench.knee(plain),
                         "rule": "first offered rate with p99 above three times the lowest rate's p99, or completions under 90% of the arrivals' rate"},
           "workload": "Poisson arrivals, 70% forward / 30% gradient, 2D 201x201..1001x401 (1 reflector) and 3D "
                       "64^3..256x256x128 grids log-uniform, 1-64 sources, 50% resident-model reuse, 8 slots, "
                       "150 GB budget; latency from arrival to host result"}
    return res


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)

    import torch
    import pfast_gb300 as pg

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    vt, v0, src, srnum, rec, nxyz = workload()
    ctx = pg.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    # observed picks: plain FP64 traveltimes on the true model + 2 ms noise (the reference arm
    # makes the same rows on the CPU)
    from pfast_gb300.workloads import observed_picks
    tobs = observed_picks(ctx, vt, src, srnum, rec, pg.PFAST_PLAIN_FP64, PICK_NOISE_S, PICK_NOISE_SEED)
    sv = pg.Survey3D(ctx, NR, NC, NZ, H, H, H, src, srnum, rec, nxyz, tobs)
    d_vp = torch.from_numpy(v0).cuda()
    grad = torch.empty_like(d_vp)

    # ---- the FP64 roof (a DGEMM, before anything is timed), autotuning on this workload (each
    # (schedule, tile shape) candidate once), then warm-up
    fp64_gflops = fp64_peak_gflops() if rank == 0 else None
    tune = sv.autotune(d_vp, precision=pg.PFAST_MIXED)
    # ---- device-resident timing (inputs already in HBM)
    for _ in range(args.warmup):
        sv.eval(d_vp, grad=grad, precision=pg.PFAST_MIXED)
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stats = []
    with ClockSampler(local) as clk:
        barrier()
        # an NVTX range around the timed steps, so that a profiler can select their kernels
        # (ncu --nvtx --nvtx-include "timed/")
        torch.cuda.nvtx.range_push("timed")
        for k in range(args.steps):
            ev[k][0].record(stream)
            _, misfit, st = sv.eval(d_vp, grad=grad, precision=pg.PFAST_MIXED)
            ev[k][1].record(stream)
            stats.append(st)
        torch.cuda.nvtx.range_pop()
        barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_ms = float(sum(step_ms))
    if dist:
        t = torch.tensor([t_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_ms = float(t.item())
    value = world * args.steps / (t_ms / 1e3)
    clocks = clk.summary()
    st = stats[-1]
    g_mixed = grad.clone()

    # ---- the plain FP64 path on the full workload (all 256 sources, one evaluation after a
    # warm-up one), and the accuracy of the mixed results against it over all sources
    g_plain = torch.empty_like(d_vp)
    sv.eval(d_vp, grad=g_plain, precision=pg.PFAST_PLAIN_FP64)   # warm-up
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    _, e_plain, st_plain = sv.eval(d_vp, grad=g_plain, precision=pg.PFAST_PLAIN_FP64)
    b.record(stream)
    torch.cuda.synchronize()
    plain_ms = a.elapsed_time(b)
    plain_value = 1.0 / (plain_ms / 1e3)
    gp, gm = g_plain.cpu().numpy(), g_mixed.cpu().numpy()
    grad_rel_l2 = float(np.linalg.norm(gm - gp) / np.linalg.norm(gp))
    pk_plain, _ = sv.forward(d_vp, precision=pg.PFAST_PLAIN_FP64)
    pk_mixed, _ = sv.forward(d_vp, precision=pg.PFAST_MIXED)
    pkp = pk_plain.cpu().numpy()
    tt_max_rel = float(np.max(np.abs(pk_mixed.cpu().numpy() - pkp) / pkp))
    del g_plain, pk_plain, pk_mixed

    # ---- end to end through the host-buffer C-ABI entry (copies inside the timed region)
    e2e_steps = args.e2e_steps if args.e2e_steps is not None else args.steps
    h_vp = torch.from_numpy(v0.copy()).pin_memory().numpy()
    h_grad = torch.empty(v0.shape, dtype=torch.float64).pin_memory().numpy()
    pg.eval3d_host(ctx, h_vp, H, H, H, src, srnum, rec, nxyz, tobs, precision=pg.PFAST_MIXED, grad=h_grad)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        pg.eval3d_host(ctx, h_vp, H, H, H, src, srnum, rec, nxyz, tobs, precision=pg.PFAST_MIXED, grad=h_grad)
    barrier()
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * e2e_steps / e2e_s
    h2d = v0.nbytes + src.nbytes + srnum.nbytes + rec.nbytes + nxyz.nbytes + tobs.nbytes
    d2h = v0.nbytes + 8

    # ---- roofline of the dominant kernel (the sweep kernel of the longest phase)
    phases = {"fwd32": (st["ms_fwd32"], st["fwd_node_updates"] - st["fwd64_node_updates"], 4, "kFwdFast32", "fwd32"),
              "fwd64": (st["ms_fwd64"], st["fwd64_node_updates"], 8, "kFwdPolish64", "fwd64_polish"),
              "adj32": (st["ms_adj32"], st["adj_node_updates"] - st["adj64_node_updates"], 4, "kAdjFast32", "adj32"),
              "adj64": (st["ms_adj64"], st["adj64_node_updates"], 8, "kAdjPolish64", "adj64_polish")}
    dom = max(phases, key=lambda k: phases[k][0])
    ms_dom, upd_dom, w, kind_name, kind_key = phases[dom]
    # the (schedule, tile shape) the autotuner gave that phase
    cand = pg._capi.phase_candidates(st).get(kind_key, "diagonal 4x8x32")
    sched, tshape = cand.split()
    # FP64 instructions per executed node update of the polish kernels (the residual-form
    # updates; everything else in them runs on the integer and FP32 pipes)
    fp64_per_update = {"fwd32": 0, "fwd64": 7, "adj32": 0, "adj64": 13}[dom]   # isotropic grid
    alg_bytes = upd_dom * 3 * w                       # read U + read slowness/T + write U per node update
    iters_dom = {"fwd32": st["fwd32_iters_max"], "fwd64": st["fwd_iters_max"], "adj32": st["adj32_iters_max"],
                 "adj64": st["adj_iters_max"]}[dom]
    tk, ti, tj = (int(x) for x in tshape.split("x"))
    ndiag = -(-NZ // tk) + -(-NR // ti) + -(-NC // tj) - 2   # tile diagonals: nbk + nbi + nbj - 2
    if sched == "persistent":   # one dataflow launch per phase and batch
        kname = f"sweep3d_dataflow<{kind_name}, {tshape}>"
        launches_dom = st["batches"]
    elif sched == "hybrid":   # the first outer iteration per diagonal, then one dataflow launch
        kname = f"sweep3d_kernel + sweep3d_dataflow<{kind_name}, {tshape}>"
        launches_dom = (8 * ndiag + 1) * st["batches"]
    else:   # outer iterations x 8 sweep orders x tile diagonals
        kname = f"sweep3d_kernel<{kind_name}, {tshape}>"
        launches_dom = iters_dom * 8 * ndiag * st["batches"]
    peaks, peak_kind = measured_peaks()
    achieved = alg_bytes / (ms_dom / 1e3) / 1e9 if ms_dom > 0 else 0.0
    # DRAM traffic per launch of the polish kernels: the algorithmic bytes per launch times the
    # ratio of measured DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum, 9-source
    # case of this grid) to the algorithmic bytes of the same launches, per (phase, schedule and
    # tile shape): forward polish over the 1680 per-diagonal launches of the phase (box); both
    # polish kinds in the dataflow kernel (register windows, one launch per phase); the FP32 bulk
    # kinds per diagonal (16-source case; their writes reach DRAM under later kernels, so these
    # two compare reads with the algorithmic total).  Above 1: the halo re-read; below 1:
    # resident sources sharing the slowness / traveltime lines in L2.
    traffic_ratios = {("fwd64", "diagonal 4x8x32"): 1.09, ("fwd64", "persistent 4x8x32"): 0.75,
                      ("adj64", "persistent 4x8x32"): 0.92, ("fwd32", "diagonal 4x8x32"): 1.23,
                      ("adj32", "diagonal 4x8x32"): 2.59}
    ratio = traffic_ratios.get((dom, cand))
    traffic = alg_bytes / launches_dom * ratio if (ratio and launches_dom) else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "traffic": traffic, "traffic_unit": "bytes per launch",
                "traffic_over_algorithmic": ratio, "schedule": cand,
                "algorithmic_bytes_per_launch": alg_bytes / launches_dom if launches_dom else None,
                "kernel": kname, "phase": dom,
                "peak_kind": peak_kind, "node_updates_per_s": upd_dom / (ms_dom / 1e3) if ms_dom > 0 else 0.0,
                "phase_ms": ms_dom}
    if fp64_per_update and ms_dom > 0 and fp64_gflops:
        # FP64 roof: FP64 instructions of the executed updates per second against the DGEMM rate
        # in FMA instructions per second (an FMA is one instruction, two flops).  A lower bound
        # of the FP64 pipe's occupancy: an FP64 warp instruction holds the pipe for ~75 cycles
        # however many of its lanes are active, and wavefront steps run with idle lanes.
        ach = upd_dom * fp64_per_update / (ms_dom / 1e3) / 1e9
        roofline["fp64"] = {"per_update": fp64_per_update, "achieved": ach, "peak": fp64_gflops / 2.0,
                            "unit": "G FP64 instructions/s", "frac": ach / (fp64_gflops / 2.0),
                            "peak_kind": "measured: cuBLAS DGEMM 4096^3 through torch, best of 3, FMA = 1 instruction"}

    # ---- CPU baseline (oracle port, bounded sample), rank 0 at N=1 only
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        nthreads = os.cpu_count() or 1
        ns = args.cpu_sample or nthreads
        cdt = cpu_eval_sample(v0, src, srnum, rec, nxyz, tobs, ns, nthreads)
        cv = (ns / len(srnum)) / cdt
        cpu = {"value": cv, "unit": "evals/s", "cores": nthreads, "kind": "port",
               "sample": f"{ns} of 256 sources, one misfit+gradient evaluation on the same picks ({cdt:.1f} s), "
                         "scaled to 256 sources"}

    line = None
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32+f64", "data": DATA, "config": CONFIG,
                "precision": "FP32 bulk sweeps + FP64 polish",
                "l2": "no flush: each evaluation streams 256 x 64 MiB fields, far above the 129 MB L2",
                "parallelism": "sources batched on one GPU" if world == 1 else f"{world} independent replicas",
                "e2e": {"value": e2e_value, "unit": "evals/s", "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(d2h), "entry": "pfast_eval3d (host buffers, pinned)"},
                "gpu_launches": int(sum(s["launches"] for s in stats)),
                "clocks": clocks, "roofline": roofline, "cpu_baseline": cpu,
                "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99)),
                               "of": "one 256-source misfit+gradient evaluation, device-resident"},
                "misfit": misfit,
                "autotune_ms": {k: v["ms_total"] for k, v in tune.items()},
                "step_ms": step_ms,
                "phase_ms": {k: st[k] for k in ("ms_fwd32", "ms_fwd64", "ms_adj32", "ms_adj64", "ms_other", "ms_total")},
                "phase_schedule": pg._capi.phase_candidates(st),
                "iters": {k: st[k] for k in ("fwd32_iters_max", "fwd_iters_max", "adj32_iters_max", "adj_iters_max")}}
    sv.close()
    ctx.close()
    if rank == 0:
        if world == 1 and not args.no_extras:
            line["extras"] = extras()
        # the metric's own comparison last, so that it closes the printed line
        line["plain_fp64"] = {"value": plain_value, "unit": "evals/s", "sources": len(srnum), "ms": plain_ms,
                              "misfit": e_plain, "fwd_iters": st_plain["fwd_iters_max"],
                              "adj_iters": st_plain["adj_iters_max"]}
        line["accuracy"] = {"tt_max_rel": tt_max_rel, "grad_rel_l2": grad_rel_l2, "sources": len(srnum),
                            "vs": "plain FP64 (bit-identical to the oracle)", "bar": {"tt_max_rel": 1e-5,
                                                                                     "grad_rel_l2": 1e-4}}
        line["mixed_over_plain"] = value / world / plain_value
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

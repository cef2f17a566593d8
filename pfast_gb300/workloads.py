"""Synthetic evaluation workloads (used by bench.py and for profiling).

    python -m pfast_gb300.workloads --grid 128 256 256 --sources 16 --precision mixed --evals 1

builds the 3D gradient workload on the given grid (h = 20 m, sources on a square
surface grid, receivers on every 4th surface node) and runs evaluations on cuda:0.
"""
import argparse
import time

import numpy as np

from . import synth

H = 20.0


def c3_inputs(nz=128, nr=256, nc=256, n_src_side=16, n_rec_side=64, seed=2024):
    """True model, starting model and geometry of the 3D gradient workload."""
    vt = synth.true_model3d(nz, nr, nc, H, seed=seed)
    v0 = synth.gradient_model3d(nz, nr, nc, H)
    src, srnum, rec, nxyz = synth.surface_survey3d(nr, nc, n_src_side, n_rec_side)
    return vt, v0, src, srnum, rec, nxyz


def observed_picks(ctx, vt, src, srnum, rec, precision, noise_s=0.002, seed=7):
    """First-arrival picks on the true model (GPU) plus Gaussian noise."""
    import torch
    from .api import Survey3D
    nz, nr, nc = vt.shape
    sv = Survey3D(ctx, nr, nc, nz, H, H, H, src, srnum, rec)
    picks, _ = sv.forward(torch.from_numpy(vt).cuda(), precision=precision)
    sv.close()
    return synth.add_noise(picks.cpu().numpy(), noise_s, seed)


def main():
    import torch
    from . import api
    p = argparse.ArgumentParser()
    p.add_argument("--grid", type=int, nargs=3, default=[128, 256, 256], metavar=("NZ", "NROWS", "NCOLS"))
    p.add_argument("--sources", type=int, default=16, help="number of sources (a square number)")
    p.add_argument("--precision", choices=["plain", "mixed"], default="mixed")
    p.add_argument("--evals", type=int, default=1)
    p.add_argument("--picks-precision", choices=["plain", "mixed"], default="plain",
                   help="solver of the observed picks on the true model (plain FP64 by default)")
    p.add_argument("--schedule", choices=["auto", "diagonal", "dataflow", "hybrid"], default="auto",
                   help="3D sweep schedule: one launch per tile diagonal, one dataflow launch per phase, or "
                        "the first outer iteration per diagonal and the rest in one dataflow launch")
    p.add_argument("--autotune", action="store_true",
                   help="time every (schedule, tile shape) candidate first, so that automatic phases use "
                        "the fastest (as bench.py does)")
    p.add_argument("--no-graphs", action="store_true",
                   help="launch each outer iteration's sweeps one by one instead of replaying captured graphs")
    a = p.parse_args()
    side = int(round(np.sqrt(a.sources)))
    nz, nr, nc = a.grid
    vt, v0, src, srnum, rec, nxyz = c3_inputs(nz, nr, nc, side, max(1, nr // 4))
    ctx = api.Context(0)
    if a.no_graphs:
        ctx.set_graphs(False)
    prec = api.PFAST_MIXED if a.precision == "mixed" else api.PFAST_PLAIN_FP64
    pprec = api.PFAST_MIXED if a.picks_precision == "mixed" else api.PFAST_PLAIN_FP64
    tobs = observed_picks(ctx, vt, src, srnum, rec, pprec)
    sv = api.Survey3D(ctx, nr, nc, nz, H, H, H, src, srnum, rec, nxyz, tobs)
    d = torch.from_numpy(v0).cuda()
    if a.autotune:
        sv.autotune(d, precision=prec)
    for _ in range(a.evals):
        t = time.perf_counter()
        # an NVTX range per evaluation, so that a profiler can select its kernels
        # (ncu --nvtx --nvtx-include "evaluation/")
        torch.cuda.nvtx.range_push("evaluation")
        g, e, st = sv.eval(d, precision=prec, schedule={"auto": 0, "diagonal": 1, "dataflow": 2, "hybrid": 3}[a.schedule])
        torch.cuda.nvtx.range_pop()
        print(f"eval {time.perf_counter() - t:.3f} s misfit {e:.6g}", {k: v for k, v in st.items() if v},
              api._capi.phase_candidates(st), flush=True)
    sv.close()
    ctx.close()


if __name__ == "__main__":
    main()

"""Generate the golden fixtures under tests/golden/ (run in a checkout that has the
reference tree; the fixtures are committed so nothing else needs it).

* rt2d_fw_golden.npz -- the reference's shipped 2D forward case: the model
  models/RT_SynMod2D_FW.vp, reflectors models/RT_SynMod2D.ref, sources
  models/RT_SynMod2D.src and receiver geometry, converted to node indices as the
  driver does (src/RT_PFAST2D.cpp:299-343), plus the golden picks of
  models/RT_SynMod2D_Inv.rec column 5 (transmission) and column 7 (second
  reflector) for every 4th source (the file's column 6 was zeroed by
  mfiles/RT_SynMod2D.m:127).
* rt2d_inv_golden.npz -- the shipped inversion case (models/RT_SynMod2D_Inv.vp,
  noisy picks models/RT_SynMod2D_Inv_rand2p.rec, WR = 0.5 everywhere) for the same
  sources, with the joint gradient and misfits computed by the reference's own
  Tadjoint_fsm2d / Radjoint_fsm2d built into oracle/_ref (SHA-256 of the gradient
  bytes, misfits as exact doubles).
* rt2d_inv_trace.npz -- the shipped inversion case with all 56 sources: the noisy picks
  of models/RT_SynMod2D_Inv_rand2p.rec (columns 4-6; geometry = rt2d_fw_golden's) and
  the lines the reference printed for iterations 1-4 of its three runs
  (par/RT_SynMod2D_Inv_RT.out, _Trans.out, _Ref.out: RTtag 3, 1, 2): the residual line
  and the line-search rows, numbers as printed (%g).
* pins3d.json -- seeded small 3D cases: SHA-256 of the traveltime and adjoint
  fields and the misfit bits produced by the reference's fsm3d / adjoint_fsm3d
  (oracle/_ref).

Usage: python tests/golden/make_golden.py [trace]   (trace: only rt2d_inv_trace.npz)
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref, ref  # noqa: E402
from pfast_gb300 import io as pio  # noqa: E402   (pure numpy helpers; no CUDA needed)

REF = build_ref.ref_root()
M = os.path.join(REF, "models")
SRC_SUBSET = np.arange(0, 56, 4)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def rows_of(srnum, subset):
    ch0 = np.concatenate([[0], np.cumsum(srnum)])
    return np.concatenate([np.arange(ch0[s], ch0[s + 1]) for s in subset])


def cases3d():
    """Small seeded 3D cases (inputs are regenerated from these parameters by the tests)."""
    return [
        dict(name="cube9", shape=(9, 11, 13), h=(10.0, 10.0, 10.0), seed=101),
        dict(name="aniso", shape=(9, 11, 13), h=(10.0, 12.5, 8.0), seed=102),
        dict(name="odd17", shape=(17, 19, 23), h=(20.0, 20.0, 20.0), seed=103),
    ]


def make_case3d(c):
    """Inputs of one 3D pin case: model, 3 sources (one interior, two at corners), receivers on the
    k=0 surface every 2nd row / 3rd column, one unpicked row, noisy picks."""
    rng = np.random.default_rng(c["seed"])
    nz, nr, nc = c["shape"]
    vp = 1500.0 + 2000.0 * rng.random((nz, nr, nc))
    src = np.array([[nr // 2, nc // 3, nz // 3], [0, 0, 0], [nr - 1, nc - 1, nz - 1]], np.int32)
    r1 = np.array([(i, j, 0) for i in range(0, nr, 2) for j in range(0, nc, 3)], np.int32)
    rec = np.concatenate([r1, r1, r1])
    srnum = np.full(3, len(r1), np.int32)
    nxyz = np.tile([0.0, 0.0, -1.0], (len(rec), 1))
    noise = 0.002 * (rng.random(len(rec)) - 0.5)
    return vp, src, srnum, rec, nxyz, noise


def pins3d():
    out = []
    for c in cases3d():
        vp, src, srnum, rec, nxyz, noise = make_case3d(c)
        dx, dy, dz = c["h"]
        ent = dict(c, sources=[])
        ch0 = np.concatenate([[0], np.cumsum(srnum)])
        for s in range(len(srnum)):
            U = ref.fsm3d(vp, src, s, 100, dx, dy, dz)
            rows = np.arange(ch0[s], ch0[s + 1])
            tobs = np.zeros(len(rec))
            tobs[rows] = U[rec[rows, 2], rec[rows, 0], rec[rows, 1]] + noise[rows]
            tobs[rows[3]] = 1000.0   # one unpicked receiver
            L, E = ref.adjoint3d(U, tobs, rec, nxyz, src, srnum, s, 100, dx, dy, dz)
            ent["sources"].append(dict(T_sha=sha(U), L_sha=sha(L), EE_hex=float(E).hex()))
        out.append(ent)
    return out


TRACE_ITERS = 4


def trace_lines(path, iters=TRACE_ITERS):
    """The "Average Time Residual" and "(alpha0,...)" lines of iterations 1..iters of a log."""
    out, it = [], 0
    for line in open(path):
        if line.startswith("Iterating No."):
            it += 1
            if it > iters:
                break
        elif it and (line.startswith("Average Time Residual") or line.startswith("(alpha0,alpha1")):
            out.append(line.rstrip("\n"))
    return out


def inversion_trace():
    noisy = pio.readmod(os.path.join(M, "RT_SynMod2D_Inv_rand2p.rec"), 33600 * 7).reshape(33600, 7)
    fw_rec = pio.readmod(os.path.join(M, "RT_SynMod2D_FW.rec"), 33600 * 4).reshape(33600, 4)
    assert np.array_equal(noisy[:, :4], pio.readmod(os.path.join(M, "RT_SynMod2D_Inv.rec"),
                                                    33600 * 7).reshape(33600, 7)[:, :4])
    assert np.array_equal(noisy[:, :2], fw_rec[:, :2])
    P = os.path.join(REF, "par")
    logs = {3: "RT_SynMod2D_Inv_RT.out", 1: "RT_SynMod2D_Inv_Trans.out", 2: "RT_SynMod2D_Inv_Ref.out"}
    kw = {f"log_rttag{t}": np.array(trace_lines(os.path.join(P, f))) for t, f in logs.items()}
    np.savez_compressed(os.path.join(HERE, "rt2d_inv_trace.npz"), tt=noisy[:, 4].copy(), tr=noisy[:, 5:7].copy(),
                        nxy=noisy[:, 2:4].copy(), LM=50, nux=60.0, nuz=20.0, iters=TRACE_ITERS, **kw)


def main():
    if sys.argv[1:] == ["trace"]:
        inversion_trace()
        print("rt2d_inv_trace.npz written to", HERE)
        return
    if not ref.available():
        build_ref.build()
    dx, dz = 12.5, 8.0
    srcA = pio.readmod(os.path.join(M, "RT_SynMod2D.src"), 56 * 3).reshape(56, 3)
    Z = pio.readmod(os.path.join(M, "RT_SynMod2D.ref"), 1200 * 3).reshape(1200, 3)
    numofr = 2
    fw_rec = pio.readmod(os.path.join(M, "RT_SynMod2D_FW.rec"), 33600 * 4).reshape(33600, 4)
    gold = pio.readmod(os.path.join(M, "RT_SynMod2D_Inv.rec"), 33600 * 7).reshape(33600, 7)
    noisy = pio.readmod(os.path.join(M, "RT_SynMod2D_Inv_rand2p.rec"), 33600 * 7).reshape(33600, 7)
    vp_fw = pio.readmod(os.path.join(M, "RT_SynMod2D_FW.vp"), 160 * 600).reshape(160, 600)
    vp_inv = pio.readmod(os.path.join(M, "RT_SynMod2D_Inv.vp"), 160 * 600).reshape(160, 600)
    wr = pio.readmod(os.path.join(M, "RT_SynMod2D_Inv.wr"), 160 * 600)
    assert np.all(wr == 0.5)
    src, srnum, rec, nxy, _, _ = pio.load_survey2d(srcA, fw_rec, dx, dz, numofr)
    rows = rows_of(srnum, SRC_SUBSET)
    np.savez_compressed(os.path.join(HERE, "rt2d_fw_golden.npz"), vp=vp_fw, Z=Z, src=src, srnum=srnum,
                        rec=rec.astype(np.int16), nxy=nxy, dx=dx, dz=dz, numofr=numofr, subset=SRC_SUBSET,
                        rows=rows.astype(np.int32), tt=gold[rows, 4], tr2=gold[rows, 6])
    # inversion case: the reference's own adjoints on the subset of sources
    sub_src = src[SRC_SUBSET]
    sub_srnum = srnum[SRC_SUBSET]
    sub_rec = rec[rows]
    sub_nxy = noisy[rows, 2:4].copy()
    tt = noisy[rows, 4].copy()
    tr = noisy[rows, 5:7].copy()
    gT = np.zeros((160, 600))
    gR = np.zeros((160, 600))
    Et = Er = 0.0
    v3 = vp_inv * vp_inv * vp_inv
    for s in range(len(SRC_SUBSET)):
        U, TTd, TTu = ref.rt_fsm2d(vp_inv, Z, sub_src, s, numofr, 500, dx, dz)
        LT, e1 = ref.tadjoint2d(U, tt, sub_rec, sub_nxy, sub_src, sub_srnum, s, 500, dx, dz)
        LR, e2 = ref.radjoint2d(TTd, TTu, tr, sub_rec, sub_nxy, sub_src, sub_srnum, s, numofr, 500, dx, dz)
        gT = gT - LT / v3
        gR = gR - LR / v3
        Et += e1
        Er += e2
    gRT = gT * (1. - 0.5) + gR * 0.5
    np.savez_compressed(os.path.join(HERE, "rt2d_inv_golden.npz"), vp=vp_inv, src=sub_src, srnum=sub_srnum,
                        rec=sub_rec.astype(np.int16), nxy=sub_nxy, tt=tt, tr=tr, wr=0.5, dx=dx, dz=dz, numofr=numofr,
                        Et_hex=float(Et).hex(), Er_hex=float(Er).hex(), gT_sha=sha(gT), gR_sha=sha(gR),
                        gRT_sha=sha(gRT), gT_sample=gT.ravel()[::997], gR_sample=gR.ravel()[::997])
    with open(os.path.join(HERE, "pins3d.json"), "w") as f:
        json.dump(pins3d(), f, indent=1)
    inversion_trace()
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()

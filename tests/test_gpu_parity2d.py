"""2D parity on the GPU (RT_fsm2d with Huygens reflection, transmission and
reflection adjoints, joint gradient) through the C ABI.

The golden checks use the reference's shipped case (tests/golden/): picks must
equal models/RT_SynMod2D_Inv.rec columns 5 and 7 bit for bit, and the joint
gradient / misfits must equal what the reference's own code produced.
"""
import hashlib

import numpy as np
import pytest

from helpers import bits_equal, load_fw, load_inv

pytestmark = pytest.mark.gpu


def _pg():
    import pfast_gb300 as pg
    return pg


def _torch():
    import torch
    return torch


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_golden_forward_picks_bit_exact(ctx):
    """All 56 sources, 33600 traces, 2 reflectors on one GPU; rows of every 4th source
    checked against the shipped golden columns."""
    pg, torch = _pg(), _torch()
    g = load_fw()
    sv = pg.Survey2D(ctx, 160, 600, float(g["dx"]), float(g["dz"]), g["src"], g["srnum"], g["rec"].astype(np.int32),
                     numofr=int(g["numofr"]), Z=g["Z"])
    Tr, st = sv.forward(torch.from_numpy(g["vp"]).cuda())
    Tr = Tr.cpu().numpy()
    assert Tr.shape == (33600, 3)
    assert bits_equal(Tr[g["rows"], 0], g["tt"])
    assert bits_equal(Tr[g["rows"], 2], g["tr2"])
    assert st["not_converged"] == 0


def test_golden_forward_mixed_within_tolerance(ctx):
    pg, torch = _pg(), _torch()
    g = load_fw()
    sv = pg.Survey2D(ctx, 160, 600, float(g["dx"]), float(g["dz"]), g["src"], g["srnum"], g["rec"].astype(np.int32),
                     numofr=int(g["numofr"]), Z=g["Z"])
    Tr, _ = sv.forward(torch.from_numpy(g["vp"]).cuda(), precision=pg.PFAST_MIXED)
    Tr = Tr.cpu().numpy()
    assert np.max(np.abs(Tr[g["rows"], 0] - g["tt"]) / g["tt"]) <= 1e-5
    assert np.max(np.abs(Tr[g["rows"], 2] - g["tr2"]) / g["tr2"]) <= 1e-5


def test_golden_joint_gradient_bit_exact(ctx):
    pg, torch = _pg(), _torch()
    g = load_inv()
    Z = load_fw()["Z"]
    sv = pg.Survey2D(ctx, 160, 600, float(g["dx"]), float(g["dz"]), g["src"], g["srnum"], g["rec"].astype(np.int32),
                     numofr=int(g["numofr"]), Z=Z, nxy=g["nxy"], tt_obs=g["tt"], tr_obs=g["tr"])
    WR = torch.full((160, 600), float(g["wr"]), dtype=torch.float64, device="cuda")
    r = sv.eval(torch.from_numpy(g["vp"]).cuda(), WR)
    assert float(r["Et"]).hex() == str(g["Et_hex"])
    assert float(r["Er"]).hex() == str(g["Er_hex"])
    assert sha(r["gT"].cpu().numpy()) == str(g["gT_sha"])
    assert sha(r["gR"].cpu().numpy()) == str(g["gR_sha"])
    assert sha(r["gRT"].cpu().numpy()) == str(g["gRT_sha"])
    rm = sv.eval(torch.from_numpy(g["vp"]).cuda(), WR, precision=pg.PFAST_MIXED)
    ref = r["gRT"].cpu().numpy()
    rel = np.linalg.norm(rm["gRT"].cpu().numpy() - ref) / np.linalg.norm(ref)
    assert rel <= 1e-4, rel


def test_rt_fsm2d_and_adjoint_shims_bit_exact():
    from oracle import port
    pg = _pg()
    g = load_inv()
    Z = load_fw()["Z"]
    src, srnum, rec = g["src"], g["srnum"], g["rec"].astype(np.int32)
    for s in (0, 5):
        U0, TTd0, TTu0, st, _ = port.rt_fsm2d(g["vp"], Z, src, s, 2, 500, 12.5, 8.0)
        assert st == 0
        U, TTd, TTu = np.empty((160, 600)), np.empty((2, 160, 600)), np.empty((2, 160, 600))
        pg.RT_fsm2d(g["vp"], U, TTd, TTu, Z, src, rec, srnum, s, 2, 500, 12.5, 8.0, 160, 600)
        assert bits_equal(U, U0) and bits_equal(TTd, TTd0) and bits_equal(TTu, TTu0)
        LT0, ET0, _ = port.tadjoint2d(U0, g["tt"], rec, g["nxy"], src, srnum, s, 500, 12.5, 8.0)
        LT = np.empty((160, 600))
        ET = pg.Tadjoint_fsm2d(LT, U0, g["tt"], rec, g["nxy"], src, srnum, s, 500, 12.5, 8.0, 160, 600)
        assert bits_equal(LT, LT0) and ET == ET0
        LR0, ER0, _ = port.radjoint2d(TTu0, g["tr"], rec, g["nxy"], src, srnum, s, 2, 500, 12.5, 8.0)
        LR = np.empty((160, 600))
        ER = pg.Radjoint_fsm2d(LR, TTd0, TTu0, g["tr"], rec, g["nxy"], src, srnum, s, 2, 500, 12.5, 8.0, 160, 600)
        assert bits_equal(LR, LR0) and ER == ER0


def test_first_arrival_workload_vs_oracle(ctx):
    """The 301 x 101 first-arrival workload (21 sources, 301 receivers each, no reflector)."""
    from oracle import port
    from pfast_gb300 import synth
    pg, torch = _pg(), _torch()
    vp = synth.first_arrival2d_model()
    src, srnum, rec, nxy = synth.surface_survey2d(101, 301, list(range(0, 301, 15)), list(range(301)))
    Tr0, st = port.forward2d(vp, None, src, srnum, rec, 0, 500, 10.0, 10.0, nthreads=4)
    sv = pg.Survey2D(ctx, 101, 301, 10.0, 10.0, src, srnum, rec)
    Tr, _ = sv.forward(torch.from_numpy(vp).cuda())
    assert bits_equal(Tr.cpu().numpy(), Tr0)


def test_reflection_with_iteration_counter_carry(ctx):
    """Two reflectors and a small MAXSwp: the reflection adjoint's iteration counter carries over
    from one reflector to the next, as in the reference."""
    from oracle import port
    pg, torch = _pg(), _torch()
    nr, nc = 50, 120
    vp = 1600.0 + 25.0 * np.arange(nr)[:, None] + np.zeros((1, nc))
    Z = np.concatenate([np.stack([np.full(nc, 200.0 + 10 * np.sin(np.arange(nc) / 7.0)), -np.ones(nc),
                                  np.zeros(nc)], 1),
                        np.stack([np.full(nc, 420.0), -np.ones(nc), np.zeros(nc)], 1)])
    src = np.array([[0, 15], [0, 60], [0, 100]], np.int32)
    rec = np.array([(0, j) for j in range(0, nc, 2)] * 3, np.int32)
    srnum = np.full(3, nc // 2, np.int32)
    nxy = np.tile([-1.0, 0.0], (len(rec), 1))
    Tr, st = port.forward2d(vp, Z, src, srnum, rec, 2, 500, 10.0, 10.0)
    rng = np.random.default_rng(3)
    tt = Tr[:, 0] + rng.normal(0, 1e-3, len(rec))
    tr = Tr[:, 1:] + rng.normal(0, 1e-3, (len(rec), 2))
    tr[::5, 0] = 0.0
    WRh = np.full((nr, nc), 0.3)
    for maxswp in (500, 3):
        r0 = port.eval2d(vp * 1.02, WRh, Z, src, srnum, rec, nxy, tt, tr, 2, maxswp, 10.0, 10.0)
        sv = pg.Survey2D(ctx, nr, nc, 10.0, 10.0, src, srnum, rec, numofr=2, Z=Z, nxy=nxy, tt_obs=tt, tr_obs=tr)
        r = sv.eval(torch.from_numpy(vp * 1.02).cuda(), torch.from_numpy(WRh).cuda(), maxswp=maxswp)
        assert bits_equal(r["gT"].cpu().numpy(), r0["gT"])
        assert bits_equal(r["gR"].cpu().numpy(), r0["gR"])
        assert bits_equal(r["gRT"].cpu().numpy(), r0["gRT"])
        assert r["Et"] == r0["Et"] and r["Er"] == r0["Er"]


def test_reflector_without_node_above_is_an_error(ctx):
    pg, torch = _pg(), _torch()
    nr, nc = 20, 30
    Z = np.stack([np.full(nc, 5.0), -np.ones(nc), np.zeros(nc)], 1)   # above the first row
    sv = pg.Survey2D(ctx, nr, nc, 10.0, 10.0, np.array([[0, 3]], np.int32), np.array([1], np.int32),
                     np.array([[0, 5]], np.int32), numofr=1, Z=Z)
    with pytest.raises(pg.PfastError) as e:
        sv.forward(torch.full((nr, nc), 2000.0, dtype=torch.float64, device="cuda"))
    assert e.value.status == 5   # PFAST_ERR_NO_REFLECTION_POINT


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_graph_replay_matches_launches_2d(ctx, precision):
    # 2D outer iterations replayed as captured CUDA graphs give the bits and iteration counts of
    # launching the kernels one by one (joint transmission + reflection gradient)
    pg, torch = _pg(), _torch()
    prec = pg.PFAST_PLAIN_FP64 if precision == "plain" else pg.PFAST_MIXED
    g = load_inv()
    Z = load_fw()["Z"]
    sv = pg.Survey2D(ctx, 160, 600, float(g["dx"]), float(g["dz"]), g["src"], g["srnum"], g["rec"].astype(np.int32),
                     numofr=int(g["numofr"]), Z=Z, nxy=g["nxy"], tt_obs=g["tt"], tr_obs=g["tr"])
    WR = torch.full((160, 600), float(g["wr"]), dtype=torch.float64, device="cuda")
    vp = torch.from_numpy(g["vp"]).cuda()
    try:
        ctx.set_graphs(False)
        r0 = sv.eval(vp, WR, precision=prec)
        ctx.set_graphs(True)
        r1 = sv.eval(vp, WR, precision=prec)   # a phase is captured the second time its shape comes up
        r2 = sv.eval(vp, WR, precision=prec)   # replayed
    finally:
        ctx.set_graphs(True)
    for r in (r1, r2):
        for k in ("gT", "gR", "gRT"):
            assert bits_equal(r0[k].cpu().numpy(), r[k].cpu().numpy()), k
        assert r0["Et"] == r["Et"] and r0["Er"] == r["Er"]
        for k in ("fwd_iters_max", "adj_iters_max", "launches"):
            assert r0["stats"][k] == r["stats"][k], k


def test_near_source_initialisation_2d(ctx):
    """Opt-in near-source start in 2D (not in the reference): in a homogeneous medium, where the
    exact traveltime is distance / v, starting the nodes within 4 nodes of the source from the
    straight-ray time cuts the first-order scheme's error away from the source; the mixed path
    with the same option stays within 1e-5 of the plain one; radius 0 is the reference's point
    source, bit for bit."""
    pg, torch = _pg(), _torch()
    nr, nc, h, v = 41, 61, 10.0, 2000.0
    vp = np.full((nr, nc), v)
    src = np.array([[20, 30], [0, 0], [5, 50]], np.int32)   # (row, col)
    rr, cc = np.meshgrid(np.arange(0, nr, 2), np.arange(0, nc, 2), indexing="ij")
    r1 = np.stack([rr.ravel(), cc.ravel()], 1).astype(np.int32)
    rec = np.ascontiguousarray(np.concatenate([r1] * len(src)))
    srnum = np.full(len(src), len(r1), np.int32)
    sv = pg.Survey2D(ctx, nr, nc, h, h, src, srnum, rec)
    d = torch.from_numpy(vp).cuda()
    s = np.repeat(src, len(r1), axis=0)
    dist = h * np.sqrt(((rec - s) ** 2).sum(1).astype(float))
    exact = dist / v
    far = dist > 6 * h   # outside every fixed region
    err = {}
    for r in (0, 4):
        Tr, _ = sv.forward(d, precision=pg.PFAST_PLAIN_FP64, near_source_radius=r)
        pk = Tr.cpu().numpy()[:, 0]
        err[r] = np.max(np.abs(pk[far] - exact[far]) / exact[far])
        if r:
            near = (dist > 0) & (dist <= r * h)
            assert np.allclose(pk[near], exact[near], rtol=1e-12)   # straight-ray values, exact here
            Tm, _ = sv.forward(d, precision=pg.PFAST_MIXED, near_source_radius=r)
            pm = Tm.cpu().numpy()[:, 0]
            assert np.max(np.abs(pm - pk) / np.maximum(pk, 1e-30)) <= 1e-5
    assert err[4] < 0.5 * err[0], err
    p0, _ = sv.forward(d, precision=pg.PFAST_PLAIN_FP64)
    p1, _ = sv.forward(d, precision=pg.PFAST_PLAIN_FP64, near_source_radius=0)
    assert bits_equal(p0.cpu().numpy(), p1.cpu().numpy())
    with pytest.raises(pg.PfastError):
        sv.forward(d, precision=pg.PFAST_PLAIN_FP64, near_source_radius=65)
    sv.close()


def test_joint_gradient_full_size(ctx):
    """The 2D joint inversion workload at full size (601 x 201 grid, h = 5 m, 40 sources, 400
    receivers, one reflector): the plain joint gradient equals the oracle bit for bit; the mixed
    one stays within 1e-4 relative L2 of it, with the misfits within 1e-6."""
    from oracle import port
    from pfast_gb300 import inv_bench
    pg, torch = _pg(), _torch()
    vt, v0, Z, src, srnum, rec, nxy = inv_bench.workload()
    nr, nc = vt.shape
    assert (nr, nc) == (201, 601) and len(srnum) == 40 and int(srnum[0]) == 400
    tt, tr = inv_bench.picks(ctx, vt, Z, src, srnum, rec)
    WR = np.full((nr, nc), 0.5)
    r0 = port.eval2d(v0, WR, Z, src, srnum, rec, nxy, tt, tr, 1, 500, inv_bench.H, inv_bench.H, nthreads=4)
    sv = pg.Survey2D(ctx, nr, nc, inv_bench.H, inv_bench.H, src, srnum, rec, numofr=1, Z=Z, nxy=nxy,
                     tt_obs=tt, tr_obs=tr)
    d, w = torch.from_numpy(v0).cuda(), torch.from_numpy(WR).cuda()
    rp = sv.eval(d, w, precision=pg.PFAST_PLAIN_FP64)
    for k in ("gT", "gR", "gRT"):
        assert bits_equal(rp[k].cpu().numpy(), r0[k]), k
    assert rp["Et"] == r0["Et"] and rp["Er"] == r0["Er"]
    rm = sv.eval(d, w, precision=pg.PFAST_MIXED)
    sv.close()
    for k in ("gT", "gR", "gRT"):
        g, g0 = rm[k].cpu().numpy(), r0[k]
        assert np.linalg.norm(g - g0) <= 1e-4 * np.linalg.norm(g0), k
    assert abs(rm["Et"] - r0["Et"]) <= 1e-6 * abs(r0["Et"]) and abs(rm["Er"] - r0["Er"]) <= 1e-6 * abs(r0["Er"])

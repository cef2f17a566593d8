"""3D parity on the GPU: the CUDA kernels (through the C ABI) against the oracle.

Plain FP64 must be bit-identical (the library is built with -fmad=false, the
oracle with -ffp-contract=off).  The mixed FP32-bulk + FP64-polish mode must stay
within the stated tolerances: max relative traveltime error <= 1e-5 and gradient
relative L2 error <= 1e-4 against the FP64 oracle.
"""
import json
import os

import numpy as np
import pytest

from helpers import GOLDEN, bits_equal, case3d, picks_from

pytestmark = pytest.mark.gpu

TT_REL_TOL = 1e-5      # mixed mode: max |T - T_oracle| / T_oracle
GRAD_REL_L2_TOL = 1e-4  # mixed mode: ||g - g_oracle|| / ||g_oracle||


def _pg():
    import pfast_gb300 as pg
    return pg


def _torch():
    import torch
    return torch


def _oracle_case(shape, h, seed):
    from oracle import port
    vp, src, srnum, rec, nxyz, noise = case3d(shape, h, seed)
    Ts = [port.fsm3d(vp, src, s, 100, *h)[0] for s in range(len(srnum))]
    tobs = picks_from(Ts, src, srnum, rec, noise)
    return vp, src, srnum, rec, nxyz, tobs, Ts


CASES = [((9, 11, 13), (10.0, 10.0, 10.0), 101), ((9, 11, 13), (10.0, 12.5, 8.0), 102),
         ((17, 19, 23), (20.0, 20.0, 20.0), 103), ((2, 2, 2), (1.0, 1.0, 1.0), 104),
         ((10, 21, 70), (20.0, 20.0, 20.0), 105), ((5, 3, 33), (5.0, 7.0, 3.0), 106)]


@pytest.mark.parametrize("shape,h,seed", CASES)
def test_fsm3d_shim_bit_exact(shape, h, seed):
    pg = _pg()
    vp, src, srnum, rec, nxyz, tobs, Ts = _oracle_case(shape, h, seed)
    for s in range(len(srnum)):
        U = np.empty(shape)
        pg.fsm3d(vp, U, src, s, 100, h[0], h[1], h[2], shape[1], shape[2], shape[0])
        assert bits_equal(U, Ts[s]), (shape, s)


@pytest.mark.parametrize("shape,h,seed", CASES)
def test_adjoint3d_shim_bit_exact(shape, h, seed):
    from oracle import port
    pg = _pg()
    vp, src, srnum, rec, nxyz, tobs, Ts = _oracle_case(shape, h, seed)
    for s in range(len(srnum)):
        L_ref, E_ref, _ = port.adjoint3d(Ts[s], tobs, rec, nxyz, src, srnum, s, 100, *h)
        L = np.empty(shape)
        E = pg.adjoint_fsm3d(L, Ts[s], tobs, rec, nxyz, src, srnum, s, 100, h[0], h[1], h[2], shape[1], shape[2],
                             shape[0])
        assert bits_equal(L, L_ref), (shape, s)
        assert E == E_ref


def test_pins_against_reference_hashes(ctx):
    """The GPU reproduces the fields the reference itself produced (tests/golden/pins3d.json)."""
    import hashlib
    pg = _pg()
    pins = json.load(open(os.path.join(GOLDEN, "pins3d.json")))
    for c in pins:
        shape, h = tuple(c["shape"]), c["h"]
        vp, src, srnum, rec, nxyz, noise = case3d(shape, h, c["seed"])
        Ts = []
        for s in range(3):
            U = np.empty(shape)
            pg.fsm3d(vp, U, src, s, 100, h[0], h[1], h[2], shape[1], shape[2], shape[0])
            assert hashlib.sha256(U.tobytes()).hexdigest() == c["sources"][s]["T_sha"]
            Ts.append(U)
        tobs = picks_from(Ts, src, srnum, rec, noise)
        for s in range(3):
            L = np.empty(shape)
            E = pg.adjoint_fsm3d(L, Ts[s], tobs, rec, nxyz, src, srnum, s, 100, h[0], h[1], h[2], shape[1],
                                 shape[2], shape[0])
            assert hashlib.sha256(L.tobytes()).hexdigest() == c["sources"][s]["L_sha"]
            assert float(E).hex() == c["sources"][s]["EE_hex"]


@pytest.mark.parametrize("shape,h,seed", CASES)
def test_survey_eval_plain_bit_exact(ctx, shape, h, seed):
    from oracle import port
    pg, torch = _pg(), _torch()
    vp, src, srnum, rec, nxyz, tobs, Ts = _oracle_case(shape, h, seed)
    g_ref, e_ref, fi, ai = port.eval3d(vp, src, srnum, rec, nxyz, tobs, 100, *h)
    sv = pg.Survey3D(ctx, shape[1], shape[2], shape[0], h[0], h[1], h[2], src, srnum, rec, nxyz, tobs)
    g, e, st = sv.eval(torch.from_numpy(vp).cuda())
    assert bits_equal(g.cpu().numpy(), g_ref)
    assert e == e_ref
    assert st["fwd_iters_max"] == int(fi.max())
    assert st["adj_iters_max"] == int(ai.max())
    picks, _ = sv.forward(torch.from_numpy(vp).cuda())
    want = np.concatenate([Ts[s][rec[r, 2], rec[r, 0], rec[r, 1]][None] for s in range(3)
                           for r in range(sum(srnum[:s]), sum(srnum[:s + 1]))])
    assert bits_equal(picks.cpu().numpy(), want)


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_batch_split_does_not_change_bits(ctx, precision):
    # plain: one division per source in source order; mixed: the running lambda sum in source
    # order and one division at the end -- either way the split into batches changes no bit
    pg, torch = _pg(), _torch()
    prec = pg.PFAST_PLAIN_FP64 if precision == "plain" else pg.PFAST_MIXED
    shape, h = (10, 21, 70), (20.0, 20.0, 20.0)
    vp, src, srnum, rec, nxyz, tobs, Ts = _oracle_case(shape, h, 7)
    sv = pg.Survey3D(ctx, shape[1], shape[2], shape[0], *h, src, srnum, rec, nxyz, tobs)
    d = torch.from_numpy(vp).cuda()
    g_all, e_all, _ = sv.eval(d, precision=prec)
    g_one, e_one, st = sv.eval(d, precision=prec, max_batch=1)
    g_two, e_two, st2 = sv.eval(d, precision=prec, max_batch=2)
    assert st["batches"] == 3 and st2["batches"] == 2
    assert bits_equal(g_all.cpu().numpy(), g_one.cpu().numpy()) and e_all == e_one
    assert bits_equal(g_all.cpu().numpy(), g_two.cpu().numpy()) and e_all == e_two


@pytest.mark.parametrize("maxswp", [1, 2])
def test_iteration_cap_matches_oracle(ctx, maxswp):
    from oracle import port
    pg, torch = _pg(), _torch()
    shape, h = (9, 11, 13), (10.0, 10.0, 10.0)
    vp, src, srnum, rec, nxyz, tobs, Ts = _oracle_case(shape, h, 3)
    g_ref, e_ref, _, _ = port.eval3d(vp, src, srnum, rec, nxyz, tobs, maxswp, *h)
    sv = pg.Survey3D(ctx, shape[1], shape[2], shape[0], *h, src, srnum, rec, nxyz, tobs)
    g, e, st = sv.eval(torch.from_numpy(vp).cuda(), maxswp=maxswp)
    assert bits_equal(g.cpu().numpy(), g_ref) and e == e_ref
    assert st["not_converged"] > 0


def test_edge_receivers_duplicates_unpicked_and_at_source(ctx):
    """Receivers at the source node, two rows at one node (the later wins), a source with no
    picked receiver (no adjoint iteration at all) and an empty source."""
    from oracle import port
    pg, torch = _pg(), _torch()
    shape, h = (8, 9, 10), (10.0, 10.0, 10.0)
    rng = np.random.default_rng(5)
    vp = 1800.0 + 1000.0 * rng.random(shape)
    src = np.array([[4, 4, 0], [0, 9, 0], [8, 0, 0], [3, 3, 3]], np.int32)
    rows = [[(4, 4, 0), (4, 4, 0), (2, 2, 0), (2, 2, 0), (7, 8, 0)],   # at the source, duplicates
            [(1, 1, 0), (5, 5, 0)],                                      # all unpicked
            [],                                                          # no receivers
            [(0, 0, 0), (8, 9, 0), (0, 0, 0)]]
    srnum = np.array([len(r) for r in rows], np.int32)
    rec = np.array([x for r in rows for x in r], np.int32)
    nxyz = np.tile([0.0, 0.0, -1.0], (len(rec), 1))
    Ts = [port.fsm3d(vp, src, s, 100, *h)[0] for s in range(4)]
    ch0 = np.concatenate([[0], np.cumsum(srnum)])
    tobs = np.zeros(len(rec))
    for s in range(4):
        for r in range(ch0[s], ch0[s + 1]):
            tobs[r] = Ts[s][rec[r, 2], rec[r, 0], rec[r, 1]] + 0.003 * (r + 1)
    tobs[ch0[1]:ch0[2]] = 500.0
    g_ref, e_ref, _, ai = port.eval3d(vp, src, srnum, rec, nxyz, tobs, 100, *h)
    assert ai[1] == 0 and ai[2] == 0
    sv = pg.Survey3D(ctx, shape[1], shape[2], shape[0], *h, src, srnum, rec, nxyz, tobs)
    g, e, _ = sv.eval(torch.from_numpy(vp).cuda())
    assert bits_equal(g.cpu().numpy(), g_ref) and e == e_ref


def test_host_buffer_entry_matches_device_entry(ctx):
    pg, torch = _pg(), _torch()
    shape, h = (17, 19, 23), (20.0, 20.0, 20.0)
    vp, src, srnum, rec, nxyz, tobs, Ts = _oracle_case(shape, h, 8)
    g_h, e_h, _ = pg.eval3d_host(ctx, vp, *h, src, srnum, rec, nxyz, tobs)
    sv = pg.Survey3D(ctx, shape[1], shape[2], shape[0], *h, src, srnum, rec, nxyz, tobs)
    g_d, e_d, _ = sv.eval(torch.from_numpy(vp).cuda())
    assert bits_equal(g_h, g_d.cpu().numpy()) and e_h == e_d


def test_invalid_inputs_raise(ctx):
    pg = _pg()
    with pytest.raises(pg.PfastError):
        pg.Survey3D(ctx, 5, 5, 5, 1.0, 1.0, 1.0, np.array([[5, 0, 0]], np.int32), np.array([0], np.int32),
                    np.zeros((0, 3), np.int32))
    with pytest.raises(pg.PfastError):
        pg.Survey3D(ctx, 5, 1, 5, 1.0, 1.0, 1.0, np.array([[0, 0, 0]], np.int32), np.array([0], np.int32),
                    np.zeros((0, 3), np.int32))


def test_mixed_precision_within_tolerance(ctx):
    """FP32 bulk + FP64 polish on a smooth heterogeneous model, several tiles per axis."""
    from oracle import port
    from pfast_gb300 import synth
    pg, torch = _pg(), _torch()
    nz, nr, nc, hh = 24, 40, 72, 20.0
    vt = synth.true_model3d(nz, nr, nc, hh, seed=4)
    v0 = synth.gradient_model3d(nz, nr, nc, hh)
    src, srnum, rec, nxyz = synth.surface_survey3d(nr, nc, 2, 8)
    tobs = synth.add_noise(port.forward3d(vt, src, srnum, rec, 100, hh, hh, hh, nthreads=4), 0.002, 1)
    g_ref, e_ref, _, _ = port.eval3d(v0, src, srnum, rec, nxyz, tobs, 100, hh, hh, hh, nthreads=4)
    sv = pg.Survey3D(ctx, nr, nc, nz, hh, hh, hh, src, srnum, rec, nxyz, tobs)
    d = torch.from_numpy(v0).cuda()
    g, e, st = sv.eval(d, precision=pg.PFAST_MIXED)
    rel = np.linalg.norm(g.cpu().numpy() - g_ref) / np.linalg.norm(g_ref)
    assert rel <= GRAD_REL_L2_TOL, rel
    assert abs(e - e_ref) <= 1e-6 * abs(e_ref)
    picks_ref = port.forward3d(v0, src, srnum, rec, 100, hh, hh, hh, nthreads=4)
    picks, _ = sv.forward(d, precision=pg.PFAST_MIXED)
    assert np.max(np.abs(picks.cpu().numpy() - picks_ref) / picks_ref) <= TT_REL_TOL
    assert st["fwd32_iters_max"] > 0 and st["adj32_iters_max"] > 0


def test_persistent_schedule_matches_per_diagonal(ctx):
    """1600 sources on a 7 x 9 x 11 grid: more instances than resident blocks, so the persistent
    kernel's queue hands out several instances per block.  All three schedules (per diagonal,
    dataflow, hybrid) run the same ordered sweeps per source: plain and mixed results are
    bit-identical between them, and the plain ones equal the oracle's."""
    import torch
    from oracle import port
    pg = _pg()
    rng = np.random.default_rng(77)
    nz, nr, nc, h = 7, 9, 11, 10.0
    vp = 1500.0 + 2000.0 * rng.random((nz, nr, nc))
    nsrc = 1600
    src = np.stack([rng.integers(0, nr, nsrc), rng.integers(0, nc, nsrc), rng.integers(0, nz, nsrc)], 1).astype(np.int32)
    r1 = np.array([(i, j, 0) for i in range(0, nr, 3) for j in range(0, nc, 4)], np.int32)
    rec = np.concatenate([r1] * nsrc)
    srnum = np.full(nsrc, len(r1), np.int32)
    nxyz = np.tile([0.0, 0.0, -1.0], (len(rec), 1))
    tobs = 0.3 + 0.01 * rng.random(len(rec))
    sv = pg.Survey3D(ctx, nr, nc, nz, h, h, h, src, srnum, rec, nxyz, tobs)
    d_vp = torch.from_numpy(vp).cuda()
    out = {}
    for prec in (pg.PFAST_PLAIN_FP64, pg.PFAST_MIXED):
        for sched in (1, 2, 3):   # per diagonal, dataflow, hybrid
            g, e, st = sv.eval(d_vp, precision=prec, schedule=sched)
            pk, _ = sv.forward(d_vp, precision=prec, schedule=sched)
            out[prec, sched] = (g.cpu().numpy(), e, pk.cpu().numpy(), st)
    for prec in (pg.PFAST_PLAIN_FP64, pg.PFAST_MIXED):
        for sched in (2, 3):
            a, b = out[prec, 1], out[prec, sched]
            assert bits_equal(a[0], b[0]) and a[1] == b[1] and bits_equal(a[2], b[2])
            assert a[3]["fwd_iters_max"] == b[3]["fwd_iters_max"] and a[3]["not_converged"] == b[3]["not_converged"] == 0
    g0, e0, _, _ = port.eval3d(vp, src, srnum, rec, nxyz, tobs, 100, h, h, h, nthreads=8)
    assert bits_equal(out[pg.PFAST_PLAIN_FP64, 2][0], g0) and out[pg.PFAST_PLAIN_FP64, 2][1] == e0
    sv.close()


@pytest.mark.parametrize("shape,h", [((22, 40, 100), (20.0, 20.0, 20.0)), ((13, 17, 70), (10.0, 12.5, 8.0))])
def test_dataflow_schedule_matches_per_diagonal_on_many_tiles(ctx, shape, h):
    """A grid of 6 x 5 x 4 (and 4 x 3 x 3) tiles with a few sources: in the dataflow schedule
    one block solves a source with its sweep orders overlapping as the tile dependencies allow;
    the hybrid runs the first outer iteration per diagonal and continues in the dataflow kernel.
    Plain and mixed fields, gradients, misfits and iteration counts are bit-identical to the
    per-diagonal launches, and plain equals the oracle."""
    import torch
    from oracle import port
    pg = _pg()
    vp, src, srnum, rec, nxyz, tobs, Ts = _oracle_case(shape, h, 31)
    nz, nr, nc = shape
    sv = pg.Survey3D(ctx, nr, nc, nz, *h, src, srnum, rec, nxyz, tobs)
    d_vp = torch.from_numpy(vp).cuda()
    out = {}
    for prec in (pg.PFAST_PLAIN_FP64, pg.PFAST_MIXED):
        for sched in (1, 2, 3):   # per diagonal, dataflow, hybrid
            g, e, st = sv.eval(d_vp, precision=prec, schedule=sched)
            pk, _ = sv.forward(d_vp, precision=prec, schedule=sched)
            out[prec, sched] = (g.cpu().numpy(), e, pk.cpu().numpy(), st)
        a = out[prec, 1]
        for sched in (2, 3):
            b = out[prec, sched]
            assert bits_equal(a[0], b[0]) and a[1] == b[1] and bits_equal(a[2], b[2])
            for k in ("fwd_iters_max", "adj_iters_max", "fwd32_iters_max", "adj32_iters_max", "fwd_node_updates",
                      "adj_node_updates", "not_converged"):
                assert a[3][k] == b[3][k], (sched, k)
            assert b[3]["launches"] < a[3]["launches"] if sched == 2 else b[3]["launches"] <= a[3]["launches"]
        assert a[3]["not_converged"] == 0 and a[3]["adj32_iters_max"] < 20 and a[3]["fwd32_iters_max"] < 20
    g0, e0, _, _ = port.eval3d(vp, src, srnum, rec, nxyz, tobs, 100, *h, nthreads=8)
    assert bits_equal(out[pg.PFAST_PLAIN_FP64, 2][0], g0) and out[pg.PFAST_PLAIN_FP64, 2][1] == e0
    # an iteration cap: every schedule stops after the same two iterations with the same fields
    g1, e1, s1 = sv.eval(d_vp, precision=pg.PFAST_PLAIN_FP64, maxswp=2, schedule=1)
    for sched in (2, 3):
        g2, e2, s2 = sv.eval(d_vp, precision=pg.PFAST_PLAIN_FP64, maxswp=2, schedule=sched)
        assert bits_equal(g1.cpu().numpy(), g2.cpu().numpy()) and e1 == e2
        assert s1["not_converged"] == s2["not_converged"] and s1["fwd_iters_max"] == s2["fwd_iters_max"] <= 2
    sv.close()


def test_near_source_initialisation_reduces_the_source_error(ctx):
    """Opt-in near-source start (not in the reference): in a homogeneous medium, where the exact
    traveltime is distance / v, starting the nodes within 4 nodes of the source from the
    straight-ray time cuts the first-order scheme's error; the mixed path with the same option
    stays within the usual 1e-5 of the plain one; radius 0 is the reference's point source."""
    import torch
    pg = _pg()
    n, h, v = 33, 10.0, 2000.0
    vp = np.full((n, n, n), v)
    src = np.array([[16, 16, 16], [0, 0, 0], [5, 30, 12]], np.int32)   # (row, col, z)
    g = np.arange(0, n, 2)
    r1 = np.array([(i, j, k) for k in g for i in g for j in g], np.int32)
    rec = np.concatenate([r1] * len(src))
    srnum = np.full(len(src), len(r1), np.int32)
    sv = pg.Survey3D(ctx, n, n, n, h, h, h, src, srnum, rec)
    d_vp = torch.from_numpy(vp).cuda()
    s = np.repeat(src, len(r1), axis=0)
    dist = h * np.sqrt(((rec - s) ** 2).sum(1).astype(float))
    exact = dist / v
    far = dist > 6 * h                     # outside every fixed region
    err = {}
    for r in (0, 4):
        pk, _ = sv.forward(d_vp, precision=pg.PFAST_PLAIN_FP64, near_source_radius=r)
        pk = pk.cpu().numpy()
        err[r] = np.max(np.abs(pk[far] - exact[far]) / exact[far])
        if r:
            near = (dist > 0) & (dist <= r * h)
            assert np.allclose(pk[near], exact[near], rtol=1e-12)   # straight-ray values, exact here
            pm, _ = sv.forward(d_vp, precision=pg.PFAST_MIXED, near_source_radius=r)
            assert np.max(np.abs(pm.cpu().numpy() - pk) / np.maximum(pk, 1e-30)) <= 1e-5
    assert err[4] < 0.5 * err[0], err
    # radius 0 keeps the reference's point source: identical to the default call
    p0, _ = sv.forward(d_vp, precision=pg.PFAST_PLAIN_FP64)
    p1, _ = sv.forward(d_vp, precision=pg.PFAST_PLAIN_FP64, near_source_radius=0)
    assert bits_equal(p0.cpu().numpy(), p1.cpu().numpy())
    sv.close()


@pytest.mark.parametrize("shape,h", [((22, 40, 100), (20.0, 20.0, 20.0)), ((13, 17, 70), (10.0, 12.5, 8.0))])
def test_tile_shapes_give_identical_plain_bits(ctx, shape, h):
    """The sweeps in 4x8x32 and in 8x4x32 tiles, each per diagonal and persistent: every node
    still sees its upstream neighbours' new values and its downstream ones' old values, so the
    plain FP64 fields, gradients, misfits and iteration counts are bit-identical across the four
    (schedule, tile shape) pairs and equal the oracle.  The mixed mode's FP64 polish selects
    sweep orders per tile, so its bits may differ between shapes (not between the schedules of
    one shape) but stay within the mixed-mode tolerances of the oracle."""
    import torch
    from oracle import port
    pg = _pg()
    vp, src, srnum, rec, nxyz, tobs, Ts = _oracle_case(shape, h, 32)
    nz, nr, nc = shape
    sv = pg.Survey3D(ctx, nr, nc, nz, *h, src, srnum, rec, nxyz, tobs)
    d_vp = torch.from_numpy(vp).cuda()
    g0, e0, _, _ = port.eval3d(vp, src, srnum, rec, nxyz, tobs, 100, *h, nthreads=8)
    picks0 = port.forward3d(vp, src, srnum, rec, 100, *h, nthreads=8)
    out = {}
    for prec in (pg.PFAST_PLAIN_FP64, pg.PFAST_MIXED):
        for tile in (pg._capi.PFAST_TILE_4x8x32, pg._capi.PFAST_TILE_8x4x32):
            for sched in (pg._capi.PFAST_SCHEDULE_DIAGONAL, pg._capi.PFAST_SCHEDULE_PERSISTENT):
                g, e, st = sv.eval(d_vp, precision=prec, schedule=sched, tile_shape=tile)
                pk, _ = sv.forward(d_vp, precision=prec, schedule=sched, tile_shape=tile)
                out[prec, tile, sched] = (g.cpu().numpy(), e, pk.cpu().numpy(), st)
                assert st["not_converged"] == 0
    plain = [v for k, v in out.items() if k[0] == pg.PFAST_PLAIN_FP64]
    for g, e, pk, st in plain:
        assert bits_equal(g, g0) and e == e0 and bits_equal(pk, picks0)
        for k in ("fwd_iters_max", "adj_iters_max"):
            assert st[k] == plain[0][3][k], k
    for tile in (1, 2):
        a, b = out[pg.PFAST_MIXED, tile, 1], out[pg.PFAST_MIXED, tile, 2]
        assert bits_equal(a[0], b[0]) and a[1] == b[1] and bits_equal(a[2], b[2])
        assert np.linalg.norm(a[0] - g0) / np.linalg.norm(g0) <= GRAD_REL_L2_TOL
        assert np.max(np.abs(a[2] - picks0) / np.maximum(picks0, 1e-30)) <= TT_REL_TOL   # a receiver at a source: 0
        assert abs(a[1] - e0) <= 1e-6 * abs(e0)
    with pytest.raises(pg.PfastError) as ei:
        sv.eval(d_vp, tile_shape=3)
    assert ei.value.status == pg._capi.PFAST_ERR_INVALID
    sv.close()


@pytest.mark.parametrize("shape,h,seed", CASES)
def test_every_schedule_and_tile_shape_on_small_and_ragged_grids(ctx, shape, h, seed):
    """The parity grids (down to 2 x 2 x 2, ragged tiles in every axis) under each schedule and
    tile shape: plain FP64 equals the oracle bit for bit; in the mixed mode, whose polish
    differs between tile shapes, the three schedules of one shape agree bit for bit (the
    dataflow kernel keeps the polish field in register windows, the others in a box)."""
    import torch
    from oracle import port
    pg = _pg()
    vp, src, srnum, rec, nxyz, tobs, Ts = _oracle_case(shape, h, seed)
    nz, nr, nc = shape
    sv = pg.Survey3D(ctx, nr, nc, nz, *h, src, srnum, rec, nxyz, tobs)
    d_vp = torch.from_numpy(vp).cuda()
    g0, e0, _, _ = port.eval3d(vp, src, srnum, rec, nxyz, tobs, 100, *h, nthreads=4)
    for tile in (1, 2):
        mixed = []
        for sched in (1, 2, 3):
            g, e, st = sv.eval(d_vp, precision=pg.PFAST_PLAIN_FP64, schedule=sched, tile_shape=tile)
            assert bits_equal(g.cpu().numpy(), g0) and e == e0, (tile, sched)
            gm, em, sm = sv.eval(d_vp, precision=pg.PFAST_MIXED, schedule=sched, tile_shape=tile)
            mixed.append((gm.cpu().numpy(), em, sm["not_converged"]))
        for gm, em, nc_ in mixed[1:]:
            assert bits_equal(gm, mixed[0][0]) and em == mixed[0][1] and nc_ == mixed[0][2] == 0, tile
    sv.close()


def test_dataflow_alternating_grid_sizes(ctx):
    """The dataflow kernel's shared memory grows with the grid's tile count; a larger grid's
    launch after a smaller grid's (launch shapes cached per grid and source count) still runs."""
    import torch
    pg = _pg()
    out = []
    for shape in ((22, 40, 100), (9, 11, 13), (22, 40, 100)):
        h = (20.0, 20.0, 20.0)
        vp, src, srnum, rec, nxyz, noise = case3d(shape, h, 51)
        sv = pg.Survey3D(ctx, shape[1], shape[2], shape[0], *h, src[:2], srnum[:2], rec[:int(srnum[:2].sum())],
                         nxyz[:int(srnum[:2].sum())], 0.2 + noise[:int(srnum[:2].sum())])
        g, e, st = sv.eval(torch.from_numpy(vp).cuda(), precision=pg.PFAST_MIXED, schedule=2)
        out.append((g.cpu().numpy(), e))
        sv.close()
    assert bits_equal(out[0][0], out[2][0]) and out[0][1] == out[2][1]


def test_schedule_autotune(ctx):
    """pfast_survey3d_autotune times the four (schedule, tile shape) candidates on the same
    evaluation; automatic evaluations afterwards use the fastest per phase: plain FP64 stays
    bit-identical to the oracle and the mixed mode within its tolerances."""
    import torch
    from oracle import port
    pg = _pg()
    h = (10.0, 10.0, 10.0)
    vp, src, srnum, rec, nxyz, noise = case3d((12, 16, 20), h, 41)
    tobs = 0.2 + noise
    sv = pg.Survey3D(ctx, 16, 20, 12, *h, src, srnum, rec, nxyz, tobs)
    d_vp = torch.from_numpy(vp).cuda()
    g0, e0, _, _ = port.eval3d(vp, src, srnum, rec, nxyz, tobs, 100, *h, nthreads=8)
    for prec in (pg.PFAST_PLAIN_FP64, pg.PFAST_MIXED):
        t = sv.autotune(d_vp, precision=prec)
        assert set(t) == set(pg._capi.PFAST_TUNE_CANDIDATES)
        assert all(v["ms_total"] > 0 for v in t.values())
        g, e, st = sv.eval(d_vp, precision=prec)
        g = g.cpu().numpy()
        picks = pg._capi.phase_candidates(st)   # every sweep kind that ran names a candidate
        assert set(picks) == ({"fwd64_plain", "adj64_plain"} if prec == pg.PFAST_PLAIN_FP64 else
                              {"fwd32", "fwd64_polish", "adj32", "adj64_polish"})
        assert set(picks.values()) <= set(pg._capi.PFAST_TUNE_CANDIDATES)
        if prec == pg.PFAST_PLAIN_FP64:
            assert bits_equal(g, g0) and e == e0
        else:
            assert np.linalg.norm(g - g0) / np.linalg.norm(g0) <= GRAD_REL_L2_TOL and st["not_converged"] == 0
    sv.close()


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_graph_replay_matches_launches(ctx, precision):
    # per-diagonal outer iterations replayed as captured CUDA graphs give the bits (and the
    # iteration counts) of launching the kernels one by one
    pg, torch = _pg(), _torch()
    prec = pg.PFAST_PLAIN_FP64 if precision == "plain" else pg.PFAST_MIXED
    shape, h = (12, 18, 40), (20.0, 20.0, 20.0)
    vp, src, srnum, rec, nxyz, tobs, Ts = _oracle_case(shape, h, 11)
    sv = pg.Survey3D(ctx, shape[1], shape[2], shape[0], *h, src, srnum, rec, nxyz, tobs)
    d = torch.from_numpy(vp).cuda()
    try:
        ctx.set_graphs(False)
        g0, e0, s0 = sv.eval(d, precision=prec, schedule=1)
        ctx.set_graphs(True)
        g1, e1, s1 = sv.eval(d, precision=prec, schedule=1)   # phases captured the second time
        g2, e2, s2 = sv.eval(d, precision=prec, schedule=1)   # their shapes come up, then replayed
    finally:
        ctx.set_graphs(True)
    assert bits_equal(g0.cpu().numpy(), g1.cpu().numpy()) and e0 == e1
    assert bits_equal(g0.cpu().numpy(), g2.cpu().numpy()) and e0 == e2
    for k in ("fwd_iters_max", "adj_iters_max", "fwd32_iters_max", "adj32_iters_max", "launches"):
        assert s0[k] == s1[k] == s2[k], k


def test_full_size_grid(ctx):
    """The grid of the 3D gradient workload at full size (256 x 256 x 128 nodes, h = 20 m, 4096
    receivers per source), with 4 sources: plain FP64 equals the oracle on one source (gradient,
    misfit and picks bit for bit); mixed stays within the tolerances of plain on all four; the
    mixed bits do not depend on the batch split."""
    from oracle import port
    from pfast_gb300 import workloads
    pg, torch = _pg(), _torch()
    vt, v0, src, srnum, rec, nxyz = workloads.c3_inputs(n_src_side=2, n_rec_side=64)
    nz, nr, nc = v0.shape
    h = workloads.H
    assert (nz, nr, nc) == (128, 256, 256) and len(srnum) == 4 and srnum[0] == 4096
    tobs = workloads.observed_picks(ctx, vt, src, srnum, rec, pg.PFAST_PLAIN_FP64)
    d = torch.from_numpy(v0).cuda()

    # one source, plain, against the oracle
    n0 = int(srnum[0])
    sv1 = pg.Survey3D(ctx, nr, nc, nz, h, h, h, src[:1], srnum[:1], rec[:n0], nxyz[:n0], tobs[:n0])
    g1, e1, _ = sv1.eval(d, precision=pg.PFAST_PLAIN_FP64)
    p1, _ = sv1.forward(d, precision=pg.PFAST_PLAIN_FP64)
    sv1.close()
    g_ref, e_ref, _, _ = port.eval3d(v0, src[:1], srnum[:1], rec[:n0], nxyz[:n0], tobs[:n0], 100, h, h, h)
    p_ref = port.forward3d(v0, src[:1], srnum[:1], rec[:n0], 100, h, h, h)
    assert bits_equal(g1.cpu().numpy(), g_ref) and e1 == e_ref
    assert bits_equal(p1.cpu().numpy(), p_ref)

    # four sources: mixed against plain, and the batch split
    sv = pg.Survey3D(ctx, nr, nc, nz, h, h, h, src, srnum, rec, nxyz, tobs)
    gp, ep, _ = sv.eval(d, precision=pg.PFAST_PLAIN_FP64)
    pp, _ = sv.forward(d, precision=pg.PFAST_PLAIN_FP64)
    gm, em, _ = sv.eval(d, precision=pg.PFAST_MIXED)
    gm1, em1, st1 = sv.eval(d, precision=pg.PFAST_MIXED, max_batch=1)
    assert st1["not_converged"] == 0 and st1["adj32_iters_max"] < 20 and st1["adj_iters_max"] < 20
    pm, _ = sv.forward(d, precision=pg.PFAST_MIXED)
    sv.close()
    gp, gm, pp, pm = gp.cpu().numpy(), gm.cpu().numpy(), pp.cpu().numpy(), pm.cpu().numpy()
    assert np.all(np.isfinite(pm)) and np.all(pm > 0)
    assert np.max(np.abs(pm - pp) / pp) <= TT_REL_TOL
    assert np.linalg.norm(gm - gp) / np.linalg.norm(gp) <= GRAD_REL_L2_TOL
    assert abs(em - ep) <= 1e-6 * abs(ep)
    assert st1["batches"] == 4
    assert bits_equal(gm, gm1.cpu().numpy()) and em == em1

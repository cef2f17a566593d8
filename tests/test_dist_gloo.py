"""Sources sharded over two processes (gloo, CPU): the reference's contiguous source
partition and the fixed-order reduction of the partial gradients and misfits.
Each rank computes its block with the oracle; the reduced result must equal the
rank-ordered sum of the blocks exactly and the single-process result to 1e-12."""
import os
import socket

import numpy as np
import pytest

from pfast_gb300 import dist as pdist


def test_loc_srcid_matches_the_reference_partition():
    # src/T_PFAST3D.cpp:221-236: 10 sources on 4 ranks -> 3, 3, 2, 2
    assert pdist.loc_srcid(10, 4) == [3, 6, 8, 10]
    assert pdist.loc_srcid(8, 4) == [2, 4, 6, 8]
    assert pdist.loc_srcid(3, 4) == [1, 2, 3, 3]
    assert [pdist.source_block(10, r, 4) for r in range(4)] == [(0, 3), (3, 6), (6, 8), (8, 10)]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _case():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from helpers import case3d, picks_from
    from oracle import port
    h = (10.0, 10.0, 10.0)
    vp, src, srnum, rec, nxyz, noise = case3d((7, 9, 11), h, 17)
    Ts = [port.fsm3d(vp, src, s, 100, *h)[0] for s in range(3)]
    tobs = picks_from(Ts, src, srnum, rec, noise)
    return vp, src, srnum, rec, nxyz, tobs, h


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from oracle import port as oport
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        vp, src, srnum, rec, nxyz, tobs, h = _case()
        b, e = pdist.source_block(len(srnum), rank, world)
        g, m, _, _ = oport.eval3d(vp, src, srnum, rec, nxyz, tobs, 100, *h, s_begin=b, s_end=e)
        grad, misfit = pdist.reduce_gradient(g, m)
        q.put((rank, b, e, grad, misfit))
    finally:
        dist.destroy_process_group()


def test_two_rank_reduction_equals_rank_ordered_sum():
    import multiprocessing as mp
    from oracle import port as oport
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    vp, src, srnum, rec, nxyz, tobs, h = _case()
    parts = []
    for rank, b, e, _, _ in res:
        g, m, _, _ = oport.eval3d(vp, src, srnum, rec, nxyz, tobs, 100, *h, s_begin=b, s_end=e)
        parts.append((g, m))
    want_g = parts[0][0] + parts[1][0]
    want_m = parts[0][1] + parts[1][1]
    for _, _, _, grad, misfit in res:   # both ranks hold the same reduced result
        assert np.array_equal(grad, want_g) and misfit == want_m
    g1, m1, _, _ = oport.eval3d(vp, src, srnum, rec, nxyz, tobs, 100, *h)
    assert np.linalg.norm(res[0][3] - g1) <= 1e-12 * np.linalg.norm(g1)
    assert abs(res[0][4] - m1) <= 1e-12 * abs(m1)

"""The request server on the GPU (pfast_server_*): continuous batching of forward and
gradient requests of different sizes and dimensions.

* Each request's result is the same alone and in the mix: a mix of 3D and 2D, forward and
  gradient, plain and mixed-precision requests run with 4 slots under a tight HBM budget
  (so admission waits and batches shrink) must give the same bits as the same requests
  run one at a time, and as the direct survey API.
* Admission stays inside the budget; oversized requests and unknown IDs are rejected;
  unused resident data is evicted least recently used first.
"""
import numpy as np
import pytest

from helpers import bits_equal, case3d, picks_from

pytestmark = pytest.mark.gpu


def _pg():
    import pfast_gb300 as pg
    return pg


def _models():
    from oracle import port
    out = {}
    for key, (shape, h, seed) in {"a": ((9, 11, 13), (10.0, 10.0, 10.0), 5), "b": ((12, 16, 20), (20.0, 20.0, 10.0), 6)}.items():
        vp, src, srnum, rec, nxyz, noise = case3d(shape, h, seed)
        Ts = [port.fsm3d(vp, src, s, 100, *h)[0] for s in range(len(srnum))]
        tobs = picks_from(Ts, src, srnum, rec, noise)
        out[key] = dict(vp=vp * 1.03, shape=shape, h=h, src=src, srnum=srnum, rec=rec, nxyz=nxyz, tobs=tobs)
    return out


def _model2d():
    from oracle import port
    nr, nc, h = 40, 90, 10.0
    vp = 1700.0 + 25.0 * np.arange(nr)[:, None] + np.zeros((1, nc))
    Z = np.stack([np.full(nc, 250.0), -np.ones(nc), np.zeros(nc)], 1)
    src = np.array([[0, 10], [0, 45], [0, 80]], np.int32)
    rec = np.array([(0, j) for j in range(0, nc, 3)] * 3, np.int32)
    srnum = np.full(3, nc // 3, np.int32)
    nxy = np.tile([-1.0, 0.0], (len(rec), 1))
    Tr, _ = port.forward2d(vp * 0.97, Z, src, srnum, rec, 1, 500, h, h)
    return dict(vp=vp, Z=Z, src=src, srnum=srnum, rec=rec, nxy=nxy, tt=Tr[:, 0], tr=Tr[:, 1:], h=h, shape=(nr, nc))


def _populate(srv, m3, m2):
    for k, (mid, sid) in {"a": (1, 11), "b": (2, 12)}.items():
        m = m3[k]
        srv.put_model(mid, m["vp"], m["h"])
        srv.put_survey3d(sid, m["shape"], m["h"], m["src"], m["srnum"], m["rec"], m["nxyz"], m["tobs"])
    srv.put_model(3, m2["vp"], (m2["h"], m2["h"]), WR=0.5)
    srv.put_survey2d(13, m2["shape"], (m2["h"], m2["h"]), m2["src"], m2["srnum"], m2["rec"], numofr=1, Z=m2["Z"],
                     nxy=m2["nxy"], tt_obs=m2["tt"], tr_obs=m2["tr"])


MIX = [("grad", 1, 11, 1), ("fwd", 2, 12, 1), ("grad", 3, 13, 0), ("fwd", 1, 11, 0), ("grad", 2, 12, 1),
       ("fwd", 3, 13, 1), ("grad", 1, 11, 0), ("grad", 2, 12, 0), ("fwd", 2, 12, 0), ("grad", 3, 13, 1),
       ("fwd", 1, 11, 1), ("grad", 1, 11, 1)]


def _submit_all(srv):
    pg = _pg()
    tickets = []
    for kind, mid, sid, prec in MIX:
        p = pg.PFAST_MIXED if prec else pg.PFAST_PLAIN_FP64
        tickets.append(srv.submit_gradient(mid, sid, p) if kind == "grad" else srv.submit_forward(mid, sid, p))
    return [t.result() for t in tickets]


def test_results_are_the_same_alone_and_in_the_mix(ctx):
    pg = _pg()
    m3, m2 = _models(), _model2d()
    # alone: one slot, requests one after another
    alone_srv = pg.Server(slots=1, hbm_budget_gb=8.0)
    _populate(alone_srv, m3, m2)
    alone = []
    for kind, mid, sid, prec in MIX:
        p = pg.PFAST_MIXED if prec else pg.PFAST_PLAIN_FP64
        t = alone_srv.submit_gradient(mid, sid, p) if kind == "grad" else alone_srv.submit_forward(mid, sid, p)
        alone.append(t.result())
    alone_srv.close()
    # in the mix: 4 slots, all submitted at once, a budget small enough that admission waits
    # and batches shrink (model b: 3 sources need ~3 x 170 KB per gradient batch)
    srv = pg.Server(slots=4, hbm_budget_gb=0.004)
    _populate(srv, m3, m2)
    mixed = _submit_all(srv)
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(MIX) and st["failed"] == 0
    assert st["peak_bytes"] <= st["budget_bytes"]
    batches = [r[2]["batch"] for r in mixed]
    assert min(batches) >= 1
    for (o1, e1, _), (o2, e2, _) in zip(alone, mixed):
        assert bits_equal(o1, o2)
        assert e1 == e2
    # and as the direct survey API computes them
    import torch
    m = m3["a"]
    sv = pg.Survey3D(ctx, m["shape"][1], m["shape"][2], m["shape"][0], *m["h"], m["src"], m["srnum"], m["rec"],
                     m["nxyz"], m["tobs"])
    g, e, _ = sv.eval(torch.from_numpy(m["vp"]).cuda(), precision=pg.PFAST_MIXED)
    assert bits_equal(g.cpu().numpy(), alone[0][0]) and e == alone[0][1]
    sv.close()


def test_latency_accounting_and_overlap():
    """Requests report queue and run times; with several slots the mix finishes sooner than the
    sum of its run times (the requests overlap on the device)."""
    pg = _pg()
    m3, m2 = _models(), _model2d()
    srv = pg.Server(slots=4, hbm_budget_gb=8.0)
    _populate(srv, m3, m2)
    _submit_all(srv)   # warm-up (diagonal tables, allocations)
    import time
    t0 = time.perf_counter()
    res = _submit_all(srv)
    wall = (time.perf_counter() - t0) * 1e3
    srv.close()
    info = [r[2] for r in res]
    assert all(i["total_ms"] >= i["run_ms"] >= 0 and i["queue_ms"] >= 0 for i in info)
    assert wall < sum(i["run_ms"] for i in info)


def test_admission_errors_and_eviction():
    pg = _pg()
    m3 = _models()
    m = m3["b"]
    srv = pg.Server(slots=2, hbm_budget_gb=0.0006)   # 600 KB
    srv.put_model(2, m["vp"], m["h"])
    srv.put_survey3d(12, m["shape"], m["h"], m["src"], m["srnum"], m["rec"], m["nxyz"], m["tobs"])
    with pytest.raises(pg.PfastError) as e:            # one source of a gradient needs more than the budget
        srv.submit_gradient(2, 12)
    assert e.value.status == 3
    with pytest.raises(pg.PfastError) as e:
        srv.submit_forward(99, 12)
    assert e.value.status == 1
    # models fill the budget: the least recently used unused one is evicted
    for mid in (20, 21, 22, 23):
        srv.put_model(mid, m["vp"], m["h"])        # 30.7 KB each
    st = srv.stats()
    assert st["used_bytes"] <= st["budget_bytes"]
    big = np.full((40, 40, 40), 2000.0)               # 512 KB: evicts older entries to fit
    srv.put_model(30, big, (10.0, 10.0, 10.0))
    st2 = srv.stats()
    assert st2["resident_models"] < st["resident_models"] + 1 and st2["used_bytes"] <= st2["budget_bytes"]
    srv.close()

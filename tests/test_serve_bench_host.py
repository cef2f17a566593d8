"""Host-side logic of the serving benchmark (pfast_gb300/serve_bench.py), on CPU: the per-rate
summary of a request stream and the knee rule (p99 above three times the lowest rate's, or
completions falling behind the stream's actual arrivals)."""
import numpy as np

from pfast_gb300 import serve_bench as sb


def _records(n, latency_ms, lag_ms=0.0, failed=0, kind="grad", nsrc=4):
    recs = [{"ok": True, "latency_ms": latency_ms, "queue_ms": 1.0, "nsrc": nsrc, "kind": kind, "lag_ms": lag_ms}
            for _ in range(n)]
    recs += [{"ok": False, "latency_ms": 0.0, "queue_ms": 0.0, "nsrc": nsrc, "kind": kind, "lag_ms": lag_ms}
             for _ in range(failed)]
    return recs


def test_summary_counts_solves_and_rates():
    recs = _records(10, 50.0, failed=2) + _records(5, 100.0, kind="fwd", nsrc=2)
    s = sb.summarize(recs, wall_s=2.0, rate=8.0, duration=2.0)
    assert s["requests"] == 17 and s["failed"] == 2
    assert s["requests_per_s"] == 15 / 2.0
    # a gradient request is a forward and an adjoint solve per source
    assert s["solves_per_s"] == (10 * 4 * 2 + 5 * 2) / 2.0
    assert s["arrival_rate"] == 17 / 2.0
    assert np.isclose(s["p50_ms"], 50.0) and s["p99_ms"] <= 100.0


def test_knee_rule():
    def row(rate, p99, served, arrived):
        return {"offered_rate": rate, "p99_ms": p99, "requests_per_s": served, "arrival_rate": arrived}
    # p99 grows past three times the lowest rate's
    assert sb.knee([row(4, 100, 4, 4), row(16, 250, 16, 16), row(32, 310, 31, 32)]) == 32
    # completions fall behind the arrivals first
    assert sb.knee([row(4, 100, 4, 4), row(16, 120, 13, 16), row(32, 500, 20, 32)]) == 16
    # not reached, and an empty sweep
    assert sb.knee([row(4, 100, 4, 4), row(8, 150, 8, 8)]) is None
    assert sb.knee([]) is None

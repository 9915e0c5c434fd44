"""The serving report's latency attribution (shard.latency_attribution): a
band of requests between two latency quantiles, its mean latency, queueing
and phases. Synthetic request times, no GPU."""
import math
import os
import random
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "apogee-vm_gb300"))

import shard  # noqa: E402


def _times(n=200, seed=5):
    rng = random.Random(seed)
    out = {}
    for i in range(n):
        submit = rng.randrange(10**9)
        queue = rng.randrange(0, 5 * 10**8)
        phases = [rng.uniform(1, 60) for _ in range(4)]
        run_ns = int(sum(phases) * 1e6) + rng.randrange(10**6)
        out[i] = {"submit_ns": submit, "admit_ns": submit + queue, "done_ns": submit + queue + run_ns,
                  "phase_ms": phases}
    return out


def test_band_is_the_quantile_range_and_queue_stays_below_latency():
    times = _times()
    lat = sorted((tm["done_ns"] - tm["submit_ns"]) / 1e6 for tm in times.values())
    for lo, hi in ((0.99, 1.0), (0.45, 0.55), (0.0, 1.0)):
        a = shard.latency_attribution(times, lo, hi)
        assert a["quantiles"] == [lo, hi]
        # Every request's latency is its queueing plus its run, so the band's
        # means keep that order.
        assert a["queue_ms"] <= a["latency_ms"]
        assert a["queue_ms"] + sum(a[k] for k in ("commit_ms", "forward_ms", "gkr_ms", "open_ms")) <= \
            a["latency_ms"] + 1e-9
        assert lat[0] <= a["latency_ms"] <= lat[-1]
    # The band starts at the nearest-rank quantile (the element the p99 of
    # shard.percentile is): index ceil(0.99 * 200) - 1 = 197.
    top = shard.latency_attribution(times, 0.99, 1.0)
    assert top["requests"] == 3 and abs(top["latency_ms"] - sum(lat[197:]) / 3) < 1e-9
    assert lat[197] == shard.percentile(lat, 0.99)
    mid = shard.latency_attribution(times, 0.45, 0.55)
    lo, hi = math.ceil(0.45 * 200) - 1, math.ceil(0.55 * 200)
    assert mid["requests"] == hi - lo
    assert abs(mid["latency_ms"] - sum(lat[lo:hi]) / (hi - lo)) < 1e-9


def test_empty_and_single():
    assert shard.latency_attribution({}, 0.5, 0.6) == {}
    one = _times(1)
    a = shard.latency_attribution(one, 0.99, 1.0)
    assert a["requests"] == 1

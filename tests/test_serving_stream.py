"""The seeded serving stream (CPU): Poisson arrivals, the 40/40/20 request mix, the
ranges of tile sizes and iteration budgets, and refinements that name one of the 16
latest earlier previews."""
import numpy as np

from syfrack_gb300 import workloads


def test_stream_is_seeded_and_mixed():
    a = workloads.serving_stream(seed=3, rate=200.0, duration=10.0)
    b = workloads.serving_stream(seed=3, rate=200.0, duration=10.0)
    assert [(t, k) for t, k, _ in a] == [(t, k) for t, k, _ in b]
    n = len(a)
    assert 1800 < n < 2200  # Poisson(2000)
    times = np.array([t for t, _, _ in a])
    assert np.all(np.diff(times) > 0) and times[-1] < 10.0
    gaps = np.diff(times)
    assert abs(gaps.mean() - 1 / 200.0) < 0.1 / 200.0
    kinds = [k for _, k, _ in a]
    frac = {k: kinds.count(k) / n for k in ("tile", "preview", "refine")}
    assert abs(frac["tile"] - 0.4) < 0.04 and abs(frac["preview"] - 0.4) < 0.04 and abs(frac["refine"] - 0.2) < 0.03


def test_stream_payloads():
    ev = workloads.serving_stream(seed=4, rate=200.0, duration=5.0)
    previews = []
    for i, (_, kind, payload) in enumerate(ev):
        if kind == "tile":
            f, c = payload
            assert f.family in ("Julia", "BurningShip")
            assert 1000 <= f.iterations <= 20000
            assert 256 <= c.width <= 2048 and c.width == c.height
        elif kind == "preview":
            sc, cfg = payload
            assert (cfg.width, cfg.height, cfg.samples_per_pixel, cfg.max_bounces) == (480, 270, 1, 1)
            previews.append(i)
        else:
            assert payload in previews[-workloads.SERVE_REFINE_WINDOW:]

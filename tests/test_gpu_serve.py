"""Serving (GPU): a request's result is the same alone and in a mix of other
requests (bit-exact: the same kernel runs each path and pixel, and each pixel sums
its samples in ascending order), refinements accumulate in submission order on the
film their preview left on the device, admission waits for the HBM budget, and a
preview or tile matches the plain drop-in calls."""
import numpy as np
import pytest

from syfrack_gb300 import Canvas, PlanarFractal, RenderSession, Server, SyfrackError, escape2d, workloads
from syfrack_gb300.serve import DONE, QUEUED

pytestmark = pytest.mark.gpu

GB = 1 << 30


def small_preview(i, side=(64, 40)):
    graphs = workloads.serving_graphs()
    rng = np.random.default_rng(100 + i)
    sc, cfg = workloads._preview_scene(rng, graphs)
    cfg.width, cfg.height = side
    cfg.tile_size = max(side)
    return sc, cfg


def small_tile(i, side=96, iterations=3000):
    rng = np.random.default_rng(200 + i)
    f, c = workloads._tile(rng, (side, side), (iterations, iterations))
    return f, c


def test_result_same_alone_and_in_mix(renderer):
    sc, cfg = small_preview(0)
    f, canvas = small_tile(0)
    alone = Server(renderer, hbm_budget=2 * GB, slots=2)
    p = alone.preview(sc, cfg)
    a1 = alone.wait(p)
    r = alone.refine(p, 3)
    a2 = alone.wait(r)
    t = alone.tile(f, canvas)
    a3 = alone.wait(t)
    assert a1.batch_requests == a2.batch_requests == a3.batch_requests == 1
    assert a1.samples == 1 and a2.samples == 4
    alone.close()

    # one slot: whatever arrives while the first batch runs is batched together
    mix = Server(renderer, hbm_budget=2 * GB, slots=1)
    tickets = []
    for i in range(1, 4):
        s2, c2 = small_preview(i)
        tickets.append(mix.preview(s2, c2))
        f2, k2 = small_tile(i)
        tickets.append(mix.tile(f2, k2))
    p2 = mix.preview(sc, cfg)
    t2 = mix.tile(f, canvas)
    tickets.append(mix.refine(tickets[0], 2))
    r2 = mix.refine(p2, 3)
    b1, b3, b2 = mix.wait(p2), mix.wait(t2), mix.wait(r2)
    for k in tickets:
        assert mix.wait(k).state == DONE
    assert max(b1.batch_requests, b2.batch_requests, b3.batch_requests) > 1  # genuinely batched
    np.testing.assert_array_equal(b1.accum, a1.accum)
    np.testing.assert_array_equal(b2.accum, a2.accum)
    np.testing.assert_array_equal(b3.iterations, a3.iterations)
    np.testing.assert_array_equal(b3.smooth, a3.smooth)
    st = mix.stats()
    assert st["completed"] == len(tickets) + 3 and st["failed"] == 0
    mix.close()


def test_matches_plain_drop_in(renderer, gpu_ctx):
    sc, cfg = small_preview(5)
    f, canvas = small_tile(5)
    srv = Server(renderer, hbm_budget=GB)
    p = srv.preview(sc, cfg)
    t = srv.tile(f, canvas)
    got_p, got_t = srv.wait(p), srv.wait(t)
    r = srv.wait(srv.refine(p, 4))
    srv.close()
    scfg = type(cfg)(**{**cfg.__dict__, "samples_per_pixel": 64, "samples_per_dispatch": 4})
    s = RenderSession(renderer, sc, scfg)
    s.dispatch((0, 0, cfg.width, cfg.height), 1)
    s.sync()
    ref1 = s.readback().accum
    s.dispatch((0, 0, cfg.width, cfg.height, 1), 4)  # samples 1..4 (tile.done = 1)
    s.sync()
    ref2 = s.readback().accum
    s.close()
    # the session runs the single-form trace kernel, the server the per-job form switch
    for got, ref in ((got_p.accum, ref1), (r.accum, ref2)):
        np.testing.assert_array_equal(got[..., 3], ref[..., 3])
        scale = max(1.0, float(np.abs(ref[..., :3]).max()))
        assert np.abs(got[..., :3] - ref[..., :3]).max() <= 1e-4 * scale
    plain = escape2d(gpu_ctx, f, canvas)
    np.testing.assert_array_equal(got_t.iterations, plain["iterations"])
    np.testing.assert_array_equal(got_t.smooth, plain["traps"][0])
    np.testing.assert_array_equal(got_t.distance, plain["distance"])
    np.testing.assert_array_equal(got_t.traps, plain["traps"])


def test_refinements_run_in_submission_order(renderer):
    sc, cfg = small_preview(7)
    srv = Server(renderer, hbm_budget=GB, slots=4)
    p = srv.preview(sc, cfg)
    rs = [srv.refine(p, k) for k in (1, 2, 3, 4)]
    res = [srv.wait(t) for t in rs]
    assert [x.samples for x in res] == [2, 4, 7, 11]
    assert all(x.start_ms >= y.done_ms for x, y in zip(res[1:], res[:-1]))
    assert res[-1].accum[..., 3].min() == 11
    srv.close()


def test_admission_waits_for_the_budget(renderer):
    sc, cfg = small_preview(9, side=(256, 256))
    film = 256 * 256 * 36 + 4096  # film planes + scene, rounded
    srv = Server(renderer, hbm_budget=film + (film // 2), slots=2)
    p1 = srv.preview(sc, cfg)
    srv.wait(p1)
    p2 = srv.preview(sc, cfg)
    with pytest.raises(SyfrackError) as e:
        srv.wait(p2, timeout_ms=300)
    assert "SF_ERR_TIMEOUT" in str(e.value)
    assert srv.poll(p2).state == QUEUED
    assert srv.stats()["admission_waits"] > 0
    srv.release(p1)  # frees the first film
    second = srv.wait(p2)
    np.testing.assert_array_equal(second.accum, srv.poll(p2).accum)
    srv.close()


def test_request_errors(renderer):
    srv = Server(renderer, hbm_budget=GB, path_capacity=1 << 16)
    with pytest.raises(SyfrackError, match="SF_ERR_INVALID"):
        srv.refine(12345, 8)
    with pytest.raises(SyfrackError, match="SF_ERR_INVALID"):
        srv.poll(999)
    sc, cfg = small_preview(3, side=(512, 512))  # 262144 paths > capacity 65536
    with pytest.raises(SyfrackError, match="SF_ERR_INVALID"):
        srv.preview(sc, cfg)
    f, c = small_tile(3)
    small = Server(renderer, hbm_budget=1 << 20)
    c.width = c.height = 1024  # 24 MiB of outputs > 1 MiB budget
    with pytest.raises(SyfrackError, match="SF_ERR_BUDGET"):
        small.tile(f, c)
    small.close()
    srv.close()


def test_destroy_with_requests_queued(renderer):
    srv = Server(renderer, hbm_budget=GB, slots=1)
    for i in range(6):
        f, c = small_tile(i, side=256, iterations=2000)
        srv.tile(f, c)
    srv.close()  # returns after the batch in flight; queued requests fail


def test_concurrent_clients(renderer):
    # several client threads submit and wait at once (the calls release the GIL); every
    # request completes with the result it has alone
    import threading

    srv = Server(renderer, hbm_budget=2 * GB, slots=3)
    tiles = [small_tile(20 + i, side=64, iterations=1500) for i in range(12)]
    alone = [escape2d(renderer.ctx, f, c)["iterations"] for f, c in tiles]
    out, errors = {}, []

    def client(k):
        try:
            mine = list(range(k, len(tiles), 4))
            tickets = [(i, srv.tile(*tiles[i])) for i in mine]
            for i, t in tickets:
                out[i] = srv.wait(t).iterations
                srv.release(t)
        except Exception as e:  # reported below, on the test's thread
            errors.append(e)

    threads = [threading.Thread(target=client, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=120)
    srv.close()
    assert not errors, errors
    assert sorted(out) == list(range(len(tiles)))
    for i in range(len(tiles)):
        np.testing.assert_array_equal(out[i], alone[i])


def test_sky_lit_preview_served(renderer):
    """A preview lit by a sun and a sky (three shadow segments per bounce, what the
    server's arenas hold) matches the same render through a session; a scene with more
    sky lights than the arenas hold is refused before it is queued."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from helpers import golden_scene
    from syfrack_gb300.scene import RenderConfig, SunLight

    sc = golden_scene("mandelbulb")
    cfg = RenderConfig(64, 40, 1, max_bounces=1, max_steps=512, pixel_tolerance=1.0, tile_size=64,
                       samples_per_dispatch=1, integrator="wavefront")
    srv = Server(renderer, hbm_budget=GB, path_capacity=1 << 16)
    t = srv.preview(sc, cfg)
    r = srv.wait(t)
    assert r.state == DONE and r.status == 0
    s = RenderSession(renderer, sc, cfg)
    while not s.step(0):
        pass
    ref = s.readback()
    s.close()
    # the server runs the batched kernel (per-job form switch), the session the per-form one
    scale = max(1.0, float(np.abs(ref.accum[..., :3]).max()))
    assert np.abs(r.accum[..., :3] - ref.accum[..., :3]).max() <= 1e-4 * scale
    assert r.accum[..., :3].mean() > 0.05
    srv.release(t)
    sc.lights = list(sc.lights) + [SunLight(direction=(0.3, 0.9, -0.2))]
    with pytest.raises(SyfrackError, match="SF_ERR_UNSUPPORTED"):
        srv.preview(sc, cfg)
    srv.close()

"""Batched wavefront over uneven jobs (GPU): every job's film equals the film of
the same job rendered alone by a wavefront session; graph replays equal direct
launches; the autotuner keeps films clean."""
import numpy as np
import pytest

from syfrack_gb300 import Batch, RenderSession, workloads

pytestmark = pytest.mark.gpu


def small_jobs(n=6):
    jobs = workloads.mixed_batch(seed=11, jobs=n)
    out = []
    for sc, cfg in jobs:
        side = max(16, cfg.width // 6)
        cfg.width = cfg.height = side
        cfg.tile_size = side
        cfg.samples_per_pixel = cfg.samples_per_dispatch = max(1, cfg.samples_per_pixel // 4)
        out.append((sc, cfg))
    return out


def alone(renderer, sc, cfg):
    s = RenderSession(renderer, sc, cfg)
    while not s.step(0):
        pass
    r = s.readback()
    s.close()
    return r


def test_batch_equals_jobs_alone(renderer):
    jobs = small_jobs()
    b = Batch(renderer, jobs)
    b.run(1, use_graph=False)
    assert b.sync() == 0
    forms = {renderer.compile(sc.graph).info()["form"] for sc, _ in jobs}
    assert len(forms) >= 2  # genuinely mixed
    for i, (sc, cfg) in enumerate(jobs):
        got = b.readback(i)
        ref = alone(renderer, sc, cfg)
        assert got.accum[..., 3].min() == cfg.samples_per_pixel
        scale = max(1.0, float(np.abs(ref.accum[..., :3]).max()))
        assert np.abs(got.accum[..., :3] - ref.accum[..., :3]).max() <= 1e-4 * scale, i
        np.testing.assert_allclose(got.depth, ref.depth, rtol=1e-6, atol=1e-6)
    b.close()


def test_graph_replay_equals_direct_launches(renderer):
    jobs = small_jobs(4)
    a = Batch(renderer, jobs)
    a.run(2, use_graph=False)
    a.sync()
    g = Batch(renderer, jobs)
    g.run(2, use_graph=True)
    g.sync()
    for i in range(len(jobs)):
        ra, rg = a.readback(i), g.readback(i)
        np.testing.assert_array_equal(ra.accum, rg.accum)
        assert ra.accum[..., 3].min() == 2 * jobs[i][1].samples_per_dispatch
    a.close()
    g.close()


def test_autotune_leaves_films_clean(renderer):
    jobs = small_jobs(3)
    b = Batch(renderer, jobs)
    mb, q, rg, ms = b.autotune()
    assert mb in (2, 3, 4) and q in (0, 64, 128, 256) and rg in (1, 4, 8, 16) and ms > 0
    b.run(1)
    b.sync()
    for i, (sc, cfg) in enumerate(jobs):
        assert b.readback(i).accum[..., 3].max() == cfg.samples_per_dispatch
    b.close()


def test_sky_lit_jobs_in_a_batch(renderer):
    """Jobs with a sun and a sky (three shadow slots in the batch's arena) next to
    area-lit jobs (one): each film equals the job alone."""
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from helpers import golden_scene
    from syfrack_gb300.scene import RenderConfig

    jobs = small_jobs(3)
    for name in ("menger", "mandelbulb"):
        jobs.append((golden_scene(name), RenderConfig(48, 32, 4, max_bounces=3, max_steps=256, pixel_tolerance=1.0,
                                                      tile_size=48, samples_per_dispatch=4, integrator="wavefront")))
    b = Batch(renderer, jobs)
    b.run(1, use_graph=False)
    assert b.sync() == 0
    for i, (sc, cfg) in enumerate(jobs):
        got = b.readback(i)
        ref = alone(renderer, sc, cfg)
        scale = max(1.0, float(np.abs(ref.accum[..., :3]).max()))
        assert np.abs(got.accum[..., :3] - ref.accum[..., :3]).max() <= 1e-4 * scale, i
        np.testing.assert_allclose(got.depth, ref.depth, rtol=1e-6, atol=1e-6)
    assert b.readback(len(jobs) - 1).accum[..., :3].mean() > 0.05  # the sky lights reach the form
    b.close()


def test_batched_jobs_against_oracle(renderer, oracle_mod):
    """Three jobs of the uneven batch (a Mandelbulb of an odd power, a Mandelbox of a
    scale below 1.05 in magnitude, a Menger sponge), batched, against the f32 oracle
    on seeded pixels: film RMSE within 2e-2 and first-hit depth within 1e-3 where both
    hit."""
    from syfrack_gb300.scene import AreaLight, Scene

    picks = [("mandelbulb", 5), ("mandelbox", -0.8), ("menger", 4)]
    base = workloads.mixed_batch(seed=7, jobs=3)
    jobs = []
    for (kind, value), (sc, cfg) in zip(picks, base):
        g = workloads.mixed_batch_graph(kind, value)
        scale = g.bounding_radius_hint / 2.0 if kind == "mandelbox" else 1.0
        d = np.asarray(sc.camera.position, np.float64)
        pos = d / np.linalg.norm(d) * 3.0 * scale
        cam = type(sc.camera).look_at(tuple(pos.tolist()), (0.0, 0.0, 0.0), 50.0)
        light = AreaLight(position=tuple((pos * 0.5 + np.array([0.0, 1.8 * scale, 0.0])).tolist()),
                          normal=(0.0, -1.0, 0.0), size=(1.0, 1.0), intensity=10.0)
        scene = Scene(graph=g, camera=cam, material=sc.material, lights=[light], seed=sc.seed)
        cfg.width = cfg.height = cfg.tile_size = 96
        cfg.samples_per_pixel = cfg.samples_per_dispatch = 8
        jobs.append((scene, cfg))
    b = Batch(renderer, jobs)
    b.run(1, use_graph=True)
    assert b.sync() == 0
    rng = np.random.default_rng(17)
    for i, (sc, cfg) in enumerate(jobs):
        got = b.readback(i)
        pix = np.stack([rng.integers(0, 96, 256), rng.integers(0, 96, 256)], 1).astype(np.uint32)
        ref = oracle_mod.OracleGraph(sc.graph).render(sc.desc(96, 96), cfg.desc(), pix, 0, 8, precision=32)
        mine = got.accum[pix[:, 1], pix[:, 0], :3] / 8
        rmse = float(np.sqrt(np.mean((mine - ref["accum"] / 8) ** 2)))
        assert rmse <= 2e-2, (picks[i], rmse)
        dd, rd = got.depth[pix[:, 1], pix[:, 0]], ref["depth"]
        assert (dd >= 0).mean() > 0.05, picks[i]  # the form is in view
        assert ((dd >= 0) == (rd >= 0)).mean() >= 0.97, picks[i]
        both = (dd >= 0) & (rd >= 0)
        assert np.median(np.abs(dd[both] - rd[both]) / np.maximum(rd[both], 1.0)) <= 1e-3, picks[i]
    b.close()

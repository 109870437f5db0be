"""Height fog: the oracle against the reference's Beer-Lambert and energy tests, the
device against the oracle and between its two integrators.

The CPU tests restate the reference's own fog tests with their scenes, sample counts
and tolerances: crates/syfrack-render/tests/gpu_lighting.rs:286-297 (a mirror reflection
of a softbox in absorbing fog is attenuated on both legs), :300-337 (thin-fog phase
sampling of an area light does not count its emission twice, and splitting the light
keeps the energy), :340-383 (two coloured lights in symmetric fog) and
gpu_environment.rs:296-311 (a white sky seen through thin anisotropic fog keeps its
radiance at any bounce count; here the constant sky is the gradient light with three
equal colours instead of a constant panorama)."""
import math

import numpy as np
import pytest

from syfrack_gb300 import SyfrackError
from syfrack_gb300.graph import Graph, Kind, Link, Node
from syfrack_gb300.scene import (AreaLight, Camera, EnvironmentLight, Fog, Material, RenderConfig, Scene,
                                 SunLight)

CENTRE = np.array([(x, y) for y in range(12, 20) for x in range(12, 20)], dtype=np.uint32)


def minimal(kind):
    """Graph::new_minimal (graph/mod.rs:454-482) with node 1 replaced."""
    return Graph([Node(0, Kind("Input")), Node(1, kind), Node(2, Kind("Output"))],
                 [Link((0, 0), (1, 0)), Link((1, 0), (2, 0))], safety=1.0, bounding_radius_hint=2.0)


def base_scene(kind, position=(0.0, 0.0, 3.0), target=(0.0, 0.0, 0.0)):
    """gpu_lighting.rs:14-36: a 500 mm pinhole at (0, 0, 3), grey Lambert, no lights."""
    return Scene(graph=minimal(kind), camera=Camera(position, target, 0.0, 500.0, 0.0, 3.0),
                 material=Material(albedo=(0.5, 0.5, 0.5), roughness=0.5, metallic=0.0, specular=0.0))


def mirror_scene():
    """gpu_lighting.rs:188-199: a rough-0.02 metal plane under a 4x4 softbox 5 units up."""
    s = base_scene(Kind("Plane", normal=[0.0, 0.0, 1.0], offset=0.0))
    s.material = Material(albedo=(0.8, 0.8, 0.8), roughness=0.02, metallic=1.0, specular=0.0)
    s.lights = [AreaLight(position=(0.0, 0.0, 5.0), normal=(0.0, 0.0, -1.0), size=(4.0, 4.0), intensity=3.0)]
    return s


def centre(oracle_mod, scene, spp, bounces, channel=0):
    cfg = RenderConfig(32, 32, spp, max_bounces=bounces)
    out = oracle_mod.OracleGraph(scene.graph).render(scene.desc(32, 32), cfg.desc(), CENTRE, 0, spp, precision=32)
    return float(np.mean(out["accum"][:, channel])) / spp


def test_absorbing_fog_attenuates_both_legs(oracle_mod):
    """gpu_lighting.rs:286-297: camera -> mirror 3 units, mirror -> softbox 5 units."""
    s = mirror_scene()
    clear = centre(oracle_mod, s, 128, 1)
    assert abs(clear - 2.4) < 0.10, clear
    s.fog = Fog(density=0.15, color=(0.0, 0.0, 0.0), falloff=0.0)
    expected = 2.4 * math.exp(-0.15 * 8.0)
    measured = centre(oracle_mod, s, 512, 1)
    assert abs(measured - expected) < expected * 0.07, (measured, expected)


def test_thin_fog_phase_emission_is_not_counted_twice(oracle_mod):
    """gpu_lighting.rs:300-337: NEE-only (0 bounces) against NEE + phase continuation
    (1 bounce) of a broad lateral softbox, then the softbox split in four."""
    s = base_scene(Kind("Plane", normal=[1.0, 0.0, 0.0], offset=100.0), position=(0.0, 0.0, 0.0),
                   target=(0.0, 0.0, 1.0))
    s.lights = [AreaLight(position=(3.0, 0.0, 3.0), normal=(-1.0, 0.0, 0.0), size=(20.0, 20.0), intensity=5.0)]
    s.fog = Fog(density=0.001, falloff=0.0)
    terminal = centre(oracle_mod, s, 2048, 0)
    mis = centre(oracle_mod, s, 2048, 1)
    assert terminal > 0.01, terminal
    assert 0.90 < mis / terminal < 1.15, (terminal, mis)
    s.lights = [AreaLight(position=(3.0, 0.0, 3.0), normal=(-1.0, 0.0, 0.0), size=(20.0, 20.0), intensity=1.25)
                for _ in range(4)]
    split = centre(oracle_mod, s, 2048, 1)
    assert 0.85 < split / mis < 1.15, (mis, split)


def test_coloured_lights_mix_in_symmetric_fog(oracle_mod):
    """gpu_lighting.rs:340-383: a red and a blue softbox facing each other across the
    view light the fog equally; nothing without fog; nothing green."""
    s = base_scene(Kind("Plane", normal=[1.0, 0.0, 0.0], offset=100.0), position=(0.0, 0.0, 0.0),
                   target=(0.0, 0.0, 1.0))
    s.lights = [AreaLight(position=(x, 0.0, 3.0), normal=(-math.copysign(1.0, x), 0.0, 0.0), size=(10.0, 10.0),
                          color=c, intensity=4.0) for x, c in [(3.0, (1.0, 0.0, 0.0)), (-3.0, (0.0, 0.0, 1.0))]]
    cfg = RenderConfig(32, 32, 4, max_bounces=0)
    og = oracle_mod.OracleGraph(s.graph)
    allpx = np.array([(x, y) for y in range(32) for x in range(32)], dtype=np.uint32)
    clear = og.render(s.desc(32, 32), cfg.desc(), allpx, 0, 4, precision=32)["accum"]
    assert np.all(clear == 0.0)
    s.fog = Fog(density=0.035, color=(0.9, 0.9, 0.9), falloff=0.0, anisotropy=0.15)
    cfg = RenderConfig(32, 32, 128, max_bounces=0)
    mixed = og.render(s.desc(32, 32), cfg.desc(), allpx, 0, 128, precision=32)["accum"]
    assert np.all(np.isfinite(mixed))
    red, blue = mixed[:, 0].sum(), mixed[:, 2].sum()
    assert 0.9 < red / blue < 1.1, (red, blue)
    assert np.all(mixed[:, 0] > 0.001 * 128) and np.all(mixed[:, 2] > 0.001 * 128) and np.all(mixed[:, 1] == 0.0)


def test_white_sky_through_thin_fog_keeps_its_radiance(oracle_mod):
    """gpu_environment.rs:296-311 with the gradient sky at 1 everywhere: phase sampling
    and the sky's next events share the energy by MIS at every bounce count.

    The fog acts over the 200-unit ray extent (T_MAX, common.wgsl:206-208), so a view
    ray passes with T = exp(-0.2); a scattered one sees the sky through T again (the
    next event's transmittance, or the continuation's free flight). With white fog the
    expectation after n bounces is 1 - (1 - T)^(n + 2): 0.967 at 0 bounces, 0.994 at 1,
    1.000 at 4 -- the reference's bound of 0.025 around 1 is the limit; the test holds
    each count to its closed form with that tolerance."""
    s = base_scene(Kind("Sphere", radius=0.01), position=(0.0, 0.0, 3.0), target=(0.0, 0.0, 4.0))
    s.lights = [EnvironmentLight(zenith=(1.0, 1.0, 1.0), horizon=(1.0, 1.0, 1.0), ground=(1.0, 1.0, 1.0))]
    s.fog = Fog(density=0.001, falloff=0.0, anisotropy=0.3)
    miss = 1.0 - math.exp(-0.001 * 200.0)
    for bounces in (0, 1, 4):
        measured = centre(oracle_mod, s, 1024, bounces)
        expected = 1.0 - miss ** (bounces + 2)
        assert abs(measured - expected) < 0.025 * 0.4, (bounces, measured, expected)


def test_fog_is_read_from_scene_files():
    """Atmosphere's fog fields (atmosphere.rs:7-28) reach the descriptor; a file without
    fog (scenes/mandelbulb.ron) leaves it off."""
    from helpers import golden_scene

    assert golden_scene("mandelbulb").desc(64, 32).fog.density == 0.0
    s = golden_scene("mandelbulb", atmosphere={"fog_density": 0.018, "fog_color": [0.8, 0.85, 0.9],
                                               "fog_height": 1.5, "fog_falloff": 0.4, "anisotropy": 0.2})
    d = s.desc(64, 32)
    assert (d.fog.density, d.fog.height, d.fog.falloff) == pytest.approx((0.018, 1.5, 0.4))
    assert d.fog.anisotropy == pytest.approx(0.2)
    assert list(d.fog.color) == pytest.approx([0.8, 0.85, 0.9])


# ---------------------------------------------------------------------------- device
def fog_bulb_scene():
    """The bounded Mandelbulb view in fog above the form's middle, lit by a softbox, a
    sun and the gradient sky: every kind of fog next event and the shadow slots."""
    from syfrack_gb300 import workloads

    _, cam, *_ = workloads.mandelbulb_primary()
    return Scene(graph=workloads.mandelbulb_primary_graph(), camera=cam,
                 material=Material(albedo=(0.8, 0.7, 0.6), roughness=0.35),
                 lights=[AreaLight(position=(0.0, 2.5, 1.0), normal=(0.0, -1.0, -0.3), size=(1.5, 1.5),
                                   intensity=8.0),
                         SunLight(direction=(0.3, 0.9, -0.2), intensity=2.0),
                         EnvironmentLight()],
                 fog=Fog(density=0.08, color=(0.85, 0.9, 0.95), height=0.2, falloff=0.7, anisotropy=0.25),
                 seed=5)


@pytest.mark.gpu
def test_fog_wavefront_equals_megakernel_and_follows_the_oracle(renderer, oracle_mod):
    from syfrack_gb300 import RenderSession

    scene = fog_bulb_scene()
    films = []
    for integ in ("wavefront", "megakernel"):
        cfg = RenderConfig(96, 64, 8, max_bounces=3, max_steps=256, pixel_tolerance=1.0, tile_size=64,
                           samples_per_dispatch=4, integrator=integ)
        s = RenderSession(renderer, scene, cfg)
        while not s.step(0):
            pass
        films.append(s.readback())
        s.close()
    # one bounce body in both kernels; the segment's line-integral terms land before the
    # bounce's emission in the megakernel and after it in the wavefront: equal to a few
    # roundings of the sum
    np.testing.assert_allclose(films[0].accum, films[1].accum, rtol=1e-5, atol=1e-6)
    np.testing.assert_array_equal(films[0].depth, films[1].depth)
    rng = np.random.default_rng(11)
    pix = np.stack([rng.integers(0, 96, 128), rng.integers(0, 64, 128)], 1).astype(np.uint32)
    ref = oracle_mod.OracleGraph(scene.graph).render(scene.desc(96, 64), cfg.desc(), pix, 0, 8, precision=32)
    mine = films[0].accum[pix[:, 1], pix[:, 0], :3] / 8
    rmse = float(np.sqrt(np.mean((mine - ref["accum"] / 8) ** 2)))
    assert rmse <= 2e-2, rmse
    assert mine.mean() > 0.02


@pytest.mark.gpu
def test_device_absorbing_fog_attenuates_both_legs(renderer):
    from syfrack_gb300 import RenderSession

    s = mirror_scene()
    s.fog = Fog(density=0.15, color=(0.0, 0.0, 0.0), falloff=0.0)
    cfg = RenderConfig(32, 32, 512, max_bounces=1, integrator="wavefront", samples_per_dispatch=64)
    sess = RenderSession(renderer, s, cfg)
    while not sess.step(0):
        pass
    film = sess.readback()
    sess.close()
    measured = float(film.accum[12:20, 12:20, 0].mean()) / 512
    expected = 2.4 * math.exp(-0.15 * 8.0)
    assert abs(measured - expected) < expected * 0.07, (measured, expected)


@pytest.mark.gpu
def test_fog_scenes_past_eight_shadow_segments_are_refused(renderer):
    from syfrack_gb300 import RenderSession

    s = mirror_scene()
    s.lights = [AreaLight(position=(float(i), 0.0, 5.0), normal=(0.0, 0.0, -1.0)) for i in range(8)]
    cfg = RenderConfig(32, 32, 1, max_bounces=1, integrator="wavefront")
    RenderSession(renderer, s, cfg).close()  # no fog: one area slot
    s.fog = Fog(density=0.1)
    with pytest.raises(SyfrackError, match="SF_ERR_UNSUPPORTED"):
        RenderSession(renderer, s, cfg)


@pytest.mark.gpu
def test_fog_jobs_in_a_batch_equal_their_sessions(renderer):
    """A fog job (four shadow slots: area, sun, sky and the segment's area estimate)
    batched with an area-lit job: each film equals the job rendered alone."""
    from syfrack_gb300 import Batch, RenderSession

    cfg = RenderConfig(48, 32, 4, max_bounces=3, max_steps=256, pixel_tolerance=1.0, tile_size=48,
                       samples_per_dispatch=4, integrator="wavefront")
    fog = fog_bulb_scene()
    clear = fog_bulb_scene()
    clear.fog = None
    clear.lights = clear.lights[:1]
    jobs = [(clear, cfg), (fog, cfg)]
    b = Batch(renderer, jobs)
    b.run(1, use_graph=False)
    assert b.sync() == 0
    for i, (sc, c) in enumerate(jobs):
        got = b.readback(i)
        s = RenderSession(renderer, sc, c)
        while not s.step(0):
            pass
        ref = s.readback()
        s.close()
        scale = max(1.0, float(np.abs(ref.accum[..., :3]).max()))
        assert np.abs(got.accum[..., :3] - ref.accum[..., :3]).max() <= 1e-4 * scale, i
    b.close()


def test_oracle_volume_planes(oracle_mod):
    """The oracle's film planes (pathtrace.wgsl:1243-1266): volume + surface = radiance,
    moments >= 0, counts = samples; a clear scene has no volume part."""
    scene = fog_bulb_scene()
    cfg = RenderConfig(96, 64, 8, max_bounces=3, max_steps=256)
    pix = np.stack([np.arange(0, 96, 3), np.full(32, 30)], 1).astype(np.uint32)
    r = oracle_mod.OracleGraph(scene.graph).render(scene.desc(96, 64), cfg.desc(), pix, 0, 8, precision=32,
                                                    planes=True)
    np.testing.assert_allclose(r["volume"][:, :3] + r["surface"][:, :3], r["accum"], rtol=1e-5, atol=1e-6)
    assert (r["volume"][:, 3] == 8).all() and (r["moments"][:, 3] == 8).all() and (r["surface"][:, 3] == 8).all()
    assert (r["moments"][:, :3] >= 0).all() and r["volume"][:, :3].sum() > 0
    clear = fog_bulb_scene()
    clear.fog = None
    c = oracle_mod.OracleGraph(clear.graph).render(clear.desc(96, 64), cfg.desc(), pix, 0, 8, precision=32,
                                                    planes=True)
    assert (c["volume"][:, :3] == 0).all() and (c["moments"][:, :3] == 0).all()
    np.testing.assert_array_equal(c["surface"][:, :3], c["accum"])


def _session_planes(renderer, scene, cfg):
    from syfrack_gb300 import RenderSession

    s = RenderSession(renderer, scene, cfg)
    while not s.step(0):
        pass
    planes = s.film_planes()
    s.close()
    return planes


@pytest.mark.gpu
def test_fog_volume_planes_against_the_oracle(renderer, oracle_mod):
    """The film's volume layer split on the device: both integrators keep it, it adds
    up to the radiance, and it follows the f32 oracle's planes."""
    scene = fog_bulb_scene()
    out = {}
    for integ in ("wavefront", "megakernel"):
        cfg = RenderConfig(96, 64, 8, max_bounces=3, max_steps=256, pixel_tolerance=1.0, tile_size=64,
                           samples_per_dispatch=4, integrator=integ)
        out[integ] = _session_planes(renderer, scene, cfg)
    wf, mk = out["wavefront"], out["megakernel"]
    for k in ("volume", "moments", "surface"):
        assert (wf[k][..., 3] == 8).all(), k
        np.testing.assert_allclose(wf[k], mk[k], rtol=1e-4, atol=1e-5, err_msg=k)
    np.testing.assert_allclose(wf["volume"][..., :3] + wf["surface"][..., :3], wf["accum"][..., :3], rtol=1e-5,
                               atol=1e-5)
    assert (wf["moments"][..., :3] >= 0).all()
    assert wf["volume"][..., :3].mean() > 1e-3  # the fog's light reaches the camera
    rng = np.random.default_rng(23)
    pix = np.stack([rng.integers(0, 96, 128), rng.integers(0, 64, 128)], 1).astype(np.uint32)
    ref = oracle_mod.OracleGraph(scene.graph).render(scene.desc(96, 64), cfg.desc(), pix, 0, 8, precision=32,
                                                      planes=True)
    for k in ("volume", "surface"):
        mine = wf[k][pix[:, 1], pix[:, 0], :3] / 8
        rmse = float(np.sqrt(np.mean((mine - ref[k][:, :3] / 8) ** 2)))
        assert rmse <= 2e-2, (k, rmse)


@pytest.mark.gpu
def test_clear_scene_has_no_volume_part(renderer):
    from syfrack_gb300 import workloads

    cfg = workloads.mandelbox_pathtrace_config(width=64, height=36, spp=4, samples_per_dispatch=4)
    p = _session_planes(renderer, workloads.mandelbox_scene(), cfg)
    assert (p["volume"][..., :3] == 0).all() and (p["volume"][..., 3] == 4).all()
    np.testing.assert_array_equal(p["surface"], p["accum"])


@pytest.mark.gpu
def test_fog_volume_planes_survive_a_checkpoint(renderer, tmp_path):
    """A fog session saved after its first dispatch and resumed ends with the planes of
    the uninterrupted render, bit for bit."""
    from syfrack_gb300 import RenderSession

    scene = fog_bulb_scene()
    cfg = RenderConfig(64, 48, 8, max_bounces=3, max_steps=256, pixel_tolerance=1.0, tile_size=64,
                       samples_per_dispatch=4, integrator="wavefront")
    whole = _session_planes(renderer, scene, cfg)
    s = RenderSession(renderer, scene, cfg)
    s.step(0)
    s.save(str(tmp_path / "ck"))
    s.close()
    r = RenderSession.resume(renderer, scene, cfg, str(tmp_path / "ck"))
    while not r.step(0):
        pass
    got = r.film_planes()
    r.close()
    for k in ("accum", "volume", "moments", "surface"):
        np.testing.assert_array_equal(got[k], whole[k], err_msg=k)


@pytest.mark.gpu
def test_fog_job_volume_planes_in_a_batch(renderer):
    """A batched fog job keeps the volume layer split of its session."""
    from syfrack_gb300 import Batch

    cfg = RenderConfig(48, 32, 4, max_bounces=3, max_steps=256, pixel_tolerance=1.0, tile_size=48,
                       samples_per_dispatch=4, integrator="wavefront")
    fog = fog_bulb_scene()
    clear = fog_bulb_scene()
    clear.fog = None
    clear.lights = clear.lights[:1]
    b = Batch(renderer, [(clear, cfg), (fog, cfg)])
    b.run(1, use_graph=False)
    assert b.sync() == 0
    got = b.film_planes(1)
    b.close()
    ref = _session_planes(renderer, fog, cfg)
    for k in ("volume", "moments", "surface"):
        np.testing.assert_allclose(got[k], ref[k], rtol=1e-4, atol=1e-4 * max(1.0, float(np.abs(ref[k]).max())),
                                   err_msg=k)

"""Scenes of more than the descriptor's eight inline lights on the device (Scene::lights
up to MAX_LIGHTS = 96, light.rs:7; GpuLight array uniforms.rs:621, 783-827): lights
past the eighth are read from the scene's device light table. Dark emitters put in
front of a scene's lights leave the device film bit for bit unchanged on both
integrators; the reference's 14-light scenes/showcase/la-cathedrale-des-marees-neons.ron
(projectors, tubes, area lights and four sky lights; without its fog, 5 shadow segments
per bounce) renders through both integrators and follows the oracle; the 82-light fog scene
scenes/studies/cathedrale-des-marees-20261020/etude-neons.ron (86 shadow segments per
bounce) renders through the megakernel, which traces them as it issues them, while the
wavefront, which stores at most 8 per bounce, refuses it, as batches and previews
refuse more than 8 lights."""
import numpy as np
import pytest

from helpers import golden_scene
from syfrack_gb300 import RenderSession, SyfrackError
from syfrack_gb300.scene import RenderConfig

from test_lights import compact_scene, padded_scene

pytestmark = pytest.mark.gpu
BOTH = ["megakernel", "wavefront"]


def render(renderer, scene, cfg):
    s = RenderSession(renderer, scene, cfg)
    while not s.step(0):
        pass
    out = s.readback()
    assert s.sync() == 0
    s.close()
    return out


@pytest.mark.parametrize("integrator", BOTH)
def test_dark_lights_in_front_leave_the_device_film_unchanged(renderer, integrator):
    cfg = RenderConfig(width=96, height=54, samples_per_pixel=8, max_bounces=3, max_steps=512, tile_size=64,
                       samples_per_dispatch=8, integrator=integrator)
    a = render(renderer, compact_scene(), cfg)
    b = render(renderer, padded_scene(), cfg)
    np.testing.assert_array_equal(a.accum, b.accum)
    np.testing.assert_array_equal(a.depth, b.depth)
    assert float(a.accum[..., :3].mean()) > 0.01


def test_many_lights_film_against_the_oracle(renderer, oracle_mod):
    """The padded scene's device film against the f32 oracle on seeded pixels (RMSE <=
    2e-2, as the other film tests)."""
    scene = padded_scene()
    cfg = RenderConfig(width=96, height=54, samples_per_pixel=16, max_bounces=3, max_steps=512, tile_size=64,
                       samples_per_dispatch=8, integrator="wavefront")
    a = render(renderer, scene, cfg)
    rng = np.random.default_rng(17)
    pix = np.stack([rng.integers(0, cfg.width, 96), rng.integers(0, cfg.height, 96)], 1).astype(np.uint32)
    ref = oracle_mod.OracleGraph(scene.graph).render(scene.desc(cfg.width, cfg.height), cfg.desc(), pix, 0,
                                                     cfg.samples_per_pixel, precision=32)
    mine = a.accum[pix[:, 1], pix[:, 0], :3] / cfg.samples_per_pixel
    rmse = float(np.sqrt(np.mean((mine - ref["accum"][:, :3] / cfg.samples_per_pixel) ** 2)))
    assert rmse <= 2e-2, rmse


def film_against_oracle(renderer, oracle_mod, scene, cfg, seed):
    out = render(renderer, scene, cfg)
    rng = np.random.default_rng(seed)
    pix = np.stack([rng.integers(0, cfg.width, 96), rng.integers(0, cfg.height, 96)], 1).astype(np.uint32)
    ref = oracle_mod.OracleGraph(scene.graph).render(scene.desc(cfg.width, cfg.height), cfg.desc(), pix, 0,
                                                     cfg.samples_per_pixel, precision=32)
    mine = out.accum[pix[:, 1], pix[:, 0], :3].astype(np.float64) / cfg.samples_per_pixel
    theirs = ref["accum"][:, :3] / cfg.samples_per_pixel
    scale = max(float(np.abs(theirs).mean()), 1e-3)
    rel_rmse = float(np.sqrt(np.mean((mine - theirs) ** 2))) / scale
    print(scene.lights.__len__(), "lights: image mean", scale, "relative RMSE", rel_rmse)
    assert np.all(np.isfinite(mine))
    assert abs(mine.mean() / theirs.mean() - 1.0) < 0.05, (mine.mean(), theirs.mean())
    assert rel_rmse <= 0.1, rel_rmse
    return out


def test_fourteen_light_reference_scene_through_both_integrators(renderer, oracle_mod):
    scene = golden_scene("la-cathedrale-des-marees-neons")
    assert len(scene.lights) == 14 and scene.fog is not None
    scene.fog = None
    cfg = RenderConfig(width=64, height=36, samples_per_pixel=8, max_bounces=4, max_steps=256, tile_size=64,
                       samples_per_dispatch=8, integrator="wavefront")
    a = film_against_oracle(renderer, oracle_mod, scene, cfg, 23)
    cfg.integrator = "megakernel"
    b = render(renderer, scene, cfg)
    np.testing.assert_array_equal(a.accum, b.accum)
    np.testing.assert_array_equal(a.depth, b.depth)


def test_eighty_two_light_fog_scene_on_the_megakernel(renderer, oracle_mod):
    scene = golden_scene("etude-neons")
    assert len(scene.lights) == 82 and scene.fog is not None
    cfg = RenderConfig(width=64, height=36, samples_per_pixel=8, max_bounces=3, max_steps=256, tile_size=64,
                       samples_per_dispatch=8, integrator="megakernel")
    film_against_oracle(renderer, oracle_mod, scene, cfg, 29)
    cfg.integrator = "wavefront"
    with pytest.raises(SyfrackError, match="shadow segments"):
        RenderSession(renderer, scene, cfg)


def test_batches_and_previews_take_eight_lights(renderer):
    from syfrack_gb300.render import Batch, PreviewSession

    scene = golden_scene("la-cathedrale-des-marees-neons")
    scene.fog = None
    cfg = RenderConfig(width=32, height=18, samples_per_pixel=1, max_bounces=1, max_steps=64)
    with pytest.raises(SyfrackError, match="more than 8 lights"):
        PreviewSession(renderer, scene, (32, 18))
    with pytest.raises(SyfrackError, match="more than 8 lights"):
        Batch(renderer, [(scene, cfg)])

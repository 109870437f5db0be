"""Reference scene files through the device: scenes/puits-des-eons.ron (a volumetric
texture with its own graph, surface variation, trap colouring) and
scenes/eclosion-brume.ron (two projectors, two tubes, two area lights and a sky in
height fog, eight finishes, four with detail patterns, a 139-op graph whose union of
bounded branches takes the exact union search). Both integrators render them (bit
for bit without fog; in fog the segment's line-integral terms are summed in another
order, as in test_fog), and the film follows the f32 oracle's."""
import numpy as np
import pytest

from helpers import golden_scene
from syfrack_gb300 import RenderSession
from syfrack_gb300.scene import RenderConfig

pytestmark = pytest.mark.gpu


def render(renderer, scene, cfg):
    s = RenderSession(renderer, scene, cfg)
    while not s.step(0):
        pass
    out = s.readback()
    assert s.sync() == 0
    s.close()
    return out


@pytest.mark.parametrize("name", ["puits-des-eons", "eclosion-brume"])
def test_reference_scene_renders_through_both_integrators_and_follows_the_oracle(renderer, oracle_mod, name):
    scene = golden_scene(name)
    cfg = RenderConfig(width=64, height=36, samples_per_pixel=8, max_bounces=4, max_steps=256, tile_size=64,
                       samples_per_dispatch=8, integrator="wavefront")
    a = render(renderer, scene, cfg)
    cfg.integrator = "megakernel"
    b = render(renderer, scene, cfg)
    if scene.fog is not None:
        np.testing.assert_allclose(a.accum, b.accum, rtol=1e-5, atol=1e-6)
    else:
        np.testing.assert_array_equal(a.accum, b.accum)
    np.testing.assert_array_equal(a.depth, b.depth)
    assert (a.depth >= 0).mean() > 0.2
    og = oracle_mod.OracleGraph(scene.graph)
    tg = oracle_mod.OracleGraph(scene.material.texture.graph) if scene.material.texture else None
    rng = np.random.default_rng(5)
    pix = np.stack([rng.integers(0, cfg.width, 96), rng.integers(0, cfg.height, 96)], 1).astype(np.uint32)
    ref = og.render(scene.desc(cfg.width, cfg.height, texture_graph=tg.h if tg else None), cfg.desc(), pix, 0,
                    cfg.samples_per_pixel, precision=32)
    mine = a.accum[pix[:, 1], pix[:, 0], :3].astype(np.float64) / cfg.samples_per_pixel
    theirs = ref["accum"][:, :3] / cfg.samples_per_pixel
    scale = max(float(np.abs(theirs).mean()), 1e-3)
    rel_rmse = float(np.sqrt(np.mean((mine - theirs) ** 2))) / scale
    print(name, "image mean", scale, "relative RMSE", rel_rmse)
    assert np.all(np.isfinite(mine))
    assert abs(mine.mean() / theirs.mean() - 1.0) < 0.05, (mine.mean(), theirs.mean())
    assert rel_rmse <= 0.1, rel_rmse

"""Projector and tube lights on the device, with the reference's known answers
(gpu_photometric.rs:48-132, gpu_volume_sampling.rs:122-218) on both integrators, a
fractal lit by both kinds in fog against the oracle, and the parameter bounds of
Light::visit_params (light.rs:162-226)."""
import numpy as np
import pytest

from syfrack_gb300 import RenderSession, SyfrackError, workloads
from syfrack_gb300.graph import Kind
from syfrack_gb300.scene import Camera, Fog, Material, ProjectorLight, RenderConfig, Scene, TubeLight

from test_lights import PROJECTOR_QUADRATURE, photometric_scene, projector_scene

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


def mean(renderer, scene, spp, bounces, integrator):
    """gpu_photometric.rs:36-47: the image mean of a 24 x 24 render."""
    out = render(renderer, scene, RenderConfig(width=24, height=24, samples_per_pixel=spp, max_bounces=bounces,
                                               integrator=integrator))
    c = out.color[..., :3].astype(np.float64)
    assert np.all(np.isfinite(c))
    return c.reshape(-1, 3).mean(0)


def tube(x, color):
    """gpu_photometric.rs:25-34"""
    return TubeLight(start=(x, -1.5, 2.0), end=(x, 1.5, 2.0), radius=0.16, color=color, intensity=15.0)


@pytest.mark.parametrize("integrator", BOTH)
def test_tubes_are_visible_and_red_blue_sources_add_on_concrete(renderer, integrator):
    # gpu_photometric.rs:48-86
    s = photometric_scene(Kind("Plane", normal=[0.0, 0.0, 1.0], offset=0.0), [tube(-2.0, (1.0, 0.0, 0.0))])
    a = mean(renderer, s, 512, 0, integrator)
    s.lights = [tube(2.0, (0.0, 0.0, 1.0))]
    b = mean(renderer, s, 512, 0, integrator)
    s.lights = [tube(-2.0, (1.0, 0.0, 0.0)), tube(2.0, (0.0, 0.0, 1.0))]
    both = mean(renderer, s, 1024, 0, integrator)
    assert a[0] > 0.01 and b[2] > 0.01, (a, b)
    for c in (0, 2):
        assert abs(both[c] - (a[c] + b[c])) < 0.10 * (a[c] + b[c]), (both, a, b)
    s = photometric_scene(Kind("Sphere", radius=0.01),
                          [TubeLight(start=(-2.0, 0.0, 1.0), end=(2.0, 0.0, 1.0), radius=0.7,
                                     color=(1.0, 0.1, 0.025), intensity=4.0)])
    np.testing.assert_allclose(mean(renderer, s, 4, 0, integrator), [4.0, 0.4, 0.1], atol=1e-4)


@pytest.mark.parametrize("integrator", BOTH)
def test_red_and_blue_tubes_add_in_scattering_air(renderer, integrator):
    # gpu_photometric.rs:95-132
    s = photometric_scene(Kind("Plane", normal=[1.0, 0.0, 0.0], offset=100.0), [])
    s.camera = Camera((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 0.0, 500.0, 0.0, 3.0)
    s.fog = Fog(density=0.01, color=(0.8, 0.8, 0.8), height=0.0, falloff=0.0, anisotropy=0.25)
    s.lights = [tube(-1.2, (1.0, 0.0, 0.0))]
    a = mean(renderer, s, 1024, 0, integrator)
    s.lights = [tube(1.2, (0.0, 0.0, 1.0))]
    b = mean(renderer, s, 1024, 0, integrator)
    s.lights = [tube(-1.2, (1.0, 0.0, 0.0)), tube(1.2, (0.0, 0.0, 1.0))]
    mixed = mean(renderer, s, 2048, 0, integrator)
    for c in (0, 2):
        assert a[c] + b[c] > 0.001
        assert abs(mixed[c] - (a[c] + b[c])) < 0.13 * (a[c] + b[c]), (mixed, a, b)
    multiple = mean(renderer, s, 2048, 3, integrator)
    assert multiple[0] > mixed[0] * 0.9 and multiple[2] > mixed[2] * 0.9, (multiple, mixed)


@pytest.mark.parametrize("integrator", BOTH)
def test_projector_segment_integral_matches_independent_quadrature(renderer, integrator):
    # gpu_volume_sampling.rs:122-218
    cfg = RenderConfig(width=32, height=32, samples_per_pixel=32, max_bounces=0, integrator=integrator)
    out = render(renderer, projector_scene(), cfg)
    c = out.color[..., :3].reshape(-1, 3).astype(np.float64)
    for ch in (0, 2):
        m = c[:, ch].mean()
        assert abs(m / PROJECTOR_QUADRATURE - 1.0) < 0.03, (ch, m)
        assert c[:, ch].std() / m < 0.16
    s = projector_scene(fog=False)
    s.lights = s.lights[:1]
    s.camera = Camera((0.0, 0.0, 0.0), (-3.0, 0.0, 10.0), 0.0, 1200.0, 0.0, 3.0)
    assert np.all(np.abs(render(renderer, s, cfg).color[..., :3]) < 1e-6)
    s.camera = Camera((3.0, 0.0, 10.0), (-3.0, 0.0, 10.0), 0.0, 1200.0, 0.0, 3.0)
    on = render(renderer, s, cfg).color
    assert np.all(np.abs(on[..., 0] - 50.0) < 1e-5) and np.all(on[..., 1:3] == 0.0)


def lit_fractal(fog):
    scene = workloads.mandelbox_scene()
    scene.lights = [TubeLight(start=(-2.5, 2.8, -2.0), end=(2.5, 2.8, -2.0), radius=0.12, color=(1.0, 0.6, 0.3),
                              intensity=12.0),
                    ProjectorLight(position=(3.0, 3.5, -4.0), normal=(-3.0, -3.5, 4.0), size=(0.8, 0.8),
                                   color=(0.4, 0.6, 1.0), intensity=40.0, inner_angle=12.0, outer_angle=25.0)]
    if fog:
        scene.fog = Fog(density=0.03, color=(0.9, 0.9, 0.9), height=1.0, falloff=0.5, anisotropy=0.2)
    return scene


@pytest.mark.parametrize("fog", [False, True])
def test_projector_and_tube_film_against_the_oracle(renderer, oracle_mod, fog):
    """Both integrators render the same film, bit for bit without fog (in fog the
    segment's line-integral terms are summed in another order by the two, as in
    test_fog: a few roundings of the sum), and it follows the f32 oracle's (RMSE <=
    2e-2 on seeded pixels, as the other film tests)."""
    scene = lit_fractal(fog)
    cfg = RenderConfig(width=96, height=54, samples_per_pixel=16, max_bounces=3, max_steps=512, tile_size=64,
                       samples_per_dispatch=8, integrator="wavefront")
    a = render(renderer, scene, cfg)
    cfg.integrator = "megakernel"
    b = render(renderer, scene, cfg)
    if fog:
        np.testing.assert_allclose(a.accum, b.accum, rtol=1e-5, atol=1e-6)
    else:
        np.testing.assert_array_equal(a.accum, b.accum)
    np.testing.assert_array_equal(a.depth, b.depth)
    assert (a.depth >= 0).mean() > 0.2
    rng = np.random.default_rng(11)
    pix = np.stack([rng.integers(0, cfg.width, 96), rng.integers(0, cfg.height, 96)], 1).astype(np.uint32)
    ref = oracle_mod.OracleGraph(scene.graph).render(scene.desc(cfg.width, cfg.height), cfg.desc(), pix, 0,
                                                     cfg.samples_per_pixel, precision=32)
    mine = a.accum[pix[:, 1], pix[:, 0], :3] / cfg.samples_per_pixel
    rmse = float(np.sqrt(np.mean((mine - ref["accum"][:, :3] / cfg.samples_per_pixel) ** 2)))
    assert rmse <= 2e-2, rmse
    assert float(mine.mean()) > 0.01


def test_light_parameters_are_bounded(renderer):
    """Light::visit_params (light.rs:162-226): projector angles, tube radius; a tube
    needs two distinct ends."""
    cfg = RenderConfig(width=8, height=8, samples_per_pixel=1)
    bad = [ProjectorLight(inner_angle=20.0, outer_angle=10.0), ProjectorLight(inner_angle=5.0, outer_angle=89.5),
           TubeLight(radius=0.0), TubeLight(start=(0.0, 1.0, 0.0), end=(0.0, 1.0, 0.0))]
    for light in bad:
        scene = workloads.mandelbox_scene()
        scene.lights = [light]
        with pytest.raises(SyfrackError):
            RenderSession(renderer, scene, cfg)
    scene = workloads.mandelbox_scene()
    scene.lights = [ProjectorLight(), TubeLight()]
    RenderSession(renderer, scene, cfg).close()

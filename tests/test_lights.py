"""Projector and tube lights (Light::Projector / Light::Tube, light.rs:88-105; their
emitter code lights.wgsl:5-160, 285-356; packing uniforms.rs:671-729) on the oracle,
with the reference's known answers: a tube filling the view is seen at exactly its
radiance (gpu_photometric.rs:74-86); a projector is dark outside its cone and seen at
exactly its radiance on its axis; the fog-scattered light of two projectors equals
the reference's independent area x line quadrature within 3%
(gpu_volume_sampling.rs:122-218). The device's versions are in test_gpu_lights.py."""
import numpy as np

from syfrack_gb300.graph import Graph, Kind, Link, Node
import pytest

from syfrack_gb300 import workloads
from syfrack_gb300.scene import AreaLight, Camera, Fog, Material, ProjectorLight, RenderConfig, Scene, SunLight, TubeLight


def minimal(kind):
    """Graph::new_minimal (graph/mod.rs:454-482) with its node 1 replaced."""
    return Graph([Node(0, Kind("Input")), Node(1, kind), Node(2, Kind("Output"))],
                 [Link((0, 0), (1, 0)), Link((1, 0), (2, 0))], safety=1.0, bounding_radius_hint=2.0)


def photometric_scene(kind, lights):
    """gpu_photometric.rs:9-34: camera at (0, 0, 3) looking at the origin, 500 mm,
    albedo 0.5 with no specular."""
    return Scene(graph=minimal(kind), camera=Camera((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), 0.0, 500.0, 0.0, 3.0),
                 material=Material(albedo=(0.5, 0.5, 0.5), roughness=0.5, metallic=0.0, specular=0.0),
                 lights=lights, seed=1)


def projector_scene(fog=True):
    """gpu_volume_sampling.rs:122-160: two projectors across the view of a camera
    looking down +z, a black plane far to the side, uniform fog."""
    lights = [ProjectorLight(position=(x, 0.0, 10.0), normal=(-np.sign(x), 0.0, 0.0), size=(2.0, 2.0), color=rgb,
                             intensity=50.0, inner_angle=10.0, outer_angle=18.0)
              for x, rgb in ((-3.0, (1.0, 0.0, 0.0)), (3.0, (0.0, 0.0, 1.0)))]
    return Scene(graph=minimal(Kind("Plane", normal=[1.0, 0.0, 0.0], offset=100.0)),
                 camera=Camera((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 0.0, 1200.0, 0.0, 3.0),
                 material=Material(albedo=(0.0, 0.0, 0.0), roughness=0.5, metallic=0.0, specular=0.0),
                 lights=lights, seed=1,
                 fog=Fog(density=0.014, color=(0.9, 0.9, 0.9), height=0.0, falloff=0.0, anisotropy=0.15) if fog else None)


# the reference's independent area x line Gauss-Legendre quadrature (128 x 128 x 256)
PROJECTOR_QUADRATURE = 0.015958553887736832


def oracle_pixels(oracle_mod, scene, w, h, spp, bounces, pixels=None, precision=32):
    cfg = RenderConfig(width=w, height=h, samples_per_pixel=spp, max_bounces=bounces)
    if pixels is None:
        pixels = [(x, y) for y in range(h) for x in range(w)]
    pix = np.array(pixels, np.uint32)
    r = oracle_mod.OracleGraph(scene.graph).render(scene.desc(w, h), cfg.desc(), pix, 0, spp, precision=precision)
    return r["accum"][:, :3] / spp


def test_tube_filling_the_view_is_seen_at_its_radiance(oracle_mod):
    # gpu_photometric.rs:74-86
    tube = TubeLight(start=(-2.0, 0.0, 1.0), end=(2.0, 0.0, 1.0), radius=0.7, color=(1.0, 0.1, 0.025), intensity=4.0)
    s = photometric_scene(Kind("Sphere", radius=0.01), [tube])
    c = oracle_pixels(oracle_mod, s, 24, 24, 4, 0)
    np.testing.assert_allclose(c.mean(0), [4.0, 0.4, 0.1], atol=1e-4)


def test_projector_is_dark_outside_its_cone_and_bright_on_its_axis(oracle_mod):
    # gpu_volume_sampling.rs:190-217 (without fog)
    s = projector_scene(fog=False)
    s.lights = s.lights[:1]
    s.camera = Camera((0.0, 0.0, 0.0), (-3.0, 0.0, 10.0), 0.0, 1200.0, 0.0, 3.0)
    off = oracle_pixels(oracle_mod, s, 32, 32, 32, 0, pixels=[(x, y) for y in range(0, 32, 4) for x in range(0, 32, 4)])
    assert np.all(np.abs(off) < 1e-6)
    s.camera = Camera((3.0, 0.0, 10.0), (-3.0, 0.0, 10.0), 0.0, 1200.0, 0.0, 3.0)
    on = oracle_pixels(oracle_mod, s, 32, 32, 32, 0, pixels=[(x, y) for y in range(0, 32, 4) for x in range(0, 32, 4)])
    assert np.all(np.abs(on[:, 0] - 50.0) < 1e-5) and np.all(on[:, 1:] == 0.0)


def test_projector_beams_in_fog_match_the_quadrature(oracle_mod):
    # gpu_volume_sampling.rs:160-189: the mean of each beam's channel within 3%, its
    # coefficient of variation over the pixels below 0.16
    c = oracle_pixels(oracle_mod, projector_scene(), 32, 32, 32, 0).astype(np.float64)
    for ch in (0, 2):
        mean = c[:, ch].mean()
        assert abs(mean / PROJECTOR_QUADRATURE - 1.0) < 0.03, (ch, mean)
        assert c[:, ch].std() / mean < 0.16, (ch, c[:, ch].std() / mean)


def compact_scene():
    """The Mandelbox workload scene lit by an area light, a sun and a tube."""
    scene = workloads.mandelbox_scene()
    scene.lights = scene.lights + [SunLight(direction=(-0.4, 0.8, 0.3), intensity=3.0),
                                   TubeLight(start=(-2.0, 3.0, -2.5), end=(2.0, 3.0, -2.5), radius=0.1, intensity=8.0)]
    return scene


def dark():
    """An emitter of zero radiance far below the scene (beyond the ray extent): it is
    never selected for next events (zero weight) and never met by a ray."""
    return AreaLight(position=(0.0, -5000.0, 0.0), normal=(0.0, -1.0, 0.0), size=(0.1, 0.1), intensity=0.0)


def padded_scene():
    """compact_scene's lights at indices 4, 10 and 11 of twelve: the area light among
    the eight the descriptor holds inline, the sun and the tube past them."""
    scene = compact_scene()
    area, sun, tube = scene.lights
    scene.lights = [dark() for _ in range(4)] + [area] + [dark() for _ in range(5)] + [sun, tube]
    return scene


def test_a_scene_of_97_lights_is_refused():
    # Scene::validate (scene/mod.rs:512-514), its test at :971-975
    scene = workloads.mandelbox_scene()
    scene.lights = [scene.lights[0]] * 97
    with pytest.raises(ValueError, match="at most 96 lights"):
        scene.desc(8, 8)
    scene.lights = [scene.lights[0]] * 96
    d = scene.desc(8, 8)
    assert d.light_count == 0 and d.light_list_count == 96 and d.light_list[95].radiance[0] == 10.0


def test_dark_lights_in_front_leave_the_film_unchanged(oracle_mod):
    w, h, spp = 24, 16, 4
    pix = [(x, y) for y in range(0, h, 2) for x in range(0, w, 2)]
    a = oracle_pixels(oracle_mod, compact_scene(), w, h, spp, 3, pixels=pix)
    b = oracle_pixels(oracle_mod, padded_scene(), w, h, spp, 3, pixels=pix)
    np.testing.assert_array_equal(a, b)
    assert a.mean() > 0.01

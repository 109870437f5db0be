"""The reference's analytic render tests (crates/syfrack-render/tests/gpu_render.rs),
restated on the device with their scenes, sizes and tolerances: white furnaces,
a sun on a Lambertian plane, the sun seen directly and in a mirror, fog in a furnace
and thin single scattering, next events at small pixel cones, identical lights
sharing the selection, the pixel tolerance's hit error, tile and dispatch
invariance, zero fog and cavity darkness. The reference renders with its default
integrator (the megakernel); the wavefront runs the analytic ones too."""
import math

import numpy as np
import pytest

from syfrack_gb300 import RenderSession, workloads
from syfrack_gb300.graph import Graph, Kind, Link, Node, sphere as sphere_graph
from syfrack_gb300.scene import (AreaLight, Camera, EnvironmentLight, Fog, Material, RenderConfig, Scene,
                                 SunLight)

pytestmark = pytest.mark.gpu
BOTH = ["megakernel", "wavefront"]


def sphere(radius, ground=None):
    """gpu_render.rs:12-53: graphs/sphere.ron with the sphere's radius (and its trap
    scale); with a ground, the plane at that offset, else the plane and the union
    dropped and the bounding hint set to the radius."""
    g = sphere_graph(radius=radius, ground=0.0 if ground is None else ground)
    for n in g.nodes:
        if n.kind.name == "Trap":
            n.kind.fields["scale"] = radius
    if ground is None:
        g.nodes = [n for n in g.nodes if n.kind.name not in ("Plane", "Union")]
        keep = {n.id for n in g.nodes}
        g.links = [l for l in g.links if l.src[0] in keep and l.dst[0] in keep]
        out = next(n.id for n in g.nodes if n.kind.name == "Output")
        sph = next(n.id for n in g.nodes if n.kind.name == "Sphere")
        g.links.append(Link((sph, 0), (out, 0)))
        g.bounding_radius_hint = radius
    return g


def furnace_scene():
    """gpu_render.rs:62-104: a unit sphere (albedo 0.5, roughness 0.5, no specular) in a
    uniform white environment, orbit camera at distance 3, 50 mm."""
    return Scene(graph=sphere(1.0), camera=Camera.orbit((0.0, 0.0, 0.0), 3.0, 0.0, 0.0, focal_mm=50.0),
                 material=Material(albedo=(0.5, 0.5, 0.5), roughness=0.5, metallic=0.0, specular=0.0),
                 lights=[EnvironmentLight(zenith=(1.0, 1.0, 1.0), horizon=(1.0, 1.0, 1.0), ground=(1.0, 1.0, 1.0),
                                          intensity=1.0)], seed=3)


def render(renderer, scene, cfg):
    s = RenderSession(renderer, scene, cfg)
    while not s.step(0):
        pass
    out = s.readback()
    assert s.sync() == 0
    s.close()
    return out


def mean_rgb(out, x0, y0, n):
    """gpu_render.rs:423-432: the mean of (r + g + b) / 3 over an n x n block."""
    c = out.color[y0:y0 + n, x0:x0 + n, :3].astype(np.float64)
    return float(c.mean())


def rim_pixel(out):
    """gpu_render.rs:436-452: the deepest hit whose 3x3 neighbourhood is all hits."""
    d = out.depth
    h, w = d.shape
    best, best_d = (w // 2, h // 2), -1.0
    for y in range(1, h - 1):
        for x in range(1, w - 1):
            if np.all(d[y - 1:y + 2, x - 1:x + 2] >= 0.0) and d[y, x] > best_d:
                best_d, best = float(d[y, x]), (x, y)
    return best


@pytest.mark.parametrize("integrator", BOTH)
def test_furnace_sphere_matches_albedo_and_background_matches_environment(renderer, integrator):
    # gpu_render.rs:456-476
    cfg = RenderConfig(width=48, height=48, samples_per_pixel=64, tile_size=32, integrator=integrator)
    out = render(renderer, furnace_scene(), cfg)
    centre, corner = mean_rgb(out, 22, 22, 4), mean_rgb(out, 0, 0, 3)
    assert abs(centre - 0.5) < 0.03, centre
    assert abs(corner - 1.0) < 1e-3, corner
    assert out.samples_min == 64 and out.samples_max == 64


def test_depth_of_centre_pixel_is_distance_minus_radius(renderer):
    # gpu_render.rs:479-491
    out = render(renderer, furnace_scene(), RenderConfig(width=33, height=33, samples_per_pixel=1))
    assert abs(out.depth[16, 16] - 2.0) < 0.05, out.depth[16, 16]
    assert out.depth[0, 0] < 0.0


@pytest.mark.parametrize("integrator", BOTH)
def test_furnace_rim_pixel_does_not_gain_energy(renderer, integrator):
    # gpu_render.rs:572-581
    out = render(renderer, furnace_scene(), RenderConfig(width=48, height=48, samples_per_pixel=256,
                                                         integrator=integrator))
    rx, ry = rim_pixel(out)
    m = mean_rgb(out, rx - 1, ry - 1, 3)
    assert 0.3 <= m <= 1.0, (m, rx, ry)


@pytest.mark.parametrize("integrator", BOTH)
def test_metallic_furnace_does_not_exceed_unit_energy(renderer, integrator):
    # gpu_render.rs:585-606
    scene = furnace_scene()
    scene.material = Material(albedo=(1.0, 1.0, 1.0), roughness=0.5, metallic=1.0, specular=0.04)
    out = render(renderer, scene, RenderConfig(width=48, height=48, samples_per_pixel=256, integrator=integrator))
    rx, ry = rim_pixel(out)
    centre, rim = mean_rgb(out, 22, 22, 4), mean_rgb(out, rx - 1, ry - 1, 3)
    assert centre <= 1.02 and rim <= 1.02, (centre, rim)


def test_output_is_identical_across_tile_size_and_samples_per_dispatch(renderer):
    # gpu_render.rs:610-636 (the reference's dispatch time budget has no counterpart:
    # sessions dispatch whole tiles)
    scene = workloads.mandelbox_scene()

    def run(tile, spd):
        return render(renderer, scene, RenderConfig(width=65, height=41, samples_per_pixel=16, tile_size=tile,
                                                    samples_per_dispatch=spd))

    a = run(32, 8)
    for b in (run(64, 8), run(32, 1), run(128, 8)):
        np.testing.assert_array_equal(a.color, b.color)
        np.testing.assert_array_equal(a.depth, b.depth)
        np.testing.assert_array_equal(a.normals, b.normals)


def lambert_plane_scene(focal_mm):
    """gpu_render.rs:641-684 / :994-1042: a plane at y = 0 (and a tiny sphere) seen from
    straight above under a sun straight above: radiance rho E / pi."""
    return Scene(graph=sphere(0.01, 0.0), camera=Camera((0.0, 3.0, 0.5), (0.0, 0.0, 0.5), 0.0, focal_mm, 0.0, 3.0),
                 material=Material(albedo=(0.5, 0.5, 0.5), roughness=0.5, metallic=0.0, specular=0.0),
                 lights=[SunLight(direction=(0.0, 1.0, 0.0), color=(1.0, 1.0, 1.0), intensity=2.0, angular_size=0.5)],
                 seed=5)


@pytest.mark.parametrize("integrator", BOTH)
def test_sun_irradiance_on_lambertian_plane_matches_albedo_e_over_pi(renderer, integrator):
    # gpu_render.rs:641-693
    out = render(renderer, lambert_plane_scene(50.0),
                 RenderConfig(width=16, height=16, samples_per_pixel=256, max_bounces=1, integrator=integrator))
    centre, expected = mean_rgb(out, 6, 6, 4), 0.5 * 2.0 / math.pi
    assert abs(centre - expected) < 0.03 * expected, (centre, expected)


@pytest.mark.parametrize("integrator", BOTH)
def test_nee_plane_is_exact_at_small_pixel_cones(renderer, integrator):
    # gpu_render.rs:994-1052
    out = render(renderer, lambert_plane_scene(1000.0),
                 RenderConfig(width=64, height=64, samples_per_pixel=512, max_bounces=1, integrator=integrator))
    centre, expected = mean_rgb(out, 30, 30, 4), 0.5 * 2.0 / math.pi
    assert abs(centre - expected) < 0.02 * expected, (centre, expected)


def mirror_scene():
    scene = furnace_scene()
    scene.lights = [SunLight(direction=(0.3, 0.9, 0.3), color=(1.0, 1.0, 1.0), intensity=2.0, angular_size=2.0)]
    scene.material = Material(albedo=(0.9, 0.9, 0.9), roughness=0.05, metallic=1.0, specular=0.04)
    return scene


@pytest.mark.parametrize("integrator", BOTH)
def test_sun_is_visible_in_a_mirror_reflection(renderer, integrator):
    # gpu_render.rs:770-805
    out = render(renderer, mirror_scene(), RenderConfig(width=64, height=64, samples_per_pixel=64, max_bounces=2,
                                                        integrator=integrator))
    lum = np.sort(out.color[..., 1].ravel())
    median, mx = float(lum[len(lum) // 2]), float(lum[-1])
    assert mx > 5.0, mx
    assert mx > 20.0 * max(median, 1e-3), (mx, median)


@pytest.mark.parametrize("integrator", BOTH)
def test_glossy_sun_highlight_survives_at_the_last_bounce(renderer, integrator):
    # gpu_render.rs:963-990
    out = render(renderer, mirror_scene(), RenderConfig(width=64, height=64, samples_per_pixel=64, max_bounces=0,
                                                        integrator=integrator))
    assert float(out.color[..., 1].max()) > 300.0


@pytest.mark.parametrize("integrator", BOTH)
def test_camera_ray_into_the_sun_sees_its_radiance(renderer, integrator):
    # gpu_render.rs:808-837: radiance E / solid angle of the disk
    scene = furnace_scene()
    scene.graph = sphere(0.01)
    scene.camera = Camera((0.0, 0.0, 5.0), (0.0, 0.0, 6.0), 0.0, 200.0, 0.0, 3.0)
    angular = 4.0
    scene.lights = [SunLight(direction=(0.0, 0.0, 1.0), color=(1.0, 1.0, 1.0), intensity=1.0, angular_size=angular)]
    out = render(renderer, scene, RenderConfig(width=33, height=33, samples_per_pixel=16, integrator=integrator))
    centre = float(out.color[16, 16, 0])
    expected = 1.0 / (2.0 * math.pi * (1.0 - math.cos(math.radians(angular * 0.5))))
    assert abs(centre - expected) < 0.05 * expected, (centre, expected)


@pytest.mark.parametrize("integrator", BOTH)
def test_weighted_area_selection_preserves_the_sum_of_identical_lights(renderer, integrator):
    # gpu_render.rs:397-420: two identical lamps equal one of twice the intensity
    lamp = dict(position=(0.0, 3.0, 3.0), normal=(0.0, -1.0, -1.0), size=(3.0, 3.0), color=(1.0, 1.0, 1.0))
    cfg = RenderConfig(width=32, height=32, samples_per_pixel=32, max_bounces=0, integrator=integrator)
    scene = furnace_scene()
    scene.lights = [AreaLight(intensity=4.0, **lamp), AreaLight(intensity=4.0, **lamp)]
    pair = render(renderer, scene, cfg)
    scene.lights = [AreaLight(intensity=8.0, **lamp)]
    one = render(renderer, scene, cfg)
    assert np.abs(pair.color[..., :3] - one.color[..., :3]).max() < 1e-5


def test_pixel_tolerance_reduces_analytic_sphere_hit_error(renderer):
    # gpu_render.rs:113-145: the hit radius recovered from depth and normal
    scene = furnace_scene()
    scene.camera = Camera((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), 0.0, 50.0, 0.0, 3.0)

    def mean_error(tol):
        out = render(renderer, scene, RenderConfig(width=64, height=64, samples_per_pixel=1, max_bounces=0,
                                                   max_steps=512, pixel_tolerance=tol))
        t = out.depth[20:44, 20:44].astype(np.float64)
        nz = out.normals[20:44, 20:44, 2].astype(np.float64)
        assert np.all(t > 0.0) and np.all(nz > 0.0)
        radius = 3.0 * nz - np.sqrt(np.maximum(t * t - 9.0 * (1.0 - nz * nz), 0.0))
        return float(np.abs(radius - 1.0).mean())

    coarse, fine = mean_error(1.0), mean_error(0.25)
    assert coarse > 1e-5 and fine < coarse * 0.6, (coarse, fine)


# The reference's two fog known answers were written for 100 units of fog along a ray
# that leaves the scene ("a ray crosses 100 units of fog", "optical depth ~2 to the far
# cap"); its renderer now marches and integrates fog over ray_extent() =
# max(T_MAX = 200, 2 * hint + |camera|) (common.wgsl:7, :206-208; uniforms.rs:778-782,
# "the old fixed 200-unit tracing distance"), which this build follows. The two tests
# below keep the reference's scenes and tolerances on that extent: the furnace at the
# optical depth the reference states (density 0.01 over 200 units), the single-scatter
# formula over 200 units.
@pytest.mark.parametrize("integrator", BOTH)
def test_scattering_fog_in_a_white_furnace_conserves_energy(renderer, integrator):
    # gpu_render.rs:870-896
    scene = furnace_scene()
    scene.material = Material(albedo=(1.0, 1.0, 1.0), roughness=0.5, metallic=0.0, specular=0.0)
    scene.fog = Fog(density=0.01, color=(1.0, 1.0, 1.0), height=50.0, falloff=0.1, anisotropy=0.3)
    out = render(renderer, scene, RenderConfig(width=32, height=32, samples_per_pixel=256, max_bounces=32,
                                               integrator=integrator))
    g = out.color[..., 1].astype(np.float64)
    assert abs(g.mean() - 1.0) < 0.06, g.mean()
    assert np.all(g < 1.3), g.max()


@pytest.mark.parametrize("integrator", BOTH)
def test_thin_scattering_fog_single_scatter_matches_analytic(renderer, integrator):
    # gpu_render.rs:1055-1091: L = E/(4 pi) (1 - e^-tau_ray) e^-tau_sun for single
    # scattering (no bounce after the scattering event), tau_ray over the ray extent;
    # two bounces add multiple scattering on top of it
    scene = furnace_scene()
    scene.graph = sphere(0.01)
    scene.camera = Camera((0.0, 0.0, 5.0), (0.0, 0.0, 6.0), 0.0, 1000.0, 0.0, 3.0)
    scene.lights = [SunLight(direction=(0.0, 1.0, 0.0), color=(1.0, 1.0, 1.0), intensity=2.0, angular_size=60.0)]
    scene.fog = Fog(density=0.001, color=(1.0, 1.0, 1.0), height=50.0, falloff=0.1, anisotropy=0.0)

    def centre(bounces):
        out = render(renderer, scene, RenderConfig(width=16, height=16, samples_per_pixel=4096, max_bounces=bounces,
                                                   integrator=integrator))
        return mean_rgb(out, 6, 6, 4)

    single, multiple = centre(0), centre(2)
    tau_ray, tau_sun = 0.001 * 200.0, 0.001 * 50.0 + 0.001 / 0.1
    expected = 2.0 / (4.0 * math.pi) * (1.0 - math.exp(-tau_ray)) * math.exp(-tau_sun)
    assert abs(single - expected) < 0.15 * expected, (single, expected)
    assert 1.0 < multiple / single < 1.35, (single, multiple)


def test_zero_fog_density_is_bit_identical_to_no_atmosphere(renderer):
    # gpu_render.rs:947-960
    a = workloads.mandelbox_scene()
    b = workloads.mandelbox_scene()
    b.fog = Fog(density=0.0, color=(0.3, 0.2, 0.1), height=0.0, falloff=1.0, anisotropy=0.5)
    cfg = RenderConfig(width=48, height=32, samples_per_pixel=4)
    np.testing.assert_array_equal(render(renderer, a, cfg).color, render(renderer, b, cfg).color)


def test_cavity_darkness_only_darkens_and_is_monotonic(renderer):
    # gpu_render.rs:840-867
    cfg = RenderConfig(width=48, height=48, samples_per_pixel=8)

    def with_cavity(c):
        s = workloads.mandelbox_scene()
        s.cavity_darkness = c
        return render(renderer, s, cfg).color[..., 1].astype(np.float64)

    a, mid, b = with_cavity(0.0), with_cavity(0.4), with_cavity(0.8)
    assert b.sum() < mid.sum() < a.sum()
    assert np.all(b <= a + 1e-4)

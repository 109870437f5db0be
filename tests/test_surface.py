"""The rest of the shade stage: finish details (finish_detail.wgsl), volumetric fractal
textures (texture.wgsl, pattern.wgsl), orbit colouring and dielectric optics
(optics.wgsl and radiance's optical branches, pathtrace.wgsl:833-1107).

CPU tests pin the oracle to the reference's own tests of these features:
texture.rs:217-263 (texture values bounded, varying and deterministic; fan mapping
periodic in its staggered rows) and gpu_optics.rs:14-111 (coverage cut-outs, a clear
interface, Beer-Lambert tint, a white furnace, subsurface random walk, total internal
reflection), with the reference's scenes and tolerances. GPU tests hold the device to
the same properties through both integrators, to the f32 oracle on seeded pixels, and
to the reference's GPU texture tests (gpu_render.rs:149-330: effects change shading but
not geometry; zero strengths and an unselected mask change nothing)."""
import numpy as np
import pytest

from syfrack_gb300 import SyfrackError
from syfrack_gb300.graph import Graph, Kind, Link, Node
from syfrack_gb300.scene import (AreaLight, Camera, Coloring, EnvironmentLight, Finish, FinishDetail,
                                 FINISH_PATTERNS, FractalTexture, Material, Optics, OrbitColoring, Ramp,
                                 RenderConfig, Scene, SunLight)


def minimal():
    """Graph::new_minimal (graph/mod.rs:454-482): a unit sphere."""
    return Graph([Node(0, Kind("Input")), Node(1, Kind("Sphere", radius=1.0)), Node(2, Kind("Output"))],
                 [Link((0, 0), (1, 0)), Link((1, 0), (2, 0))], safety=1.0, bounding_radius_hint=2.0)


def tagged_sphere(index=1):
    """A unit sphere whose surface carries MaterialTag `index`."""
    return Graph([Node(0, Kind("Input")), Node(1, Kind("Sphere", radius=1.0)),
                  Node(2, Kind("MaterialTag", index=index)), Node(3, Kind("Output"))],
                 [Link((0, 0), (1, 0)), Link((1, 0), (2, 0)), Link((2, 0), (3, 0))], safety=1.0,
                 bounding_radius_hint=2.0)


def optics_scene(optics, position=(0.0, 0.0, 3.0), target=(0.0, 0.0, 0.0)):
    """gpu_optics.rs:16-36: the minimal sphere, a 1000 mm pinhole at (0, 0, 3), a white
    gradient sky of radiance 1, the example scene's material."""
    mat = Material(albedo=(0.7, 0.65, 0.6), roughness=0.4, metallic=0.0, specular=0.04)
    mat.optics = optics
    return Scene(graph=minimal(), camera=Camera(position, target, 0.0, 1000.0, 0.0, 3.0), material=mat,
                 lights=[EnvironmentLight(zenith=(1.0, 1.0, 1.0), horizon=(1.0, 1.0, 1.0), ground=(1.0, 1.0, 1.0))])


ALL_PX = np.array([(x, y) for y in range(17) for x in range(24)], dtype=np.uint32)


def oracle_color(oracle_mod, scene, cfg, pixels=ALL_PX, texture=None, precision=32):
    og = oracle_mod.OracleGraph(scene.graph)
    tg = oracle_mod.OracleGraph(scene.material.texture.graph) if scene.material.texture else None
    d = scene.desc(cfg.width, cfg.height, texture_graph=tg.h if tg else None)
    out = og.render(d, cfg.desc(), pixels, 0, cfg.samples_per_pixel, precision=precision)
    return out["accum"] / cfg.samples_per_pixel, out


# ---------------------------------------------------------------------------- textures (oracle)
def default_texture():
    """FractalTexture::default (texture.rs:110-136): the bundled Mandelbox, trap 0."""
    return FractalTexture(graph=Graph.bundled("mandelbox"))


def texture_values(oracle_mod, tex, points):
    s = Scene(graph=minimal(), material=Material())
    s.material.texture = tex
    tg = oracle_mod.OracleGraph(tex.graph)
    return oracle_mod.texture_values(s.desc(8, 8, texture_graph=tg.h), tg, points)


def test_texture_values_are_bounded_varying_and_deterministic(oracle_mod):
    """texture.rs:217-231 on the shader's pattern_value."""
    tex = default_texture()
    pts = np.array([(i * 0.047, 0.31, -0.2) for i in range(40)], np.float32)
    v = texture_values(oracle_mod, tex, pts)
    assert np.all(np.isfinite(v)) and np.all((v >= 0) & (v <= 1))
    assert v.max() - v.min() > 0.05, (v.min(), v.max())
    one = np.array([(1.0, 1.0, 1.0)] * 2, np.float32)
    a = texture_values(oracle_mod, tex, one)
    assert a[0] == a[1]


def test_fan_texture_repeats_in_staggered_rows(oracle_mod):
    """texture.rs:233-263: a fan texture (period 2.6 x 2.0, 18 rays) repeats by 2.6 along
    x and by two rows (4.0) along z within 1e-5, stays in [0, 1] and keeps its detail."""
    tex = default_texture()
    tex.fan = (2.6, 2.0, 18)
    tex.rotation, tex.offset, tex.scale, tex.contrast = (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 1.0, 1.0
    p = np.array([0.37, 0.0, 0.71], np.float32)
    pts = np.array([p, p + np.float32([2.6, 0, 0]), p + np.float32([0, 0, 4.0])], np.float32)
    v = texture_values(oracle_mod, tex, pts)
    assert abs(v[0] - v[1]) < 1e-5 and abs(v[0] - v[2]) < 1e-5, v
    line = texture_values(oracle_mod, tex, np.array([(i * 0.026, 0.0, 0.8) for i in range(100)], np.float32))
    assert np.all(np.isfinite(line)) and np.all((line >= 0) & (line <= 1))
    assert line.max() - line.min() > 0.15


def test_orbit_texture_channel_keeps_its_sign(oracle_mod):
    """The Orbit channel is not clamped (pattern.wgsl:27-47): a negative trap weight gives
    negative values."""
    tex = default_texture()
    tex.channel = ("orbit", OrbitColoring(traps=(-1.0, 0.0, 0.0, 0.0)))
    tex.contrast = 1.0
    v = texture_values(oracle_mod, tex, np.array([(i * 0.05, 0.2, 0.1) for i in range(20)], np.float32))
    assert np.all(np.isfinite(v)) and v.min() < 0.0


# ---------------------------------------------------------------------------- optics (oracle)
def test_oracle_dielectric_coverage_beer_furnace_subsurface_and_tir(oracle_mod):
    """gpu_optics.rs:14-111 on the oracle (24x17, 32 samples per pixel)."""
    cfg = RenderConfig(24, 17, 32, max_bounces=0, pixel_tolerance=0.25)
    cut, _ = oracle_color(oracle_mod, optics_scene(Optics(opacity=0.0)), cfg)
    np.testing.assert_allclose(cut, 1.0, atol=1e-6)  # a cut-out shows the white sky
    cfg.max_bounces = 8
    clear, _ = oracle_color(oracle_mod, optics_scene(Optics(ior=1.0)), cfg)
    np.testing.assert_allclose(clear, 1.0, atol=1e-6)  # an index-matched interface is invisible
    tinted, _ = oracle_color(oracle_mod, optics_scene(Optics(ior=1.0, absorption_color=(0.5, 0.25, 1.0),
                                                             absorption_distance=2.0)), cfg)
    np.testing.assert_allclose(tinted.mean(0), [0.5, 0.25, 1.0], atol=0.002)  # Beer-Lambert over the chord 2
    s = optics_scene(Optics())
    s.material.roughness = 0.02
    cfg.max_bounces = 16
    furnace, _ = oracle_color(oracle_mod, s, cfg)
    assert np.all(np.isfinite(furnace)) and np.all(furnace >= 0)
    np.testing.assert_allclose(furnace.mean(0), 1.0, atol=0.015)  # glass in a white furnace
    cfg.max_bounces = 32
    scatter, _ = oracle_color(oracle_mod, optics_scene(Optics(ior=1.0, subsurface=1.0, subsurface_radius=0.35,
                                                              subsurface_color=(0.9, 0.5, 0.2))), cfg)
    r, g, b = scatter.mean(0)
    assert r > g > b and r < 1.0 and b > 0.0, (r, g, b)
    assert np.all(np.isfinite(scatter)) and np.all((scatter >= 0) & (scatter <= 1.0001))
    cfg.max_bounces = 8
    s = optics_scene(Optics(), position=(0.0, 0.0, 0.9), target=(1.0, 0.0, 0.9))
    s.material.roughness = 0.02  # the furnace's smooth glass (the reference mutates one scene)
    trapped, _ = oracle_color(oracle_mod, s, cfg)
    assert trapped.mean(0)[0] < 0.001  # total internal reflection keeps the paths inside


# ---------------------------------------------------------------------------- finish details (oracle)
def detail_scene(pattern, bump=0.02, fog=None):
    """A tagged sphere whose finish carries a detail pattern, lit by a softbox and the sky."""
    finish = Finish(albedo=(0.6, 0.55, 0.5), roughness=0.45, metallic=0.3, specular=0.04,
                    detail=FinishDetail(pattern=pattern, seed=11, scale=6.0, strength=0.8, bump=bump,
                                        roughness_delta=0.2, tint=(0.2, 0.3, 0.1)))
    mat = Material(albedo=(0.7, 0.7, 0.7), roughness=0.5)
    mat.finishes = [finish]
    return Scene(graph=tagged_sphere(1), camera=Camera((0.0, 0.6, 3.2), (0.0, 0.0, 0.0), 0.0, 40.0, 0.0, 3.0),
                 material=mat, lights=[AreaLight(position=(1.5, 2.5, 2.0), normal=(-0.4, -0.8, -0.5), size=(1.5, 1.5),
                                                 intensity=6.0), EnvironmentLight()],
                 dune_wind=35.0, seed=3)


def test_oracle_finish_details_shade_without_moving_geometry(oracle_mod):
    """Every pattern changes the colour of the tagged sphere but neither its depth nor the
    first-hit normal; f32 follows f64."""
    cfg = RenderConfig(24, 17, 4, max_bounces=2)
    plain = detail_scene("VeinedStone")
    plain.material.finishes[0].detail = None
    base, bout = oracle_color(oracle_mod, plain, cfg)
    for pattern in FINISH_PATTERNS:
        col, out = oracle_color(oracle_mod, detail_scene(pattern), cfg)
        assert np.all(np.isfinite(col)), pattern
        assert np.abs(col - base).mean() > 1e-3, pattern
        np.testing.assert_array_equal(out["depth"], bout["depth"])
        np.testing.assert_array_equal(out["aux"], bout["aux"])
    c32, _ = oracle_color(oracle_mod, detail_scene("Concrete"), cfg)
    c64, _ = oracle_color(oracle_mod, detail_scene("Concrete"), cfg, precision=64)
    assert float(np.sqrt(np.mean((c32 - c64) ** 2))) < 2e-2


def test_scene_descriptor_carries_surface_features():
    s = detail_scene("Sand")
    s.material.optics = Optics(opacity=0.5)
    s.material.coloring = Coloring(ramp=Ramp(), orbit=OrbitColoring(traps=(0.5, 0.5, 0.0, 0.0), logarithmic=2.0))
    d = s.desc(8, 8)
    assert d.details[0].pattern == FINISH_PATTERNS.index("Sand") + 1 and d.dune_wind == pytest.approx(35.0)
    assert d.optics[0].enabled == 1 and d.optics[0].opacity == pytest.approx(0.5) and d.optics[1].enabled == 0
    assert d.coloring.slot == 6 and d.coloring_orbit.logarithmic == pytest.approx(2.0)
    s.material.texture = default_texture()
    with pytest.raises(ValueError):
        s.desc(8, 8)  # a texture needs its compiled graph


# ---------------------------------------------------------------------------- device
def render(renderer, scene, cfg):
    from syfrack_gb300 import RenderSession

    s = RenderSession(renderer, scene, cfg)
    while not s.step(0):
        pass
    out = s.readback()
    s.close()
    return out


def both(renderer, scene, w, h, spp, **kw):
    out = {}
    for integ in ("wavefront", "megakernel"):
        cfg = RenderConfig(w, h, spp, integrator=integ, tile_size=64, samples_per_dispatch=min(spp, 8), **kw)
        out[integ] = render(renderer, scene, cfg)
    return out, cfg


@pytest.mark.gpu
def test_device_dielectric_coverage_beer_furnace_subsurface_and_tir(renderer):
    """gpu_optics.rs:14-111 through both integrators."""
    for integ in ("wavefront", "megakernel"):
        def run(scene, bounces):
            cfg = RenderConfig(24, 17, 32, max_bounces=bounces, pixel_tolerance=0.25, integrator=integ,
                               samples_per_dispatch=8)
            return render(renderer, scene, cfg).color[..., :3].reshape(-1, 3)

        np.testing.assert_allclose(run(optics_scene(Optics(opacity=0.0)), 0), 1.0, atol=1e-6, err_msg=integ)
        np.testing.assert_allclose(run(optics_scene(Optics(ior=1.0)), 8), 1.0, atol=1e-6, err_msg=integ)
        tinted = run(optics_scene(Optics(ior=1.0, absorption_color=(0.5, 0.25, 1.0), absorption_distance=2.0)), 8)
        np.testing.assert_allclose(tinted.mean(0), [0.5, 0.25, 1.0], atol=0.002, err_msg=integ)
        s = optics_scene(Optics())
        s.material.roughness = 0.02
        furnace = run(s, 16)
        assert np.all(np.isfinite(furnace)) and np.all(furnace >= 0), integ
        np.testing.assert_allclose(furnace.mean(0), 1.0, atol=0.015, err_msg=integ)
        scatter = run(optics_scene(Optics(ior=1.0, subsurface=1.0, subsurface_radius=0.35,
                                          subsurface_color=(0.9, 0.5, 0.2))), 32)
        r, g, b = scatter.mean(0)
        assert r > g > b and r < 1.0 and b > 0.0, (integ, r, g, b)
        assert np.all((scatter >= 0) & (scatter <= 1.0001)), integ
        s = optics_scene(Optics(), position=(0.0, 0.0, 0.9), target=(1.0, 0.0, 0.9))
        s.material.roughness = 0.02
        trapped = run(s, 8)
        assert trapped.mean(0)[0] < 0.001, integ


def glass_bulb_scene():
    """Glass, frosted coverage and a tinted thin sheet on a tagged Mandelbulb beside a
    diffuse one, under a softbox, a sun and the sky: every optical branch at once."""
    from syfrack_gb300 import workloads

    _, cam, *_ = workloads.mandelbulb_primary()
    bulb = workloads.mandelbulb_primary_graph()
    mat = Material(albedo=(0.8, 0.75, 0.7), roughness=0.3)
    mat.optics = Optics(ior=1.45, absorption_color=(0.8, 0.9, 0.6), absorption_distance=1.5, opacity=0.85,
                        transmission=0.9, subsurface=0.3, subsurface_radius=0.8)
    return Scene(graph=bulb, camera=cam, material=mat,
                 lights=[AreaLight(position=(0.0, 2.5, 1.0), normal=(0.0, -1.0, -0.3), size=(1.5, 1.5), intensity=8.0),
                         SunLight(direction=(0.3, 0.9, -0.2), intensity=2.0), EnvironmentLight()], seed=9)


def glass_sphere_scene():
    """A frosted, tinted, scattering glass sphere and a thin tinted sheet finish on a
    tagged half, under a softbox, a sun and the sky."""
    g = Graph([Node(0, Kind("Input")), Node(1, Kind("Sphere", radius=1.0)),
               Node(2, Kind("Box", half=[0.8, 0.02, 0.8])), Node(3, Kind("Translate", offset=[0.0, 1.3, 0.0])),
               Node(4, Kind("MaterialTag", index=1)), Node(5, Kind("Union")), Node(6, Kind("Output"))],
              [Link((0, 0), (1, 0)), Link((0, 0), (3, 0)), Link((3, 0), (2, 0)), Link((2, 0), (4, 0)),
               Link((1, 0), (5, 0)), Link((4, 0), (5, 1)), Link((5, 0), (6, 0))], safety=1.0, bounding_radius_hint=2.0)
    mat = Material(albedo=(0.8, 0.75, 0.7), roughness=0.15)
    mat.optics = Optics(ior=1.5, absorption_color=(0.7, 0.85, 0.6), absorption_distance=1.2, opacity=0.9,
                        transmission=0.95, subsurface=0.4, subsurface_radius=0.6)
    sheet = Finish(albedo=(0.9, 0.9, 0.9), roughness=0.1, metallic=0.0, specular=0.04,
                   optics=Optics(thin_walled=True, absorption_color=(0.9, 0.5, 0.4), opacity=0.7))
    mat.finishes = [sheet]
    return Scene(graph=g, camera=Camera((0.4, 0.9, 3.2), (0.0, 0.2, 0.0), 0.0, 40.0, 0.0, 3.0), material=mat,
                 lights=[AreaLight(position=(1.5, 3.0, 1.5), normal=(-0.4, -0.8, -0.4), size=(1.5, 1.5), intensity=8.0),
                         SunLight(direction=(0.3, 0.9, -0.2), intensity=2.0), EnvironmentLight()], seed=4)


@pytest.mark.gpu
def test_device_optics_follow_the_oracle(renderer, oracle_mod):
    """A glass sphere under a tinted sheet (coverage, refraction, absorption, subsurface,
    thin walls, shadows through coverage, all three light kinds): both integrators agree
    and follow the f32 oracle within the film tolerance on 128 seeded pixels."""
    scene = glass_sphere_scene()
    out, cfg = both(renderer, scene, 96, 64, 16, max_bounces=6, max_steps=256)
    wf, mk = out["wavefront"], out["megakernel"]
    assert np.all(np.isfinite(wf.accum)) and np.all(np.isfinite(mk.accum))
    assert float(np.sqrt(np.mean((wf.color[..., :3] - mk.color[..., :3]) ** 2))) < 1e-2
    rng = np.random.default_rng(5)
    pix = np.stack([rng.integers(0, 96, 128), rng.integers(0, 64, 128)], 1).astype(np.uint32)
    ref, _ = oracle_color(oracle_mod, scene, cfg, pixels=pix)
    mine = wf.color[pix[:, 1], pix[:, 0], :3]
    rmse = float(np.sqrt(np.mean((mine - ref) ** 2)))
    assert rmse <= 2e-2, rmse
    assert mine.mean() > 0.05


@pytest.mark.gpu
def test_glass_mandelbulb_at_the_binary32_floor(renderer, oracle_mod):
    """A glass Mandelbulb: the Newton refinement on a fractal field (steps clamped to 0.5)
    and the refractions make paths chaotic, so the f32 oracle itself differs from FP64
    by branch flips. The device is held to that floor: its image error against the f32
    oracle at most 1.5 times the f32 oracle's against FP64, its mean within 2%."""
    scene = glass_bulb_scene()
    out, cfg = both(renderer, scene, 96, 64, 32, max_bounces=4, max_steps=256)
    wf, mk = out["wavefront"], out["megakernel"]
    assert np.all(np.isfinite(wf.accum)) and np.all(np.isfinite(mk.accum))
    rng = np.random.default_rng(5)
    pix = np.stack([rng.integers(0, 96, 128), rng.integers(0, 64, 128)], 1).astype(np.uint32)
    ref32, _ = oracle_color(oracle_mod, scene, cfg, pixels=pix)
    ref64, _ = oracle_color(oracle_mod, scene, cfg, pixels=pix, precision=64)
    floor = float(np.sqrt(np.mean((ref32 - ref64) ** 2)))
    for film in (wf, mk):
        mine = film.color[pix[:, 1], pix[:, 0], :3]
        rmse = float(np.sqrt(np.mean((mine - ref32) ** 2)))
        assert rmse <= 1.5 * floor + 2e-3, (rmse, floor)
        assert abs(mine.mean() - ref64.mean()) <= 0.02 * ref64.mean(), (mine.mean(), ref64.mean())


@pytest.mark.gpu
def test_device_finish_details_follow_the_oracle(renderer, oracle_mod):
    """Each pattern on the tagged sphere: the device film follows the f32 oracle and keeps
    the geometry of the undetailed render (depth and first-hit normals)."""
    plain = detail_scene("VeinedStone")
    plain.material.finishes[0].detail = None
    base, _ = both(renderer, plain, 48, 34, 4, max_bounces=2)
    for pattern in FINISH_PATTERNS:
        scene = detail_scene(pattern)
        out, cfg = both(renderer, scene, 48, 34, 4, max_bounces=2)
        for integ, film in out.items():
            np.testing.assert_array_equal(film.depth, base[integ].depth, err_msg=pattern)
            assert np.all(np.isfinite(film.accum)), pattern
        rng = np.random.default_rng(7)
        pix = np.stack([rng.integers(0, 48, 96), rng.integers(0, 34, 96)], 1).astype(np.uint32)
        ref, _ = oracle_color(oracle_mod, scene, cfg, pixels=pix)
        mine = out["wavefront"].color[pix[:, 1], pix[:, 0], :3]
        rmse = float(np.sqrt(np.mean((mine - ref) ** 2)))
        assert rmse <= 2e-2, (pattern, rmse)
        assert np.abs(out["wavefront"].color - base["wavefront"].color).mean() > 1e-3, pattern


def textured_scene(**kw):
    """gpu_render.rs:149-203: the example's metallic 0.5 form with a fractal texture."""
    from syfrack_gb300 import workloads

    scene = workloads.mandelbox_scene()
    scene.material.metallic = 0.5
    tex = default_texture()
    for k, v in kw.items():
        setattr(tex, k, v)
    scene.material.texture = tex
    return scene


@pytest.mark.gpu
def test_texture_changes_colour_roughness_and_relief_without_changing_geometry(renderer):
    """gpu_render.rs:149-203: zero strengths keep the render; colour, roughness and bump
    each change it while depth and first-hit normals stay."""
    cfg = RenderConfig(48, 48, 16, max_bounces=1, integrator="wavefront", samples_per_dispatch=8)
    base_scene = textured_scene()
    base_scene.material.texture = None
    base = render(renderer, base_scene, cfg)
    neutral = render(renderer, textured_scene(strength=0.0, roughness=0.0, bump=0.0), cfg)
    # the textured scene runs the kernel built with the texture interpreter, whose fused
    # operations elsewhere may round differently: equal to float rounding (the
    # reference's bound is a mean difference below 1e-6)
    np.testing.assert_allclose(neutral.accum, base.accum, rtol=1e-6, atol=1e-7)
    assert np.abs(neutral.color - base.color).mean() < 1e-6
    for effect in ("strength", "roughness", "bump"):
        kw = dict(strength=0.0, roughness=0.0, bump=0.0)
        kw[effect] = 0.8
        out = render(renderer, textured_scene(**kw), cfg)
        np.testing.assert_array_equal(out.depth, base.depth, err_msg=effect)
        np.testing.assert_array_equal(out.normals, base.normals, err_msg=effect)
        assert np.all(np.isfinite(out.color)) and np.all(out.color >= 0), effect
        assert np.abs(out.color[..., :3] - base.color[..., :3]).sum(-1).mean() > 0.002, effect


@pytest.mark.gpu
def test_parallax_and_mask(renderer):
    """gpu_render.rs:260-283 and :308-330: parallax offsets the texture lookups only; a
    mask on an unwritten trap (value 1) selects nothing, one at the trap's value does."""
    cfg = RenderConfig(48, 32, 16, max_bounces=1, integrator="wavefront", samples_per_dispatch=8)
    flat = render(renderer, textured_scene(scale=2.0, roughness=0.0, bump=0.15), cfg)
    deep = render(renderer, textured_scene(scale=2.0, roughness=0.0, bump=0.15, parallax=0.5, parallax_steps=16), cfg)
    np.testing.assert_array_equal(flat.depth, deep.depth)
    np.testing.assert_array_equal(flat.normals, deep.normals)
    assert not np.array_equal(flat.color, deep.color)
    assert np.all(np.isfinite(deep.color)) and np.all(deep.color >= 0)
    base_scene = textured_scene()
    base_scene.material.texture = None
    base = render(renderer, base_scene, cfg)
    masked = render(renderer, textured_scene(fan=(2.6, 2.0, 18), mask=(3, 0.0, 0.05)), cfg)  # trap 3 unwritten
    np.testing.assert_allclose(masked.accum, base.accum, rtol=1e-6, atol=1e-7)  # the textured kernel's rounding
    shown = render(renderer, textured_scene(fan=(2.6, 2.0, 18), mask=(3, 1.0, 0.05)), cfg)
    assert not np.array_equal(shown.accum, base.accum)
    np.testing.assert_array_equal(shown.depth, base.depth)


@pytest.mark.gpu
def test_device_texture_follows_the_oracle(renderer, oracle_mod):
    """A textured Mandelbox with parallax and relief, orbit-coloured: both integrators
    agree and follow the f32 oracle on seeded pixels."""
    scene = textured_scene(parallax=0.3, parallax_steps=12, bump=0.4)
    scene.material.coloring = Coloring(ramp=Ramp(stops=[(0.9, 0.5, 0.2), (0.2, 0.4, 0.9)]),
                                       orbit=OrbitColoring(traps=(0.7, 0.0, 0.0, 0.3), iterations=0.2,
                                                           logarithmic=1.5))
    out, cfg = both(renderer, scene, 64, 36, 4, max_bounces=2, max_steps=512, hit_epsilon=1e-4)
    diff = out["wavefront"].color[..., :3] - out["megakernel"].color[..., :3]
    assert float(np.sqrt(np.mean(diff ** 2))) < 2e-2
    rng = np.random.default_rng(13)
    pix = np.stack([rng.integers(0, 64, 96), rng.integers(0, 36, 96)], 1).astype(np.uint32)
    ref, _ = oracle_color(oracle_mod, scene, cfg, pixels=pix)
    mine = out["wavefront"].color[pix[:, 1], pix[:, 0], :3]
    rmse = float(np.sqrt(np.mean((mine - ref) ** 2)))
    assert rmse <= 2e-2, rmse


@pytest.mark.gpu
def test_surface_feature_jobs_in_a_batch_equal_their_sessions(renderer):
    """A detailed, a textured, a glass and a plain job batched together: each film equals
    the job rendered alone by a session (the batch runs the multi-job trace kernel with
    the optics states and the shading kernel with the texture interpreter)."""
    from syfrack_gb300 import Batch

    cfg = RenderConfig(48, 32, 4, max_bounces=3, max_steps=256, pixel_tolerance=1.0, tile_size=48,
                       samples_per_dispatch=4, integrator="wavefront")
    plain = detail_scene("Patina")
    plain.material.finishes[0].detail = None
    jobs = [(detail_scene("Concrete"), cfg), (textured_scene(bump=0.4, parallax=0.2), cfg), (glass_sphere_scene(), cfg),
            (plain, cfg)]
    b = Batch(renderer, jobs)
    b.run(1, use_graph=False)
    assert b.sync() == 0
    for i, (sc, c) in enumerate(jobs):
        got = b.readback(i)
        ref = render(renderer, sc, c)
        scale = max(1.0, float(np.abs(ref.accum[..., :3]).max()))
        err = np.abs(got.accum[..., :3] - ref.accum[..., :3])
        # the glass job's refractions amplify last-ulp differences between the two
        # kernels into a few diverging samples: its bound is on the image, not per pixel
        if i == 2:
            assert float(np.sqrt(np.mean((got.color - ref.color) ** 2))) < 1e-2, i
        else:
            assert err.max() <= 1e-4 * scale, (i, float(err.max()))
    b.close()


@pytest.mark.gpu
def test_surface_feature_previews_served_equal_their_sessions(renderer):
    """A detailed, a textured and a glass preview, each with a refinement, served
    together: every film equals the same samples rendered by a session (the server's
    batched kernels, the session's per-form ones)."""
    from syfrack_gb300 import Server
    from syfrack_gb300.serve import DONE

    scenes = [detail_scene("Sand"), textured_scene(bump=0.3), glass_sphere_scene()]
    cfg = RenderConfig(48, 32, 2, max_bounces=3, max_steps=256, pixel_tolerance=1.0, tile_size=48,
                       samples_per_dispatch=2, integrator="wavefront")
    srv = Server(renderer, hbm_budget=1 << 30, path_capacity=1 << 16)
    previews = [srv.preview(sc, cfg) for sc in scenes]
    refines = [srv.refine(t, 2) for t in previews]
    for t in previews:
        assert srv.wait(t).state == DONE
    results = [srv.wait(t) for t in refines]
    for i, (sc, r) in enumerate(zip(scenes, results)):
        assert r.state == DONE and r.status == 0, i
        ref = render(renderer, sc, RenderConfig(**{**cfg.__dict__, "samples_per_pixel": 4}))
        if i == 2:  # the glass refractions amplify last-ulp differences between the kernels
            got = r.accum[..., :3] / np.maximum(r.accum[..., 3:], 1)
            assert float(np.sqrt(np.mean((got - ref.color[..., :3]) ** 2))) < 1e-2
        else:
            scale = max(1.0, float(np.abs(ref.accum[..., :3]).max()))
            assert np.abs(r.accum[..., :3] - ref.accum[..., :3]).max() <= 1e-4 * scale, i
    for t in previews + refines:
        srv.release(t)
    srv.close()


@pytest.mark.gpu
def test_textured_scenes_are_not_checkpointed(renderer, tmp_path):
    """The texture graph is a caller object (like a panorama): no checkpoint."""
    from syfrack_gb300 import RenderSession

    cfg = RenderConfig(32, 32, 4, max_bounces=1, integrator="wavefront")
    s = RenderSession(renderer, textured_scene(), cfg)
    s.step(0)
    with pytest.raises(SyfrackError, match="SF_ERR_UNSUPPORTED"):
        s.save(str(tmp_path / "ck"))
    s.close()

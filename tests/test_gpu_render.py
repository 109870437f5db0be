"""Path-traced film on the GPU: wavefront stages against the per-pixel
megakernel, both against the oracle; session stepping, checkpoints (GPU).

Reference conventions: accum holds sample sums added in ascending sample order
(pathtrace.wgsl:1243-1245); depth/aux from sample 0; the wavefront result equals
the tiled megakernel (gpu_export.rs:110-163 uses 1e-4); save/resume is
bit-for-bit (gpu_render.rs:1120); a corrupt state is refused (:1180)."""
import os

import numpy as np
import pytest

from syfrack_gb300 import RenderSession, SyfrackError, workloads
from syfrack_gb300.graph import Graph
from syfrack_gb300.scene import AreaLight, Camera, Material, RenderConfig, Scene

pytestmark = pytest.mark.gpu


def small_cfg(integrator, w=96, h=54, spp=8, spd=4, tile=64):
    return RenderConfig(width=w, height=h, samples_per_pixel=spp, max_bounces=4, max_steps=512,
                        pixel_tolerance=1.0, tile_size=tile, samples_per_dispatch=spd, integrator=integrator)


def render(renderer, scene, cfg):
    s = RenderSession(renderer, scene, cfg)
    while not s.step(0):
        pass
    out = s.readback()
    assert s.sync() == 0
    s.close()
    return out


def test_wavefront_equals_megakernel(renderer):
    scene = workloads.mandelbox_scene()
    a = render(renderer, scene, small_cfg("wavefront"))
    b = render(renderer, scene, small_cfg("megakernel"))
    assert a.accum[..., 3].min() == 8 and b.accum[..., 3].min() == 8
    diff = np.abs(a.accum[..., :3] - b.accum[..., :3])
    assert diff.max() <= 1e-4 * max(1.0, float(np.abs(b.accum[..., :3]).max()))
    np.testing.assert_array_equal(a.depth >= 0, b.depth >= 0)
    np.testing.assert_allclose(a.depth, b.depth, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(a.normals, b.normals, atol=1e-5)
    assert a.color[..., :3].mean() > 0.01  # the light reaches the form


@pytest.mark.parametrize("shape", [(2, 16, 1), (4, 64, 8), (3, 256, 32), (7, 0, 4), (6, 128, 8)])
def test_launch_shapes_give_the_same_film(renderer, shape):
    # march state saved at a step quantum and resumed by the next launch, any
    # regeneration threshold and any register budget: the same film bit for bit
    scene = workloads.mandelbox_scene()
    cfg = small_cfg("wavefront")
    base = RenderSession(renderer, scene, cfg)
    base.set_launch(3, 0, 4)
    while not base.step(0):
        pass
    ref = base.readback()
    base.close()
    s = RenderSession(renderer, scene, cfg)
    s.set_launch(*shape)
    while not s.step(0):
        pass
    out = s.readback()
    assert s.sync() == 0
    s.close()
    np.testing.assert_array_equal(out.accum, ref.accum)
    np.testing.assert_array_equal(out.depth, ref.depth)


def test_film_planes(renderer):
    # without fog or volumes: volume and moments carry only the sample counts, surface = accum
    scene = workloads.mandelbox_scene()
    cfg = small_cfg("wavefront", spp=4, spd=4, tile=96)
    s = RenderSession(renderer, scene, cfg)
    s.dispatch((0, 0, cfg.width, cfg.height, 0), 4)
    s.sync()
    p = s.film_planes()
    r = s.readback()
    s.close()
    np.testing.assert_array_equal(p["accum"], r.accum)
    np.testing.assert_array_equal(p["surface"], p["accum"])
    for k in ("volume", "moments"):
        assert (p[k][..., :3] == 0).all()
        np.testing.assert_array_equal(p[k][..., 3], p["accum"][..., 3])
    np.testing.assert_array_equal(p["depth"], r.depth)


def test_film_against_oracle(renderer, oracle_mod):
    scene = workloads.mandelbox_scene()
    cfg = small_cfg("wavefront", spp=16, spd=8)
    out = render(renderer, scene, cfg)
    rng = np.random.default_rng(1)
    pix = np.stack([rng.integers(0, cfg.width, 96), rng.integers(0, cfg.height, 96)], 1).astype(np.uint32)
    og = oracle_mod.OracleGraph(scene.graph)
    for prec, tol in ((32, 2e-2), (64, 2e-2)):
        ref = og.render(scene.desc(cfg.width, cfg.height), cfg.desc(), pix, 0, cfg.samples_per_pixel, precision=prec)
        mine = out.accum[pix[:, 1], pix[:, 0], :3] / cfg.samples_per_pixel
        mean_ref = ref["accum"] / cfg.samples_per_pixel
        rmse = float(np.sqrt(np.mean((mine - mean_ref) ** 2)))
        assert rmse <= tol, (prec, rmse)
        hit = ref["depth"] >= 0
        np.testing.assert_array_equal(out.depth[pix[:, 1], pix[:, 0]] >= 0, hit)
        np.testing.assert_allclose(out.depth[pix[:, 1], pix[:, 0]][hit], ref["depth"][hit], rtol=1e-3)


def test_step_equals_one_shot(renderer):
    scene = workloads.mandelbox_scene()
    cfg = small_cfg("wavefront", spp=8, spd=8, tile=128)
    a = render(renderer, scene, cfg)
    cfg2 = small_cfg("wavefront", spp=8, spd=2, tile=32)
    b = render(renderer, scene, cfg2)
    np.testing.assert_array_equal(a.accum, b.accum)
    np.testing.assert_array_equal(a.depth, b.depth)


def test_readback_colour_is_the_mean(renderer):
    """RenderOutput.color (renderer.rs:151-164) is filled by the library's readback:
    accum rgb / max(count, 1), alpha 1, the same numbers numpy gives."""
    scene = workloads.mandelbox_scene()
    out = render(renderer, scene, small_cfg("wavefront", spp=4, spd=4, tile=128))
    want = out.accum[..., :3] / np.maximum(out.accum[..., 3:4], np.float32(1.0))
    np.testing.assert_array_equal(out.color[..., :3], want)
    assert np.all(out.color[..., 3] == 1.0)


def test_save_resume_bit_for_bit(renderer, tmp_path):
    scene = workloads.mandelbox_scene()
    cfg = small_cfg("wavefront", spp=8, spd=4)
    full = render(renderer, scene, cfg)
    s = RenderSession(renderer, scene, cfg)
    s.step(1)  # stops after the first dispatch that exceeds 1 ms
    d = str(tmp_path / "ck")
    s.save(d)
    prog = s.progress()
    s.close()
    r = RenderSession.resume(renderer, scene, cfg, d)
    assert r.progress()["pixel_samples_done"] == prog["pixel_samples_done"]
    while not r.step(0):
        pass
    out = r.readback()
    np.testing.assert_array_equal(out.accum, full.accum)
    np.testing.assert_array_equal(out.depth, full.depth)
    r.close()


def test_corrupt_and_foreign_checkpoints_are_refused(renderer, tmp_path):
    scene = workloads.mandelbox_scene()
    cfg = small_cfg("wavefront", spp=4, spd=4)
    s = RenderSession(renderer, scene, cfg)
    s.step(0)
    d = str(tmp_path / "ck")
    s.save(d)
    s.close()
    film = os.path.join(d, "film.bin")
    data = bytearray(open(film, "rb").read())
    data[100] ^= 0xFF
    open(film, "wb").write(bytes(data))
    with pytest.raises(SyfrackError) as e:
        RenderSession.resume(renderer, scene, cfg, d)
    assert e.value.status == 9
    s = RenderSession(renderer, scene, cfg)
    s.step(0)
    s.save(d)
    s.close()
    other = Scene(graph=Graph.bundled("menger"), camera=scene.camera, lights=scene.lights)
    with pytest.raises(SyfrackError) as e:
        RenderSession.resume(renderer, other, cfg, d)
    assert e.value.status == 9


def test_sphere_centre_depth(renderer):
    # gpu_render.rs:479: centre-pixel depth = camera distance - radius
    g = Graph.bundled("sphere", ground=-50.0)
    scene = Scene(graph=g, camera=Camera.look_at((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), 40.0),
                  lights=[AreaLight(position=(0, 3, -2))])
    cfg = RenderConfig(width=65, height=65, samples_per_pixel=1, max_bounces=1, integrator="wavefront")
    out = render(renderer, scene, cfg)
    assert abs(out.depth[32, 32] - 3.0) < 2e-2
    n = out.normals[32, 32, :3]
    assert n[2] < -0.99


def test_config_validation(renderer):
    scene = workloads.mandelbox_scene()
    with pytest.raises(SyfrackError):
        RenderSession(renderer, scene, RenderConfig(width=8, height=8, samples_per_pixel=1, max_bounces=33))
    with pytest.raises(SyfrackError):
        RenderSession(renderer, scene, RenderConfig(width=8, height=8, samples_per_pixel=1, pixel_tolerance=2.0))


def test_budget_admission(gpu_ctx):
    from syfrack_gb300 import GpuContext, Renderer

    ctx = GpuContext(hbm_budget=8 << 20)
    r = Renderer(ctx)
    with pytest.raises(SyfrackError) as e:
        RenderSession(r, workloads.mandelbox_scene(), workloads.mandelbox_pathtrace_config())
    assert e.value.status == 7
    ctx.close()


@pytest.mark.parametrize("name", ["mandelbulb", "mandelbox", "menger"])
def test_unit_normals_each_fractal(renderer, name):
    # first-hit normals (tetrahedral taps, normalised) are unit vectors on every form
    g = Graph.bundled(name)
    d = 3.0 if name != "mandelbox" else 7.0
    cam = Camera.look_at((0.3 * d, 0.4 * d, -d), (0.0, 0.0, 0.0), 50.0)
    light = AreaLight(position=(0.0, d, 0.0), normal=(0.0, -1.0, 0.0), size=(1.0, 1.0), intensity=10.0)
    scene = Scene(graph=g, camera=cam, material=Material(albedo=(0.7, 0.7, 0.7)), lights=[light], seed=3)
    cfg = small_cfg("wavefront", spp=1, spd=1, tile=96)
    out = render(renderer, scene, cfg)
    hit = out.depth >= 0
    assert hit.mean() > 0.05
    lengths = np.linalg.norm(out.normals[..., :3][hit], axis=-1)
    assert np.abs(lengths - 1.0).max() < 1e-3


def test_rerender_is_bit_identical(renderer):
    scene = workloads.mandelbox_scene()
    a = render(renderer, scene, small_cfg("wavefront"))
    b = render(renderer, scene, small_cfg("wavefront"))
    np.testing.assert_array_equal(a.accum, b.accum)
    np.testing.assert_array_equal(a.depth, b.depth)
    np.testing.assert_array_equal(a.normals, b.normals)


def test_image_error_at_the_fp32_floor(renderer, oracle_mod):
    # The estimator branches (hit or miss, light selection, roulette) on values that
    # last-ulp differences can flip, so any binary32 evaluation differs from FP64 on a
    # few percent of pixels. The device's error against the FP64 oracle must stay at
    # the level of the reference's own binary32 arithmetic (the f32 oracle).
    scene = workloads.mandelbox_scene()
    cfg = workloads.mandelbox_pathtrace_config(width=320, height=180, spp=16, samples_per_dispatch=8)
    out = render(renderer, scene, cfg)
    rng = np.random.default_rng(7)
    pix = np.stack([rng.integers(0, cfg.width, 2048), rng.integers(0, cfg.height, 2048)], 1).astype(np.uint32)
    og = oracle_mod.OracleGraph(scene.graph)
    desc, cd = scene.desc(cfg.width, cfg.height), cfg.desc()
    r64 = og.render(desc, cd, pix, 0, cfg.samples_per_pixel, precision=64)["accum"] / cfg.samples_per_pixel
    r32 = og.render(desc, cd, pix, 0, cfg.samples_per_pixel, precision=32)["accum"] / cfg.samples_per_pixel
    mine = out.accum[pix[:, 1], pix[:, 0], :3] / cfg.samples_per_pixel
    rmse = lambda a, b: float(np.sqrt(np.mean((a - b) ** 2)))
    device, floor = rmse(mine, r64), rmse(r32, r64)
    per_pixel = np.sqrt(np.mean((mine - r64) ** 2, axis=1))
    print(f"image error vs FP64: device {device:.2e}, f32 oracle {floor:.2e}")
    assert np.median(per_pixel) < 1e-5  # most pixels follow the same paths
    assert device <= 1.5 * floor + 2e-3, (device, floor)


@pytest.mark.parametrize("graph", ["bounded", "mandelbulb"])
def test_skippable_bound_film(renderer, oracle_mod, graph):
    """A Bounded Mandelbulb beside a sphere (and the plain Mandelbulb close up): the
    trace kernel and the megakernel both march on the fast sample with the exact
    re-evaluation near acceptance, and agree with each other and with the f32 oracle."""
    from helpers import bounded_bulb

    mat = Material(albedo=(0.7, 0.7, 0.7), roughness=0.2, metallic=0.0, specular=0.04)
    light = AreaLight(position=(0.5, 3.0, -2.5), normal=(-0.5, -3.0, 2.5), size=(1.0, 1.0),
                      color=(1.0, 1.0, 1.0), intensity=10.0)
    g = bounded_bulb() if graph == "bounded" else workloads.mandelbulb_primary_graph()
    scene = Scene(graph=g, camera=Camera.look_at((1.0, 0.8, -3.2), (0.6, 0.0, 0.0), 55.0),
                  material=mat, lights=[light], seed=99)
    a = render(renderer, scene, small_cfg("wavefront"))
    b = render(renderer, scene, small_cfg("megakernel"))
    # the two integrators run the same arithmetic (fixed fusion), so the films are equal
    np.testing.assert_array_equal(a.accum, b.accum)
    np.testing.assert_array_equal(a.depth, b.depth)
    cfg = small_cfg("wavefront")
    assert (a.depth >= 0).mean() > 0.2
    rng = np.random.default_rng(3)
    pix = np.stack([rng.integers(0, cfg.width, 96), rng.integers(0, cfg.height, 96)], 1).astype(np.uint32)
    ref = oracle_mod.OracleGraph(scene.graph).render(scene.desc(cfg.width, cfg.height), cfg.desc(), pix, 0,
                                                     cfg.samples_per_pixel, precision=32)
    mine = a.accum[pix[:, 1], pix[:, 0], :3] / cfg.samples_per_pixel
    rmse = float(np.sqrt(np.mean((mine - ref["accum"] / cfg.samples_per_pixel) ** 2)))
    assert rmse <= 2e-2, rmse
    hit = ref["depth"] >= 0
    np.testing.assert_array_equal(a.depth[pix[:, 1], pix[:, 0]] >= 0, hit)
    np.testing.assert_allclose(a.depth[pix[:, 1], pix[:, 0]][hit], ref["depth"][hit], rtol=1e-3)

"""HDRI panoramas (EnvironmentMap, crates/syfrack-render/src/environment.rs:237-437;
environment.wgsl). The table builder is checked, in the library and in the oracle,
against the reference's own tests (environment.rs:398-437): the distribution
integrates to one and keeps dark cells in support, a black map samples uniformly,
non-finite or empty maps are refused, and downsampling keeps a tiny source's energy.
On the GPU, a panorama-lit scene renders the same through both integrators and
follows the f32 oracle."""
import math

import numpy as np
import pytest

from syfrack_gb300 import SyfrackError
from syfrack_gb300.scene import panorama_tables

UNIFORM_MIX = 0.0625


def cell_area(w, h, row):
    top, bottom = math.pi * row / h, math.pi * (row + 1) / h
    return 2.0 * math.pi / w * 2.0 * math.sin((top + bottom) * 0.5) * math.sin((bottom - top) * 0.5)


def cell_pdf(texels, uniform, i):
    h, w = texels.shape[:2]
    if uniform:
        return 1.0 / (4.0 * math.pi)
    cdf = texels[..., 3].reshape(-1).astype(np.float64)
    mass = cdf[i] - (cdf[i - 1] if i else 0.0)
    return (1.0 - UNIFORM_MIX) * mass / cell_area(w, h, i // w) + UNIFORM_MIX / (4.0 * math.pi)


def builders(oracle_mod):
    yield "library", lambda rgb: panorama_tables(rgb)

    def orc(rgb):
        t = oracle_mod.panorama(rgb)
        return t, bool(np.all(t[..., :3] == t[0, 0, :3]))

    yield "oracle", orc


def test_distribution_integrates_to_one(oracle_mod):
    rgb = np.zeros((8, 16, 3), np.float32)
    rgb.reshape(-1, 3)[22] = 1e8
    for name, build in builders(oracle_mod):
        t, uni = build(rgb)
        pdf = [cell_pdf(t, uni, i) for i in range(128)]
        integral = sum(p * cell_area(16, 8, i // 16) for i, p in enumerate(pdf))
        assert abs(integral - 1.0) < 1e-10, name
        assert all(math.isfinite(p) and p > 0.0 for p in pdf), name
        assert pdf[22] > pdf[23] * 4.0, name


def test_black_map_is_uniform_and_bad_maps_are_refused(oracle_mod):
    t, uni = panorama_tables(np.zeros((16, 32, 3), np.float32))
    assert uni
    assert all(abs(cell_pdf(t, uni, i) - 1.0 / (4.0 * math.pi)) < 1e-5 for i in range(512))
    for bad in (np.array([[[np.nan, 0, 0]]], np.float32), np.array([[[np.inf, 0, 0]]], np.float32),
                np.zeros((1, 0, 3), np.float32)):
        with pytest.raises(SyfrackError):
            panorama_tables(bad)
        with pytest.raises(ValueError):
            oracle_mod.panorama(bad)


def test_downsampling_keeps_a_tiny_sources_energy(oracle_mod):
    w, h = 4097, 1
    rgb = np.zeros((h, w, 3), np.float32)
    rgb[0, 2048] = 1000.0
    for name, build in builders(oracle_mod):
        t, _ = build(rgb)
        assert t.shape[:2] == (1, 2048), name
        actual = float((t[0, :, 0].astype(np.float64) * cell_area(2048, 1, 0)).sum())
        expected = 1000.0 * cell_area(w, h, 0)
        assert abs(actual - expected) < expected * 1e-6, name


def test_library_and_oracle_tables_agree(oracle_mod):
    rng = np.random.default_rng(1)
    rgb = (rng.random((96, 192, 3)) ** 6 * 20).astype(np.float32)
    a, _ = panorama_tables(rgb)
    np.testing.assert_array_equal(a, oracle_mod.panorama(rgb))


def sky_panorama(w=256, h=128):
    """A synthetic sky: blue gradient, warm horizon, dark ground and a bright sun spot."""
    y = ((np.arange(h) + 0.5) / h)[:, None, None]
    sky = (0.2 + 0.6 * np.clip(1.0 - 2.0 * y, 0, 1)) * np.array([0.35, 0.55, 1.0])
    rgb = np.broadcast_to(np.where(y < 0.5, sky, np.array([0.12, 0.1, 0.08])), (h, w, 3)).astype(np.float32).copy()
    cy, cx = int(0.22 * h), int(0.3 * w)
    rgb[cy - 2:cy + 2, cx - 2:cx + 2] = 2000.0
    return rgb


@pytest.mark.gpu
def test_panorama_lit_film(renderer, oracle_mod, gpu_ctx, tmp_path):
    from syfrack_gb300 import RenderSession, workloads
    from syfrack_gb300.scene import HdriLight, Material, Panorama, RenderConfig, Scene

    rgb = sky_panorama()
    pano = Panorama(gpu_ctx, rgb)
    oracle_mod.panorama(rgb, key=pano.h.value)
    _, cam, *_ = workloads.mandelbulb_primary()
    scene = Scene(graph=workloads.mandelbulb_primary_graph(), camera=cam,
                  material=Material(albedo=(0.8, 0.7, 0.6), roughness=0.3),
                  lights=[HdriLight(pano, intensity=1.5, rotation=30.0)], seed=3)
    films = []
    for integ in ("wavefront", "megakernel"):
        cfg = RenderConfig(96, 64, 8, max_bounces=3, max_steps=256, pixel_tolerance=1.0, tile_size=64,
                           samples_per_dispatch=4, integrator=integ)
        s = RenderSession(renderer, scene, cfg)
        while not s.step(0):
            pass
        films.append(s.readback())
        if integ == "wavefront":
            with pytest.raises(SyfrackError, match="SF_ERR_UNSUPPORTED"):
                s.save(str(tmp_path / "ck"))
        s.close()
    np.testing.assert_allclose(films[0].accum, films[1].accum, rtol=1e-6, atol=1e-6)
    rng = np.random.default_rng(8)
    pix = np.stack([rng.integers(0, 96, 128), rng.integers(0, 64, 128)], 1).astype(np.uint32)
    ref = oracle_mod.OracleGraph(scene.graph).render(scene.desc(96, 64), cfg.desc(), pix, 0, 8, precision=32)
    mine = films[0].accum[pix[:, 1], pix[:, 0], :3] / 8
    rmse = float(np.sqrt(np.mean((mine - ref["accum"] / 8) ** 2)))
    assert rmse <= 2e-2, rmse
    assert mine.mean() > 0.05  # the panorama lights the form and the background
    pano.close()

"""Escape-time sampling on the GPU against the oracle (GPU).

Iteration counts are bit-exact against the reference's binary32 arithmetic
(the f32 oracle): the device evaluates the orbit with unfused, explicitly
rounded operations. Traps follow gpu_planar.rs:101-130 (within 0.006; Newton
and Nova smooth time within 0.09)."""
import numpy as np
import pytest

from syfrack_gb300 import Canvas, PlanarFractal, escape2d
from syfrack_gb300.render import FAMILIES

pytestmark = pytest.mark.gpu


def oracle_params(oracle_mod, f: PlanarFractal):
    p = oracle_mod.PlanarParams()
    p.family = FAMILIES.index(f.family)
    p.power, p.iterations = f.power, f.iterations
    p.julia[:] = [float(np.float32(x)) for x in f.julia]
    p.center[:] = [float(np.float32(x)) for x in f.center]
    for k in ("zoom", "angle", "inversion", "twist", "relaxation", "memory", "bailout", "trap_radius", "stripes"):
        setattr(p, k, float(np.float32(getattr(f, k))))
    return p


def grid289():
    xs = np.linspace(-1.6, 1.6, 17, dtype=np.float32)
    return np.array([[x, y] for y in xs for x in xs], np.float32)


@pytest.mark.parametrize("family", FAMILIES)
def test_planar_iterations_bit_exact(gpu_ctx, oracle_mod, family):
    rng = np.random.default_rng(5)
    pts = np.concatenate([grid289(), rng.uniform(-2, 2, (4000, 2)).astype(np.float32)])
    for power in (2, 3):
        f = PlanarFractal(family=family, power=power, iterations=256)
        gpu = f.sample(gpu_ctx, pts)
        ref = oracle_mod.planar(oracle_params(oracle_mod, f), pts, precision=32)
        np.testing.assert_array_equal(gpu["iterations"], ref["iterations"])
        d = np.abs(gpu["traps"] - ref["traps"])
        assert np.quantile(d[:, 1:], 0.999) <= 0.006
        tol = 0.09 if family in ("Newton", "Nova") else 0.006
        assert np.quantile(d[:, 0], 0.999) <= tol
        np.testing.assert_allclose(gpu["distance"], ref["distance"], atol=1e-5)


def test_planar_mapping_bit_exact(gpu_ctx, oracle_mod):
    f = PlanarFractal(family="Julia", iterations=300, zoom=1.7, angle=30.0, inversion=0.8, twist=12.0,
                      center=(0.1, -0.2))
    pts = np.random.default_rng(2).uniform(-1.5, 1.5, (8192, 2)).astype(np.float32)
    np.testing.assert_array_equal(f.sample(gpu_ctx, pts)["iterations"],
                                  oracle_mod.planar(oracle_params(oracle_mod, f), pts, precision=32)["iterations"])


def canvas_points(c: Canvas, sample=None):
    """The flat-canvas map (pathtrace.wgsl:1226-1239) in unfused binary32."""
    f = np.float32
    ys, xs = np.mgrid[0:c.height, 0:c.width]
    jx = np.full(xs.shape, f(0.5), np.float32)
    jy = jx.copy()
    u = (xs.astype(np.float32) + jx) / f(c.width)
    v = (ys.astype(np.float32) + jy) / f(c.height)
    scale = f(6.0) / f(c.zoom)
    aspect = f(c.width) / f(c.height)
    ax = (u - f(0.5)) * scale
    ay = ((f(0.5) - v) / aspect) * scale
    r = f(c.rotation) * f(np.pi / 180.0)
    cs, sn = f(np.cos(r)), f(np.sin(r))
    qx = f(c.center[0]) + (cs * ax - sn * ay)
    qy = f(c.center[1]) + (sn * ax + cs * ay)
    return np.stack([qx.ravel(), qy.ravel()], 1).astype(np.float32)


def test_escape2d_canvas_against_oracle(gpu_ctx, oracle_mod):
    c = Canvas(width=160, height=90, center=(-0.5, 0.0), zoom=2.0)
    f = PlanarFractal(family="Mandelbrot", iterations=2000)
    out = escape2d(gpu_ctx, f, c)
    ref = oracle_mod.planar(oracle_params(oracle_mod, f), canvas_points(c), precision=32)
    np.testing.assert_array_equal(out["iterations"].ravel(), ref["iterations"])


def test_beyond_reference_caps(gpu_ctx, oracle_mod):
    # 20,000 iterations and zoom 1e5 (the reference caps 512 and 1e4), seahorse valley
    f = PlanarFractal(family="Mandelbrot", iterations=20000, zoom=1e5, center=(-0.7436, 0.1318))
    pts = np.random.default_rng(8).uniform(-1, 1, (2048, 2)).astype(np.float32)
    gpu = f.sample(gpu_ctx, pts)
    ref = oracle_mod.planar(oracle_params(oracle_mod, f), pts, precision=32)
    np.testing.assert_array_equal(gpu["iterations"], ref["iterations"])
    assert gpu["iterations"].max() > 512


def test_tiles_and_jitter(gpu_ctx):
    c = Canvas(width=64, height=48, seed=3)
    f = PlanarFractal(family="Julia", iterations=200)
    full = escape2d(gpu_ctx, f, c, sample=5)
    part = escape2d(gpu_ctx, f, c, tile=(16, 8, 32, 20), sample=5)
    np.testing.assert_array_equal(part["iterations"], full["iterations"][8:28, 16:48])
    other = escape2d(gpu_ctx, f, c, sample=6)
    assert (other["iterations"] != full["iterations"]).any()


@pytest.mark.parametrize("stripes", [12.0, -5.0, 7.5, 0.0])
def test_stripe_bands_integer_and_general(gpu_ctx, oracle_mod, stripes):
    # integer stripe counts use sin(k theta) = Im(u^k); others use sin(k * atan2)
    f = PlanarFractal(family="Mandelbrot", iterations=400, stripes=stripes)
    pts = np.random.default_rng(12).uniform(-2.0, 1.0, (6000, 2)).astype(np.float32)
    gpu = f.sample(gpu_ctx, pts)
    ref = oracle_mod.planar(oracle_params(oracle_mod, f), pts, precision=32)
    np.testing.assert_array_equal(gpu["iterations"], ref["iterations"])
    d = np.abs(gpu["traps"] - ref["traps"])
    assert np.quantile(d, 0.999) <= 0.006


def test_escape2d_without_traps_keeps_counts(gpu_ctx):
    from syfrack_gb300 import Renderer, Server

    c = Canvas(width=200, height=120, center=(-0.45, -0.5), zoom=2.0)
    f = PlanarFractal(family="BurningShip", iterations=3000)
    full = escape2d(gpu_ctx, f, c)
    srv = Server(Renderer(gpu_ctx), hbm_budget=1 << 28)
    lean = srv.wait(srv.tile(f, c, traps=False))
    srv.close()
    assert lean.traps is None and lean.distance is None
    np.testing.assert_array_equal(lean.iterations, full["iterations"])
    np.testing.assert_array_equal(lean.smooth, full["traps"][0])

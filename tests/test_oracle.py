"""The oracle pinned to the reference's golden vectors and unit-test known
answers (CPU). Tolerances are the reference's own:
graph_parity.rs:34-65 (distance 1e-5 relative / absolute below 1, traps 1e-5,
iterations equal), eval.rs:180-222, fractal.rs:87-204, planar.rs:276-345."""
import math

import numpy as np
import pytest

from helpers import FORMS, golden, lcg_points
from syfrack_gb300.graph import Graph, Kind, Link, Node


@pytest.mark.parametrize("name", FORMS)
def test_f32_oracle_matches_golden_fixture(oracle_mod, name):
    extent, pts, dist, traps, iters = golden(name)
    np.testing.assert_array_equal(pts, lcg_points(64, extent, 11))  # the fixture points are the LCG points
    og = oracle_mod.OracleGraph(Graph.bundled(name))
    r = og.de(pts, precision=32)
    err = np.abs(r["distance"] - dist) / np.maximum(np.abs(dist), 1.0)
    assert err.max() <= 1e-5
    assert np.abs(r["traps"] - traps).max() <= 1e-5
    np.testing.assert_array_equal(r["iterations"], iters)


@pytest.mark.parametrize("name", FORMS)
def test_f64_oracle_close_to_golden_fixture(oracle_mod, name):
    extent, pts, dist, traps, iters = golden(name)
    og = oracle_mod.OracleGraph(Graph.bundled(name))
    r = og.de(pts, precision=64)
    err = np.abs(r["distance"] - dist) / np.maximum(np.abs(dist), 1.0)
    assert err.max() <= 1e-5
    np.testing.assert_array_equal(r["iterations"], iters)


def test_step_scales_and_trap_scales(oracle_mod):
    # graph_parity.rs:84-88: step scales 0.6 and 0.9
    assert oracle_mod.OracleGraph(Graph.bundled("mandelbox")).info()["step_scale"] == pytest.approx(0.6, abs=1e-6)
    assert oracle_mod.OracleGraph(Graph.bundled("menger")).info()["step_scale"] == pytest.approx(0.9, abs=1e-6)
    i = oracle_mod.OracleGraph(Graph.bundled("mandelbulb")).info()
    assert i["trap_scales"] == [4.0, 1.0, 1.0, 1.0] and i["iteration_product"] == 12


def test_twist_lowers_step_scale(oracle_mod):
    # graph_parity.rs:90-117
    nodes = [Node(0, Kind("Input")), Node(1, Kind("Sphere", radius=1.0)), Node(2, Kind("Output")),
             Node(3, Kind("Twist", rate=1.0))]
    links = [Link((0, 0), (3, 0)), Link((3, 0), (1, 0)), Link((1, 0), (2, 0))]
    g = Graph(nodes, links, safety=1.0, bounding_radius_hint=2.0)
    assert oracle_mod.OracleGraph(g).info()["step_scale"] == pytest.approx(1.0 / math.sqrt(5.0), abs=1e-6)


def _power_graph(n):
    nodes = [Node(0, Kind("Input")), Node(1, Kind("Power", power=float(n))),
             Node(2, Kind("Sphere", radius=0.0)), Node(3, Kind("Output"))]
    return Graph(nodes, [Link((0, 0), (1, 0)), Link((1, 0), (2, 0)), Link((2, 0), (3, 0))])


def test_integer_spherical_powers_match_trig(oracle_mod):
    # eval.rs:180-222 on the restated f32 path: powers 1..16 against f64 trigonometry.
    rng = np.random.default_rng(12341)
    pts = np.concatenate([np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, -1]], np.float32),
                          rng.uniform(-1.5, 1.5, (300, 3)).astype(np.float32)])
    for n in range(1, 17):
        og = oracle_mod.OracleGraph(_power_graph(n))
        q = pts.astype(np.float64)
        r = np.linalg.norm(q, axis=1)
        theta = np.arccos(np.clip(q[:, 2] / r, -1, 1)) * n
        phi = np.arctan2(q[:, 1], q[:, 0]) * n
        # Sphere(0) fence of the powered point: |p_n| / dr = r^n / (n r^(n-1)) = r / n
        d = og.de(pts, precision=32)["distance"]
        expected = r ** n / (n * r ** (n - 1))
        assert np.all(np.abs(d - expected) <= 5e-6 * np.maximum(expected, 1e-20) + 1e-6), n
        assert np.all(np.isfinite(theta)) and np.all(np.isfinite(phi))


def power_component_graph(n, axis):
    """Input -> Power(n) -> Plane(normal = axis, offset 0): the distance is the powered
    point's component on the axis over the power's derivative, p_n[axis] / (n r^(n-1))."""
    normal = [0.0, 0.0, 0.0]
    normal[axis] = 1.0
    nodes = [Node(0, Kind("Input")), Node(1, Kind("Power", power=float(n))),
             Node(2, Kind("Plane", normal=normal, offset=0.0)), Node(3, Kind("Output"))]
    return Graph(nodes, [Link((0, 0), (1, 0)), Link((1, 0), (2, 0)), Link((2, 0), (3, 0))])


def spherical_power_points():
    """The points of eval.rs:180-222: the axes, two near-pole filaments, and 1,000 LCG
    points in [-1.5, 1.5]^3 (seed 12341)."""
    special = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, -1], [1e-6, 0, 1], [-1e-6, 2e-6, -1]], np.float32)
    return np.concatenate([special, lcg_points(1000, 1.5, 12341)])


def spherical_power_expected(pts, n):
    """FP64 trigonometry (eval.rs:200-210): the powered point and its derivative."""
    q = pts.astype(np.float64)
    r = np.linalg.norm(q, axis=1)
    theta = np.arccos(np.clip(q[:, 2] / r, -1, 1)) * n
    phi = np.arctan2(q[:, 1], q[:, 0]) * n
    e = np.stack([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)], 1) * (r ** n)[:, None]
    return e, n * r ** (n - 1), r


def spherical_power_error(dist_by_axis, pts, n):
    """Each component's error against FP64 trigonometry, in units of the reference's
    bounds: the point within 5e-6 r^n and the derivative within 4e-6 of itself
    (eval.rs:212-217), both carried by p_n[axis] / dr."""
    e, dr, r = spherical_power_expected(pts, n)
    worst = 0.0
    for axis in range(3):
        got = dist_by_axis[axis] * dr  # the component, through the expected derivative
        bound = 5e-6 * np.maximum(r ** n, 1e-20) + 4e-6 * np.abs(e[:, axis])
        worst = max(worst, float((np.abs(got - e[:, axis]) / bound).max()))
    return worst


def test_spherical_power_vectors_match_trig(oracle_mod):
    # eval.rs:180-222 componentwise: the powered point of n = 1..16 against FP64
    # trigonometry on the reference's own points, and the filament (1e-6, 0, 1)^8,
    # whose rounded cosine is exactly 1: x = 8e-6 within 1e-10
    pts = spherical_power_points()
    for n in range(1, 17):
        d = [oracle_mod.OracleGraph(power_component_graph(n, a)).de(pts, precision=32)["distance"] for a in range(3)]
        assert spherical_power_error(d, pts, n) <= 1.0, n
    x = oracle_mod.OracleGraph(power_component_graph(8, 0)).de(np.array([[1e-6, 0.0, 1.0]], np.float32),
                                                               precision=32)["distance"][0]
    assert abs(x * 8.0 - 8e-6) < 1e-10


def test_bulb_symmetry_and_inside_outside(oracle_mod):
    # fractal.rs:103-178: inside/far points, 2pi/7 symmetry about z, not pi/4
    og = oracle_mod.OracleGraph(Graph.bundled("mandelbulb"))
    assert og.de(np.array([[0.0, 0.0, 0.0]]))["distance"][0] < 0
    assert og.de(np.array([[0.0, 0.0, 20.0]]))["distance"][0] > 2.0
    pts = lcg_points(200, 1.2, 5).astype(np.float64)

    def rot(a):
        c, s = math.cos(a), math.sin(a)
        return np.stack([c * pts[:, 0] - s * pts[:, 1], s * pts[:, 0] + c * pts[:, 1], pts[:, 2]], 1)

    d0 = og.de(pts)["distance"]
    assert np.abs(og.de(rot(2 * math.pi / 7))["distance"] - d0).max() < 1e-4
    assert np.abs(og.de(rot(math.pi / 4))["distance"] - d0).max() > 1e-3
    og = oracle_mod.OracleGraph(Graph.bundled("menger"))
    assert og.de(np.array([[0.5, 0.5, 0.5]]))["distance"][0] < 0


def test_lipschitz_bound(oracle_mod):
    # fractal.rs: |d(a) - d(b)| <= 1.05 |a - b| on 2000 pairs, at most 20 violations
    for name in ("mandelbulb", "mandelbox", "menger"):
        og = oracle_mod.OracleGraph(Graph.bundled(name))
        a = lcg_points(2000, 1.5, 3).astype(np.float64)
        b = a + lcg_points(2000, 0.01, 4).astype(np.float64)
        da, db = og.de(a)["distance"], og.de(b)["distance"]
        ratio = np.abs(da - db) / np.linalg.norm(a - b, axis=1)
        assert (ratio > 1.05).sum() <= 20, name


def _planar(oracle_mod, **kw):
    p = oracle_mod.PlanarParams()
    base = dict(family=0, power=2, iterations=128, julia=(-0.74543, 0.11301), center=(0.0, 0.0), zoom=1.0,
                angle=0.0, inversion=0.0, twist=0.0, relaxation=1.0, memory=-0.5, bailout=16.0,
                trap_radius=0.5, stripes=12.0)
    base.update(kw)
    for k, v in base.items():
        if isinstance(v, tuple):
            getattr(p, k)[:] = list(v)
        else:
            setattr(p, k, v)
    return p


def test_planar_known_answers(oracle_mod):
    # planar.rs:300-345
    mb = _planar(oracle_mod, family=1)
    r = oracle_mod.planar(mb, np.array([[0.0, 0.0], [2.0, 1.0]]), precision=32)
    assert r["iterations"][0] == 128 and r["iterations"][1] < 5
    nw = _planar(oracle_mod, family=3, power=3)
    assert oracle_mod.planar(nw, np.array([[1.0, 0.0]]), precision=32)["iterations"][0] == 0
    grid = np.array([[(i % 10) * 0.37 - 1.6, (i // 10) * 0.31 - 1.5] for i in range(100)], np.float32)
    for fam in range(6):
        p = _planar(oracle_mod, family=fam)
        r = oracle_mod.planar(p, grid, precision=32)
        assert np.all(np.isfinite(r["distance"]))
        assert np.all((r["traps"] >= 0) & (r["traps"] <= 1)), fam


def test_planar_stripe_continuity(oracle_mod):
    # planar.rs:276-298
    p = _planar(oracle_mod, julia=(0.0, 0.0))
    a = math.pi / 32
    d = np.array([math.cos(a), math.sin(a)], np.float32)
    pts = np.stack([d * np.float32(4.0 - 1e-5), d * np.float32(4.0 + 1e-5)])
    r = oracle_mod.planar(p, pts, precision=32)
    assert r["iterations"][0] != r["iterations"][1]
    assert abs(r["traps"][0, 2] - r["traps"][1, 2]) < 1e-4
    assert abs(r["traps"][0, 0] - r["traps"][1, 0]) < 1e-5


def test_generic_graph_semantics(oracle_mod):
    # disabled fence = +inf, empty union side does not poison (eval.rs:226-228, :601-657)
    nodes = [Node(0, Kind("Input")), Node(1, Kind("Sphere", radius=1.0)),
             Node(2, Kind("Sphere", radius=2.0), enabled=False), Node(3, Kind("SmoothUnion", k=0.3)),
             Node(4, Kind("Output"))]
    links = [Link((0, 0), (1, 0)), Link((0, 0), (2, 0)), Link((1, 0), (3, 0)), Link((2, 0), (3, 1)),
             Link((3, 0), (4, 0))]
    og = oracle_mod.OracleGraph(Graph(nodes, links))
    r = og.de(np.array([[3.0, 0.0, 0.0]]))
    assert r["distance"][0] == pytest.approx(2.0)


def test_bounded_fast_and_exact_samples(oracle_mod):
    """graph_wgsl.rs:800-814 and :976-1006: outside bound + margin the GPU's march
    sample is the box bound with flags 1 (never above the exact distance); inside it,
    or through a Subtraction's second input, the sample is the exact one."""
    from helpers import bounded_bulb

    pts = lcg_points(4096, 3.0, 5)
    for subtract in (False, True):
        og = oracle_mod.OracleGraph(bounded_bulb(subtract))
        for prec in (32, 64):
            exact = og.de(pts, precision=prec)
            fast = og.de_fast(pts, precision=prec)
            flagged = fast["flags"] != 0
            np.testing.assert_array_equal(fast["distance"][~flagged], exact["distance"][~flagged])
            assert np.all(fast["distance"][flagged] <= exact["distance"][flagged] + 1e-6)
            if subtract:
                assert not flagged.any()
            else:
                assert 0.5 < flagged.mean() < 0.99
                box = np.abs(pts).max(1)
                assert np.all(box[flagged] > 1.25)  # only outside the box can a bound be skipped
    # a wider margin evaluates the detail further out
    a = oracle_mod.OracleGraph(bounded_bulb(margin=0.05)).de_fast(pts, precision=32)["flags"].mean()
    b = oracle_mod.OracleGraph(bounded_bulb(margin=1.0)).de_fast(pts, precision=32)["flags"].mean()
    assert b < a

"""Instances: independently transformed copies of a template distance branch.

Known answers restated from crates/syfrack-core/tests/architecture.rs:4-160 (the
hierarchy search equals a brute-force union of 4,097 copies within 1e-5; two torus
copies equal the transformed union within 2e-5 and keep their MaterialTag; a
disabled node passes its template through; nesting deeper than three levels and
zero scales are invalid) and bvh.rs:104-137 (every leaf's fence corners lie inside
the leaf and all its ancestors). The GPU tests compare the device with the oracle
under the gpu_de.rs rule and through the primary-ray march."""
import math

import numpy as np
import pytest

from helpers import lcg_points
from syfrack_gb300 import SyfrackError
from syfrack_gb300.graph import Graph, Kind, Link, Node


def minimal(template=None):
    """Graph::new_minimal (graph/mod.rs:454-482): Input -> Sphere(1) -> Output."""
    t = template or Kind("Sphere", radius=1.0)
    return Graph([Node(0, Kind("Input")), Node(1, t), Node(2, Kind("Output"))],
                 [Link((0, 0), (1, 0)), Link((1, 0), (2, 0))], safety=1.0, bounding_radius_hint=2.0)


def add(g, kind, inputs, enabled=True):
    nid = max(n.id for n in g.nodes) + 1
    g.nodes.append(Node(nid, kind, enabled=enabled))
    for port, src in enumerate(inputs):
        g.links.append(Link((src, 0), (nid, port)))
    return nid


def to_output(g, nid):
    g.links = [l for l in g.links if l.dst != (2, 0)] + [Link((nid, 0), (2, 0))]
    return g


def rot_matrix(angles_deg):
    """glam Quat::from_euler(EulerRot::XYZ) as a matrix: Rx @ Ry @ Rz."""
    a, b, c = (math.radians(x) for x in angles_deg)
    rx = np.array([[1, 0, 0], [0, math.cos(a), -math.sin(a)], [0, math.sin(a), math.cos(a)]])
    ry = np.array([[math.cos(b), 0, math.sin(b)], [0, 1, 0], [-math.sin(b), 0, math.cos(b)]])
    rz = np.array([[math.cos(c), -math.sin(c), 0], [math.sin(c), math.cos(c), 0], [0, 0, 1]])
    return rx @ ry @ rz


def local_points(p, pl):
    # the placements cross the C ABI as binary32
    pos, ang, sc = (np.array(x, np.float32).astype(np.float64) for x in pl)
    return ((p - pos) @ rot_matrix(ang)) / sc, sc  # R^T (p - pos) / scale, row-vector form


def box_fence(q, half, sc):
    v = (np.abs(q) - float(np.float32(half))) * sc
    return np.linalg.norm(np.maximum(v, 0.0), axis=1) + np.minimum(v.max(1), 0.0)


def big_hierarchy():
    placements = [(((i % 47) * 1.3 - 30.0, ((i // 47) % 47) * 1.1 - 20.0, (i // 2209) * 1.5),
                   ((i % 359) - 179.0, 19.0, -13.0), (0.4, 1.1, 0.7)) for i in range(4097)]
    g = minimal()
    c = add(g, Kind("Instances", placements=placements, half=[0.8, 0.8, 0.8], margin=0.1), [1])
    return to_output(g, c), placements


def big_points():
    return np.array([((i % 17) * 3.8 - 32.0, (i // 17) * 5.2 - 20.0, (i % 7) * 0.4 - 0.9) for i in range(107)])


def brute_force_spheres(points, placements, half=0.8):
    best = np.full(len(points), np.inf)
    for pl in placements:
        q, sc = local_points(points, pl)
        d = np.maximum((np.linalg.norm(q, axis=1) - 1.0) * sc.min(), box_fence(q, half, sc))
        best = np.minimum(best, d)
    return best


def torus_copies(enabled=True):
    placements = [((-1.3, 0.2, 0.3), (28.0, 45.0, -17.0), (1.4, 0.7, 1.1)),
                  ((0.4, -0.2, -0.5), (-42.0, 13.0, 60.0), (0.8, 1.2, 1.5))]
    g = minimal(Kind("Torus", radius=1.0, tube=0.2))
    tag = add(g, Kind("MaterialTag", index=1), [1])
    c = add(g, Kind("Instances", placements=placements, half=[1.5, 1.5, 1.5], margin=0.1), [tag], enabled=enabled)
    return to_output(g, c), placements


def grid_points():
    return np.array([((i % 9) * 0.7 - 2.8, ((i // 9) % 9) * 0.7 - 2.8, (i // 81) * 0.7 - 2.8) for i in range(729)])


def brute_force_torus(points, placements):
    best = np.full(len(points), np.inf)
    for pl in placements:
        q, sc = local_points(points, pl)
        d = np.hypot(np.hypot(q[:, 0], q[:, 2]) - 1.0, q[:, 1]) - 0.2
        best = np.minimum(best, np.maximum(d * sc.min(), box_fence(q, 1.5, sc)))
    return best


def nested_copies():
    """Three nested Instances levels over a unit sphere: the innermost holds two
    rotated, scaled copies; the middle one three; the outer two (12 spheres)."""
    levels = [
        [((0.9, 0.0, 0.1), (10.0, 0.0, 25.0), (0.5, 0.6, 0.55)), ((-0.8, 0.3, 0.0), (0.0, 35.0, 0.0), (0.45, 0.5, 0.5))],
        [((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), ((0.2, 1.8, 0.0), (0.0, 0.0, 90.0), (0.8, 0.8, 0.9)),
         ((-0.3, -1.7, 0.4), (20.0, 0.0, -30.0), (0.9, 1.0, 0.8))],
        [((-1.6, 0.0, 0.0), (0.0, 15.0, 0.0), (1.0, 0.9, 1.0)), ((1.7, 0.2, 0.5), (-25.0, 0.0, 10.0), (0.85, 0.85, 0.85))],
    ]
    halves = [1.6, 3.2, 4.5]
    g = minimal()
    last = 1
    for placements, half in zip(levels, halves):
        last = add(g, Kind("Instances", placements=placements, half=[half] * 3, margin=0.1), [last])
    return to_output(g, last), list(zip(levels, halves))


def brute_force_nested(points, levels):
    """eval.rs:749-814 unrolled: each level's copy is max(template(q) * min scale,
    its Box fence), the nearest copy wins; the innermost template is the unit sphere."""
    def level(p, k):
        if k < 0:
            return np.linalg.norm(p, axis=1) - 1.0
        placements, half = levels[k]
        best = np.full(len(p), np.inf)
        for pl in placements:
            q, sc = local_points(p, pl)
            best = np.minimum(best, np.maximum(level(q, k - 1) * sc.min(), box_fence(q, half, sc)))
        return best
    return level(np.asarray(points, np.float64), len(levels) - 1)


# ---------------------------------------------------------------- CPU: oracle and host

def test_nested_copies_match_the_composed_union(oracle_mod):
    """Copies of copies of copies (eval.rs:808 recurses into each copy's template, up
    to three levels) equal the brute-force composition of the levels."""
    g, levels = nested_copies()
    pts = grid_points() * 1.6
    og = oracle_mod.OracleGraph(g)
    np.testing.assert_allclose(og.de(pts, precision=64)["distance"], brute_force_nested(pts, levels), atol=1e-9,
                               rtol=0)
    np.testing.assert_allclose(og.de(pts, precision=32)["distance"], brute_force_nested(pts, levels), atol=2e-5,
                               rtol=0)


def test_hierarchy_matches_brute_force_union(oracle_mod):
    g, placements = big_hierarchy()
    pts = big_points()
    expected = brute_force_spheres(pts, placements)
    og = oracle_mod.OracleGraph(g)
    np.testing.assert_allclose(og.de(pts, precision=32)["distance"], expected, atol=1e-5, rtol=0)
    np.testing.assert_allclose(og.de(pts, precision=64)["distance"], expected, atol=1e-9, rtol=0)


def test_torus_copies_match_transformed_union(oracle_mod):
    g, placements = torus_copies()
    pts = grid_points()
    r = oracle_mod.OracleGraph(g).de(pts, precision=32)
    np.testing.assert_allclose(r["distance"], brute_force_torus(pts, placements), atol=2e-5, rtol=0)
    assert np.all(r["material"] == 1)
    off, _ = torus_copies(enabled=False)
    d = oracle_mod.OracleGraph(off).de(np.array([[1.0, 0.0, 0.0]]), precision=32)["distance"][0]
    assert abs(d + 0.2) < 1e-6  # a disabled node passes its template through


def test_fast_copies_flag_empty_space(oracle_mod):
    """graph_wgsl.rs:769-790: beyond the root fence + margin the march sample is the
    root fence (flagged); a copy whose fence is beyond the margin is not evaluated."""
    g, _ = torus_copies()
    pts = lcg_points(4096, 6.0, 21).astype(np.float64)
    og = oracle_mod.OracleGraph(g)
    exact, fast = og.de(pts, precision=64), og.de_fast(pts, precision=64)
    flagged = fast["flags"] != 0
    assert 0.3 < flagged.mean() < 0.99
    np.testing.assert_array_equal(fast["distance"][~flagged], exact["distance"][~flagged])
    assert np.all(fast["distance"][flagged] <= exact["distance"][flagged] + 1e-9)


def test_validation():
    g, _ = torus_copies()
    assert g.validate()["form"] == "generic"
    # more than three nested levels (architecture.rs:132-160)
    g = minimal()
    last = 1
    for _ in range(4):
        last = add(g, Kind("Instances", placements=[((0, 0, 0), (0, 0, 0), (1, 1, 1))], half=[2.0] * 3,
                           margin=0.1), [last])
    to_output(g, last)
    with pytest.raises(SyfrackError) as e:
        g.validate()
    assert e.value.status == 2  # SF_ERR_GRAPH
    g.node(last).enabled = False
    assert g.validate()["form"] == "generic"  # three levels are valid, and the device runs them
    for bad in ([((0, 0, 0), (0, 0, 0), (0.0, 1, 1))], [], [((2000.0, 0, 0), (0, 0, 0), (1, 1, 1))],
                [((0, 0, 0), (200.0, 0, 0), (1, 1, 1))]):
        g = minimal()
        to_output(g, add(g, Kind("Instances", placements=bad, half=[1.0] * 3, margin=0.1), [1]))
        with pytest.raises(SyfrackError):
            g.validate()


# ---------------------------------------------------------------- GPU: the device interpreter

@pytest.mark.gpu
def test_device_copies_against_brute_force_and_oracle(renderer, oracle_mod):
    from test_gpu_de import gpu_de_rule

    g, placements = torus_copies()
    pts = grid_points()
    r = renderer.compile(g).probe(pts)
    np.testing.assert_allclose(r["distance"], brute_force_torus(pts, placements), atol=1e-4, rtol=0)
    assert np.all(r["material"] == 1)
    lcg = lcg_points(4096, 3.5, 13)
    assert gpu_de_rule(renderer.compile(g).probe(lcg), oracle_mod.OracleGraph(g).de(lcg, precision=32)) <= 0.005
    big, placements = big_hierarchy()
    pts = big_points()
    r = renderer.compile(big).probe(pts)
    np.testing.assert_allclose(r["distance"], brute_force_spheres(pts, placements), atol=1e-4, rtol=0)
    off, _ = torus_copies(enabled=False)
    assert abs(renderer.compile(off).probe(np.array([[1.0, 0.0, 0.0]]))["distance"][0] + 0.2) < 1e-5


@pytest.mark.gpu
def test_device_copies_march_and_film(renderer, oracle_mod):
    """The march samples copies with the GPU's skips (root fence, far copies) and the
    exact re-evaluation near acceptance; the device follows the f32 oracle's march,
    and the wavefront film equals the megakernel's."""
    from syfrack_gb300 import RenderSession
    from syfrack_gb300.scene import AreaLight, Camera, Material, RenderConfig, Scene

    g, _ = big_hierarchy()
    g.bounding_radius_hint = 40.0
    cam = Camera.look_at((-4.0, 3.0, -9.0), (-12.0, -6.0, 3.0), 60.0)
    w = h = 96
    gpu = renderer.primary(g, cam, w, h, max_steps=256, rule="cone", eps=1e-4, t_far=60.0, normal="central")
    sd = Scene(graph=None, camera=cam).desc(w, h)
    ref = oracle_mod.OracleGraph(g).primary(sd.camera, w, h, 256, 0, 1e-4, 60.0, 1.0, 0, precision=32)
    hit_g, hit_r = gpu["t"] >= 0, ref["t"] >= 0
    assert (hit_g == hit_r).mean() >= 0.995 and hit_g.mean() > 0.3
    both = hit_g & hit_r
    assert (np.abs(gpu["t"][both] - ref["t"][both]) <= 1e-4 * ref["t"][both]).mean() >= 0.99
    ds = np.abs(gpu["steps"].astype(np.int64) - ref["steps"].astype(np.int64))
    assert (ds == 0).mean() >= 0.95

    scene = Scene(graph=g, camera=cam, material=Material(albedo=(0.7, 0.7, 0.7), roughness=0.3),
                  lights=[AreaLight(position=(-10.0, 8.0, -2.0), normal=(0.0, -1.0, 0.0), size=(4.0, 4.0),
                                    color=(1.0, 1.0, 1.0), intensity=10.0)], seed=5)

    def film(integrator):
        cfg = RenderConfig(width=64, height=48, samples_per_pixel=4, max_bounces=3, max_steps=256,
                           pixel_tolerance=1.0, tile_size=64, samples_per_dispatch=4, integrator=integrator)
        s = RenderSession(renderer, scene, cfg)
        while not s.step(0):
            pass
        out = s.readback()
        assert s.sync() == 0
        s.close()
        return out

    a, b = film("wavefront"), film("megakernel")
    np.testing.assert_array_equal(a.accum, b.accum)
    assert (a.depth >= 0).mean() > 0.3


@pytest.mark.gpu
def test_device_nested_copies_against_brute_force_and_oracle(renderer, oracle_mod):
    """Three nested levels on the device: the interpreter keeps one copy search per
    level; it follows the composed brute force and the oracle, and its march with the
    GPU's skips follows the oracle's."""
    from test_gpu_de import gpu_de_rule

    g, levels = nested_copies()
    pts = grid_points() * 1.6
    r = renderer.compile(g).probe(pts)
    np.testing.assert_allclose(r["distance"], brute_force_nested(pts, levels), atol=2e-4, rtol=0)
    lcg = lcg_points(4096, 5.0, 31)
    assert gpu_de_rule(renderer.compile(g).probe(lcg), oracle_mod.OracleGraph(g).de(lcg, precision=32)) <= 0.005
    cam_pos, target = (2.0, 3.5, -7.0), (0.0, 0.0, 0.0)
    from syfrack_gb300.scene import Camera, Scene

    cam = Camera.look_at(cam_pos, target, 55.0)
    w = h = 64
    gpu = renderer.primary(g, cam, w, h, max_steps=256, rule="cone", eps=1e-4, t_far=40.0, normal="central")
    sd = Scene(graph=None, camera=cam).desc(w, h)
    ref = oracle_mod.OracleGraph(g).primary(sd.camera, w, h, 256, 0, 1e-4, 40.0, 1.0, 0, precision=32)
    hit_g, hit_r = gpu["t"] >= 0, ref["t"] >= 0
    assert (hit_g == hit_r).mean() >= 0.99 and hit_g.mean() > 0.1
    ds = np.abs(gpu["steps"].astype(np.int64) - ref["steps"].astype(np.int64))
    assert (ds == 0).mean() >= 0.95


def test_fence_hierarchy_contains_every_copy_once(oracle_mod):
    """bvh.rs:104-137: 1,031 rotated, scaled copies; every node's escape is past it,
    every placement is one leaf, and every corner of a copy's fence box lies inside
    its leaf and all the leaf's ancestors; far away the root is far."""
    placements = [(((i % 31) * 3.0, float(i // 31), i * 0.01), (float(i), 31.0, -19.0), (0.2, 2.0, 1.3))
                  for i in range(1031)]
    half = np.array([1.0, 0.3, 2.0])
    nodes = oracle_mod.bvh_build(placements, half).astype(np.float64)
    assert len(nodes) == 2 * len(placements) - 1

    def dist(n, p):
        q = np.abs(p - n[:3]) - n[3:6]
        return np.linalg.norm(np.maximum(q, 0.0)) + min(q.max(), 0.0)

    seen = np.zeros(len(placements), bool)
    for i, n in enumerate(nodes):
        esc = int(n[6])
        assert i < esc <= len(nodes)
        leaf = int(n[7])
        if leaf < 0:
            continue
        assert not seen[leaf]
        seen[leaf] = True
        pos, ang, sc = (np.array(x, np.float64) for x in placements[leaf])
        r = rot_matrix(ang)
        parents = [nodes[j] for j in range(i) if nodes[j][6] > i]
        for corner in np.array(np.meshgrid([-1, 1], [-1, 1], [-1, 1])).reshape(3, -1).T:
            c = pos + r @ (half * sc * corner)
            assert dist(n, c) < 0.0
            for par in parents:
                assert dist(par, c) < 0.0
    assert seen.all()
    assert dist(nodes[0], np.full(3, 1e5)) > 1.0

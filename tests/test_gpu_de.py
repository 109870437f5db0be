"""DE parity of the CUDA path against the oracle (GPU).

Rules: golden fixtures as graph_parity.rs:34-65 (distance 1e-5 rel/abs, traps
1e-5, iterations equal); LCG corpora with the tolerance of gpu_de.rs:38-91
(skip |d| < 0.02; a point fails when |dd| > 1e-3 + 0.02|d|, a trap differs by
more than 0.02 or iterations differ; at most 0.5% may fail)."""
import numpy as np
import pytest

from helpers import FORMS, golden, lcg_points
from syfrack_gb300 import SyfrackError
from syfrack_gb300.graph import Graph, Kind, Link, Node

pytestmark = pytest.mark.gpu
EXTENTS = {"sphere": 3.0, "mandelbulb": 1.6, "mandelbox": 8.0, "menger": 1.6}


@pytest.mark.parametrize("name", FORMS)
def test_golden_fixture_on_gpu(renderer, name):
    extent, pts, dist, traps, iters = golden(name)
    g = renderer.compile(Graph.bundled(name))
    assert g.info()["form"] == {"sphere": "generic", "mandelbulb": "bulb", "mandelbox": "box", "menger": "menger"}[name]
    r = g.probe(pts)
    err = np.abs(r["distance"] - dist) / np.maximum(np.abs(dist), 1.0)
    assert err.max() <= 1e-5, err.max()
    assert np.abs(r["traps"] - traps).max() <= 1e-5
    np.testing.assert_array_equal(r["iterations"], iters)


def gpu_de_rule(gpu, ref, d_floor=0.02):
    d, rd = gpu["distance"].astype(np.float64), ref["distance"]
    keep = np.abs(rd) >= d_floor
    bad = (np.abs(d - rd) > 1e-3 + 0.02 * np.abs(rd)) | (np.abs(gpu["traps"] - ref["traps"]).max(1) > 0.02) | \
          (gpu["iterations"] != ref["iterations"])
    return (bad & keep).sum() / max(keep.sum(), 1)


@pytest.mark.parametrize("name", FORMS)
@pytest.mark.parametrize("prec", [32, 64])
def test_lcg_corpus_against_oracle(renderer, oracle_mod, name, prec):
    pts = lcg_points(4096, EXTENTS[name], 11)
    g = Graph.bundled(name)
    gpu = renderer.compile(g).probe(pts)
    ref = oracle_mod.OracleGraph(g).de(pts, precision=prec)
    assert gpu_de_rule(gpu, ref) <= 0.005
    if prec == 32:
        # stricter: the f32 restatement and the device agree to a few ulps almost everywhere
        rel = np.abs(gpu["distance"] - ref["distance"]) / np.maximum(np.abs(ref["distance"]), 1.0)
        assert np.quantile(rel, 0.99) < 1e-5
        assert (gpu["iterations"] == ref["iterations"]).mean() >= 0.995


def _with_disabled_tail(g):
    """Same field, but a disabled body node forces the generic interpreter."""
    it = g.nodes[1]
    nid = max(n.id for n in g.nodes) + 1
    g.nodes.append(Node(nid, Kind("Translate", offset=[5.0, 0.0, 0.0]), enabled=False))
    it.kind.fields["body"] = list(it.kind.fields["body"]) + [nid]
    return g


@pytest.mark.parametrize("name", ["mandelbulb", "mandelbox", "menger"])
def test_generic_interpreter_matches_specialised_form(renderer, name):
    pts = lcg_points(2048, EXTENTS[name] * 0.6, 3)
    fast = renderer.compile(Graph.bundled(name))
    slow = renderer.compile(_with_disabled_tail(Graph.bundled(name)))
    assert slow.info()["form"] == "generic"
    a, b = fast.probe(pts), slow.probe(pts)
    rel = np.abs(a["distance"] - b["distance"]) / np.maximum(np.abs(a["distance"]), 1.0)
    assert rel.max() < 1e-5
    assert (a["iterations"] == b["iterations"]).mean() >= 0.999


def kitchen_sink():
    """Many node kinds through the generic interpreter: transforms, folds, nested
    Iterate with AddSeed, fences, smooth/hard combinations, MaterialTag, Bounded."""
    n = [
        Node(0, Kind("Input")),
        Node(1, Kind("Rotate", angles=[10.0, 20.0, -15.0])),
        Node(2, Kind("Translate", offset=[0.1, -0.2, 0.05])),
        Node(3, Kind("Iterate", iterations=6, bailout=8.0, body=[4, 5, 6, 7, 8])),
        Node(4, Kind("Abs", x=True, y=False, z=True)),
        Node(5, Kind("SphereFold", min_radius=0.4, fixed_radius=1.1)),
        Node(6, Kind("Scale", factor=1.8)),
        Node(7, Kind("AddSeed", multiplier=[0.5, 0.5, 0.5])),
        Node(8, Kind("Trap", slot=1, measure="AxisY", scale=2.0, mode="Maximum")),
        Node(9, Kind("NormFence", inset=0.2)),
        Node(10, Kind("Twist", rate=0.3)),
        Node(11, Kind("Torus", radius=1.0, tube=0.25)),
        Node(12, Kind("SmoothUnion", k=0.3)),
        Node(13, Kind("MaterialTag", index=2)),
        Node(14, Kind("Kaleido", planes=5, phase=12.0)),
        Node(15, Kind("RoundBox", half=[0.6, 0.3, 0.6], radius=0.1)),
        Node(16, Kind("Subtraction")),
        Node(17, Kind("Box", half=[0.3, 0.3, 0.3])),
        Node(18, Kind("Bounded", half=[3.0, 3.0, 3.0], margin=0.1)),
        Node(19, Kind("Output")),
        Node(20, Kind("Trap", slot=2, measure="AngleXZ", scale=1.0, mode="Last")),
        Node(21, Kind("Cylinder", radius=0.2, half_height=2.0)),
        Node(22, Kind("Intersection")),
    ]
    L = lambda a, b, p=0: Link((a, 0), (b, p))
    links = [L(0, 1), L(1, 2), L(2, 3), L(3, 9), L(0, 10), L(10, 11), L(9, 12), L(11, 12, 1), L(12, 13),
             L(0, 14), L(14, 20), L(20, 15), L(13, 16), L(15, 16, 1), L(16, 22), L(0, 21), L(21, 22, 1),
             L(0, 18), L(22, 18, 1), L(18, 19)]
    return Graph(n, links, safety=0.8, bounding_radius_hint=3.0)


def test_spherical_power_vectors_on_the_device(renderer):
    """eval.rs:180-222 on the device's Power node (the binary-power branch for n outside
    {6, 8}, the repeated squaring for 6 and 8): the powered point of n = 1..16 against
    FP64 trigonometry on the reference's points, within the reference's bounds (5e-6
    r^n on the point, 4e-6 on the derivative), and the filament (1e-6, 0, 1)^8."""
    from test_oracle import power_component_graph, spherical_power_error, spherical_power_points

    pts = spherical_power_points()
    worst = {}
    for n in range(1, 17):
        d = [renderer.compile(power_component_graph(n, a)).probe(pts)["distance"].astype(np.float64) for a in range(3)]
        worst[n] = spherical_power_error(d, pts, n)
    print({n: round(w, 3) for n, w in worst.items()})
    assert max(worst.values()) <= 1.0, worst
    x = renderer.compile(power_component_graph(8, 0)).probe(np.array([[1e-6, 0.0, 1.0]], np.float32))["distance"][0]
    assert abs(float(x) * 8.0 - 8e-6) < 1e-10


def test_generic_node_kinds_against_oracle(renderer, oracle_mod):
    g = kitchen_sink()
    pts = lcg_points(4096, 2.5, 17)
    gpu = renderer.compile(g).probe(pts)
    ref = oracle_mod.OracleGraph(g).de(pts, precision=32)
    assert renderer.compile(g).info()["form"] == "generic"
    assert gpu_de_rule(gpu, ref) <= 0.005
    np.testing.assert_array_equal(gpu["material"], ref["material"])


def test_value_edit_without_recompile(renderer, oracle_mod):
    g = Graph.bundled("mandelbulb")
    cg = renderer.compile(g)
    g2 = Graph.bundled("mandelbulb", power=6.0)  # 6 and 8 share a topology (graph/mod.rs:397-425)
    cg.update(g2)
    pts = lcg_points(256, 1.2, 9)
    ref = oracle_mod.OracleGraph(g2).de(pts, precision=32)
    assert gpu_de_rule(cg.probe(pts), ref) <= 0.005
    with pytest.raises(SyfrackError):
        cg.update(Graph.bundled("mandelbulb", power=7.0))
    cg.update(g)


def test_sizes(renderer):
    g = renderer.compile(Graph.bundled("menger"))
    assert len(g.probe(np.zeros((0, 3)))["distance"]) == 0
    one = g.probe(np.array([[0.5, 0.5, 0.5]]))
    big_pts = lcg_points(1, 1.0, 1)
    big = np.repeat(np.array([[0.5, 0.5, 0.5]], np.float32), 1 << 20, axis=0)
    r = g.probe(big)
    assert np.all(r["distance"] == one["distance"][0]) and len(big_pts) == 1


def test_invalid_graphs_are_rejected(renderer):
    bad = Graph([Node(0, Kind("Input")), Node(1, Kind("Output"))], [Link((0, 0), (1, 0))])
    with pytest.raises(SyfrackError) as e:
        renderer.compile(bad)
    assert e.value.status == 2
    cyc = Graph([Node(0, Kind("Input")), Node(1, Kind("Translate", offset=[0, 0, 0])),
                 Node(2, Kind("Translate", offset=[0, 0, 0])), Node(3, Kind("Sphere", radius=1.0)),
                 Node(4, Kind("Output"))],
                [Link((1, 0), (2, 0)), Link((2, 0), (1, 0)), Link((2, 0), (3, 0)), Link((3, 0), (4, 0))])
    with pytest.raises(SyfrackError):
        renderer.compile(cyc)


def _c3_extent(kind, value):
    if kind == "mandelbox":  # negative scales fill the cube [-2, 2]^3; positive ones reach 2(s+1)/(s-1)
        return 4.0 if value <= 1.0 else min(2.0 * (value + 1.0) / (value - 1.0), 12.0) * 1.2
    return 1.6


C3_FORMS = ([("mandelbulb", float(p)) for p in range(2, 13)] +
            [("mandelbox", s) for s in (-2.5, -2.0, -1.5, -1.05, -0.8, -0.3, -0.01, 0.01, 0.4, 0.9, 1.05, 1.5, 2.0,
                                        2.5)] +
            [("menger", lv) for lv in range(3, 8)])


@pytest.mark.parametrize("kind,value", C3_FORMS, ids=[f"{k}-{v:g}" for k, v in C3_FORMS])
def test_mixed_batch_forms_against_oracle(renderer, oracle_mod, kind, value):
    """Every form the uneven batch draws (Mandelbulb powers 2-12, including the
    binary-exponentiation powers of eval.rs:157-177; Mandelbox scales across -2.5..2.5,
    |s| < 1.05 included; Menger levels 3-7) on the device against the f32 and f64
    oracle: the gpu_de.rs rule, and against f32 99% of relative errors below 1e-5
    with at least 99.5% of iteration counts equal."""
    from syfrack_gb300 import workloads

    if kind == "mandelbulb":
        g = workloads.mixed_batch_graph("mandelbulb", value)
    elif kind == "mandelbox":
        g = workloads.mixed_batch_graph("mandelbox", value)
    else:
        g = workloads.mixed_batch_graph("menger", int(value))
    pts = lcg_points(4096, _c3_extent(kind, value), 29)
    cg = renderer.compile(g)
    assert cg.info()["form"] == {"mandelbulb": "bulb", "mandelbox": "box", "menger": "menger"}[kind]
    gpu = cg.probe(pts)
    og = oracle_mod.OracleGraph(g)
    ref32, ref64 = og.de(pts, precision=32), og.de(pts, precision=64)
    assert gpu_de_rule(gpu, ref64) <= 0.005
    assert gpu_de_rule(gpu, ref32) <= 0.005
    rel = np.abs(gpu["distance"] - ref32["distance"]) / np.maximum(np.abs(ref32["distance"]), 1.0)
    assert np.quantile(rel, 0.99) < 1e-5, np.quantile(rel, 0.99)
    assert (gpu["iterations"] == ref32["iterations"]).mean() >= 0.995


def test_mixed_batch_scale_band_the_reference_rejects(renderer):
    """Scale factors below 1e-3 in magnitude fail validation (validate.rs:187-196), so
    the uneven batch draws its Mandelbox scales from -2.5..2.5 without that band."""
    from syfrack_gb300 import workloads

    with pytest.raises(SyfrackError) as e:
        renderer.compile(workloads.mixed_batch_graph("mandelbox", 0.0))
    assert e.value.status == 2
    jobs = workloads.mixed_batch(seed=7, jobs=64)
    scales = [n.kind.fields["factor"] for sc, _ in jobs for n in sc.graph.nodes if n.kind.name == "Scale"]
    assert len(scales) >= 20 and min(abs(x) for x in scales) >= 1e-3
    assert min(scales) < -1.0 and max(scales) > 1.0 and any(abs(x) < 1.05 for x in scales)

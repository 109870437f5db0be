"""The exact union branch-and-bound (graph_wgsl.rs:1112-1154, union_leaves :18-26).

When a graph has a skippable Bounded or Instances node and the Output's input is a
tree of enabled Unions over several distinct leaves, the reference's exact sample
probes every leaf for its conservative distance and evaluates exactly only the
leaves whose bound can still beat the best. Skippable bounds are lower bounds, so
the winner is the plain union's: the nearest leaf, the first in depth-first order on
ties. The CPU tests check which graphs take the search (sf_graph_info.
exact_union_leaves, from the host lowering); the GPU tests check that its samples are
bit-identical to the whole program's (the same graph behind a disabled MaterialTag,
which the search does not see through, as union_leaves does not), follow the oracle
under the gpu_de.rs rule, and leave the preview unchanged. The device searches in
the kernels whose work is exact samples (the batched probe and the preview), for
unions of three or more leaves; the path tracers run the whole program, which gives
the same sample."""
import numpy as np
import pytest

from helpers import bounded_bulb, lcg_points
from syfrack_gb300.graph import Graph, Kind, Link, Node


class _Builder:
    def __init__(self):
        self.nodes = [Node(0, Kind("Input"))]
        self.links = []

    def add(self, kind, inputs=(), enabled=True):
        nid = len(self.nodes)
        self.nodes.append(Node(nid, kind, enabled=enabled))
        for port, src in enumerate(inputs):
            if src is not None:
                self.links.append(Link((src, 0), (nid, port)))
        return nid

    def graph(self, root, hint=6.0):
        out = self.add(Kind("Output"), [root])
        assert out == len(self.nodes) - 1
        return Graph(self.nodes, self.links, safety=0.8, bounding_radius_hint=hint)


def _bulb(b, centre, tag, margin=0.05):
    """A Mandelbulb (AddSeed reinjects the translated point) behind a skippable box."""
    t = b.add(Kind("Translate", offset=[-x for x in centre]), [0])
    body = [b.add(Kind("Trap", slot=0, measure="Norm", scale=4.0)), b.add(Kind("Power", power=8.0)),
            b.add(Kind("AddSeed", multiplier=[1.0, 1.0, 1.0]))]
    it = b.add(Kind("Iterate", iterations=8, bailout=2.0, body=body), [t])
    fence = b.add(Kind("BulbFence"), [it])
    bound = b.add(Kind("Bounded", half=[1.25, 1.25, 1.25], margin=margin), [t, fence])
    return b.add(Kind("MaterialTag", index=tag), [bound])


def _shape(b, kind, centre, tag=None, bounded=None):
    t = b.add(Kind("Translate", offset=[-x for x in centre]), [0])
    d = b.add(kind, [t])
    if bounded is not None:
        d = b.add(Kind("Bounded", half=[bounded] * 3, margin=0.05), [t, d])
    return b.add(Kind("MaterialTag", index=tag), [d]) if tag is not None else d


def union_world(hidden=False):
    """Nine union leaves (eight distinct: one is reached twice) of every kind the search
    meets: three bounded Mandelbulbs, copies of a torus (Instances), an unbounded
    sphere (its probe is exact), a box minus a bounded sphere (a bound through a
    Subtraction's second input is evaluated exactly), two coincident bounded spheres
    with different materials (an exact tie: the first leaf wins), and a disabled Union
    (a leaf passing its first input). hidden puts a disabled MaterialTag between the
    union and the Output: the whole program runs and the sample is the same."""
    b = _Builder()
    bulbs = [_bulb(b, c, i + 1) for i, c in enumerate([(2.2, 0.0, 0.0), (-2.2, 0.0, 0.0), (0.0, 2.2, 0.0)])]
    tor = b.add(Kind("Torus", radius=0.6, tube=0.15), [0])
    tor = b.add(Kind("MaterialTag", index=4), [tor])
    copies = b.add(Kind("Instances", placements=[((0.0, -2.2, 0.0), (20.0, 0.0, 10.0), (1.0, 1.0, 1.0)),
                                                 ((0.9, -2.4, 0.6), (-30.0, 45.0, 0.0), (0.7, 0.8, 0.9))],
                        half=[0.8, 0.8, 0.8], margin=0.05), [tor])
    sphere = _shape(b, Kind("Sphere", radius=0.7), (0.0, 0.0, 2.2), tag=5)
    box = _shape(b, Kind("Box", half=[0.7, 0.7, 0.7]), (0.0, 0.0, -2.2))
    hole = _shape(b, Kind("Sphere", radius=0.85), (0.0, 0.0, -2.2), bounded=1.0)
    cut = b.add(Kind("MaterialTag", index=6), [b.add(Kind("Subtraction"), [box, hole])])
    tie_a = _shape(b, Kind("Sphere", radius=0.5), (2.0, 2.0, 0.0), tag=7, bounded=0.6)
    tie_b = _shape(b, Kind("Sphere", radius=0.5), (2.0, 2.0, 0.0), tag=8, bounded=0.6)
    rb = _shape(b, Kind("RoundBox", half=[0.4, 0.3, 0.5], radius=0.1), (-2.0, 2.0, 0.0), tag=9)
    cyl = _shape(b, Kind("Cylinder", radius=0.3, half_height=0.5), (-2.0, 2.0, 0.0), tag=10)
    off = b.add(Kind("Union"), [rb, cyl], enabled=False)
    u = lambda x, y: b.add(Kind("Union"), [x, y])
    # a left-deep chain with a balanced subtree; the sphere is reached a second time
    left = u(u(u(bulbs[0], bulbs[1]), bulbs[2]), copies)
    right = u(u(sphere, cut), u(tie_a, tie_b))
    root = u(u(left, right), u(off, sphere))
    if hidden:
        root = b.add(Kind("MaterialTag", index=11), [root], enabled=False)
    return b.graph(root)


UNION_WORLD_LEAVES = 9  # three bulbs, the copies, the sphere, the cut, the tie pair, the disabled union


def union_points():
    """LCG points over the world, and points clustered about each leaf where the
    bounds flip between skipped and evaluated."""
    centres = [(2.2, 0, 0), (-2.2, 0, 0), (0, 2.2, 0), (0, -2.2, 0), (0, 0, 2.2), (0, 0, -2.2), (2, 2, 0), (-2, 2, 0)]
    near = [lcg_points(1024, 1.4, 40 + i) + np.array(c, np.float32) for i, c in enumerate(centres)]
    return np.concatenate([lcg_points(4096, 3.6, 23)] + near).astype(np.float32)


# ---------------------------------------------------------------- CPU: the host lowering

def test_which_graphs_take_the_search():
    assert union_world().validate()["exact_union_leaves"] == UNION_WORLD_LEAVES
    # behind a disabled tag the Output's input is not a Union: one leaf, no search
    assert union_world(hidden=True).validate()["exact_union_leaves"] == 0
    # the helper's bounded bulb beside a sphere: two leaves
    assert bounded_bulb().validate()["exact_union_leaves"] == 2
    # under a Subtraction's second input the bound is not skippable: no fast node, no search
    assert bounded_bulb(subtract=True).validate()["exact_union_leaves"] == 0
    # a union with no Bounded or Instances anywhere runs the whole program
    b = _Builder()
    s1 = _shape(b, Kind("Sphere", radius=1.0), (1.0, 0.0, 0.0))
    s2 = _shape(b, Kind("Sphere", radius=1.0), (-1.0, 0.0, 0.0))
    assert b.graph(b.add(Kind("Union"), [s1, s2])).validate()["exact_union_leaves"] == 0


def test_a_leaf_reached_twice_counts_once():
    b = _Builder()
    s = _shape(b, Kind("Sphere", radius=1.0), (1.0, 0.0, 0.0), bounded=1.2)
    t = _shape(b, Kind("Torus", radius=1.0, tube=0.2), (-1.0, 0.0, 0.0))
    root = b.add(Kind("Union"), [b.add(Kind("Union"), [s, t]), s])
    assert b.graph(root).validate()["exact_union_leaves"] == 2
    # a disabled inner Union is one leaf: its first input passes through
    b = _Builder()
    s = _shape(b, Kind("Sphere", radius=1.0), (1.0, 0.0, 0.0), bounded=1.2)
    t = _shape(b, Kind("Torus", radius=1.0, tube=0.2), (-1.0, 0.0, 0.0))
    c = _shape(b, Kind("Box", half=[0.5, 0.5, 0.5]), (0.0, 2.0, 0.0))
    root = b.add(Kind("Union"), [b.add(Kind("Union"), [s, t], enabled=False), c])
    assert b.graph(root).validate()["exact_union_leaves"] == 2


def test_oracle_search_is_the_union(oracle_mod):
    """The oracle's restatement of the search (probe every leaf, then the exact leaves
    whose bound can beat the best) returns the union's own sample: equal in every field
    to the plain evaluation, in binary32 and in FP64, on points about every leaf; the
    leaves it walks are the host lowering's."""
    og = oracle_mod.OracleGraph(union_world())
    assert og.union_leaves() == (UNION_WORLD_LEAVES, True)
    assert oracle_mod.OracleGraph(union_world(hidden=True)).union_leaves()[0] == 1
    assert oracle_mod.OracleGraph(bounded_bulb(subtract=True)).union_leaves()[1] is False
    pts = union_points()
    for prec in (32, 64):
        a, b = og.de_search(pts, precision=prec), og.de(pts, precision=prec)
        for k in ("distance", "traps", "iterations", "material"):
            np.testing.assert_array_equal(a[k], b[k], err_msg=f"{k} at {prec} bits")
        # six of the nine leaves have skippable bounds (their probes are bounds); the
        # search evaluates few of them exactly
        assert a["exact_leaves"].max() <= 6 and a["exact_leaves"].mean() < 2.5, a["exact_leaves"].mean()
    # far from the world every probe of a bounded leaf loses to an exact probe (the
    # sphere, the cut, the disabled union's leaf) or to another bound: still the union
    far = lcg_points(512, 12.0, 5)
    a, b = og.de_search(far, precision=64), og.de(far, precision=64)
    np.testing.assert_array_equal(a["distance"], b["distance"])
    np.testing.assert_array_equal(a["material"], b["material"])


def test_the_world_is_within_the_device_program():
    info = union_world().validate()
    hidden = union_world(hidden=True).validate()
    assert info["form"] == "generic" and info["op_count"] == hidden["op_count"] <= 96


# ---------------------------------------------------------------- GPU

@pytest.mark.gpu
def test_search_samples_equal_the_whole_program(renderer, oracle_mod):
    from test_gpu_de import gpu_de_rule

    pts = union_points()
    g = renderer.compile(union_world())
    assert g.info()["exact_union_leaves"] == UNION_WORLD_LEAVES
    plain = renderer.compile(union_world(hidden=True))
    assert plain.info()["exact_union_leaves"] == 0
    a, b = g.probe(pts), plain.probe(pts)
    for k in ("distance", "traps", "iterations", "material"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    # every leaf wins somewhere, the tie goes to the first of the coincident spheres
    mats = set(np.unique(a["material"]).tolist())
    assert {1, 2, 3, 4, 5, 6, 7, 9} <= mats and 8 not in mats
    ref = oracle_mod.OracleGraph(union_world()).de(pts, precision=32)
    assert gpu_de_rule(a, ref) <= 0.005
    close = np.abs(ref["distance"]) >= 0.02
    assert (a["material"][close] == ref["material"][close]).mean() >= 0.999


@pytest.mark.gpu
def test_search_leaves_the_preview_unchanged(renderer):
    """The preview marches on the exact field, every step a searched sample: its
    depth, normals, step counts and shading equal the whole program's."""
    from syfrack_gb300 import PreviewSession
    from syfrack_gb300.scene import Camera, Scene

    cam = Camera.look_at((1.5, 4.5, -6.5), (0.0, 0.3, 0.0), 60.0)
    imgs = []
    for hidden in (False, True):
        p = PreviewSession(renderer, Scene(graph=union_world(hidden=hidden), camera=cam), (160, 120))
        p.wait_complete()
        imgs.append(p.readback())
        p.close()
    a, b = imgs
    assert (a["depth"] > 0).mean() > 0.2
    for k in ("accum", "depth", "aux"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.gpu
@pytest.mark.parametrize("integrator", ["wavefront", "megakernel"])
def test_path_tracers_render_the_world(renderer, integrator):
    """The path tracers take the whole-program exact sample (the search would raise
    their register allocation for no gain): the world's film is the hidden graph's."""
    from syfrack_gb300 import RenderSession
    from syfrack_gb300.scene import AreaLight, Camera, Material, RenderConfig, Scene

    def film(graph):
        scene = Scene(graph=graph, camera=Camera.look_at((1.5, 4.5, -6.5), (0.0, 0.3, 0.0), 60.0),
                      material=Material(albedo=(0.7, 0.6, 0.5), roughness=0.3),
                      lights=[AreaLight(position=(0.0, 6.0, -3.0), normal=(0.0, -1.0, 0.5), size=(2.0, 2.0),
                                        color=(1.0, 1.0, 1.0), intensity=12.0)], seed=17)
        cfg = RenderConfig(width=96, height=64, samples_per_pixel=4, max_bounces=3, max_steps=256,
                           pixel_tolerance=1.0, tile_size=64, samples_per_dispatch=4, integrator=integrator)
        s = RenderSession(renderer, scene, cfg)
        while not s.step(0):
            pass
        out = s.readback()
        assert s.sync() == 0
        s.close()
        return out

    a, b = film(union_world()), film(union_world(hidden=True))
    assert (a.depth >= 0).mean() > 0.2
    np.testing.assert_array_equal(a.accum, b.accum)
    np.testing.assert_array_equal(a.depth, b.depth)

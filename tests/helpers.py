"""Shared test inputs: the reference's LCG point sets (graph_parity.rs:4-13,
parity.rs corpus) and golden fixture loading."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FORMS = ["sphere", "mandelbulb", "mandelbox", "menger"]


def lcg_points(n, extent, seed):
    """points() of crates/syfrack-core/tests/graph_parity.rs:8-13, in binary32."""
    s = seed & 0xFFFFFFFF
    out = np.zeros((n, 3), np.float32)
    e = np.float32(extent)
    for i in range(n):
        v = []
        for _ in range(3):
            s = (s * 1664525 + 1013904223) & 0xFFFFFFFF
            v.append(np.float32(s >> 8) / np.float32(16777216.0))
        out[i] = np.array(v, np.float32) * (np.float32(2.0) * e) - e
    return out


def golden(name):
    with open(os.path.join(GOLDEN, f"de_parity_{name}.json")) as f:
        d = json.load(f)
    s = d["samples"]
    return (d["extent"], np.array([r["p"] for r in s], np.float32), np.array([r["distance"] for r in s]),
            np.array([r["traps"] for r in s]), np.array([r["iterations"] for r in s], np.uint32))


def golden_graph(name):
    from syfrack_gb300.graph import Graph

    with open(os.path.join(GOLDEN, f"graph_{name}.json")) as f:
        d = json.load(f)
    return Graph.from_ron_value(_jsonish_to_ron(d["graph"]))


def _jsonish_to_ron(g):
    """The fixture JSON keeps RON's shape; rebuild the few tuple fields."""
    from syfrack_gb300 import ron

    g = json.loads(json.dumps(g))
    for n in g["nodes"]:
        k = n["kind"]
        if isinstance(k, str):
            n["kind"] = ron.Unit(k)
        n["pos"] = ron.Tuple(None, n["pos"])
    g["links"] = [{"from": ron.Tuple(None, l["from"]), "to": ron.Tuple(None, l["to"])} for l in g["links"]]
    return g


def bounded_bulb(subtract=False, margin=0.05):
    """A Mandelbulb clipped by a Bounded box (half 1.25, the GPU may skip it outside
    the margin) beside a translated sphere. With subtract, the bounded bulb is the
    second input of a Subtraction from a large sphere, where its bound is not a lower
    bound and the GPU evaluates it exactly (graph_wgsl.rs:976-1006)."""
    from syfrack_gb300.graph import Graph, Kind, Link, Node

    g = Graph.bundled("mandelbulb", power=8.0, iterations=12, bailout=2.0, safety=0.7, hint=2.5)
    g.links = [l for l in g.links if l.dst != (6, 0)]
    g.nodes += [
        Node(7, Kind("Bounded", half=[1.25, 1.25, 1.25], margin=margin)),
        Node(8, Kind("Translate", offset=[2.2, 0.0, 0.0])),
        Node(9, Kind("Sphere", radius=0.5)),
        Node(10, Kind("Union")),
    ]
    g.links += [Link((0, 0), (7, 0)), Link((5, 0), (7, 1)), Link((0, 0), (8, 0)), Link((8, 0), (9, 0)),
                Link((7, 0), (10, 0)), Link((9, 0), (10, 1))]
    if subtract:
        g.nodes += [Node(11, Kind("Sphere", radius=4.0)), Node(12, Kind("Subtraction"))]
        g.links += [Link((0, 0), (11, 0)), Link((11, 0), (12, 0)), Link((10, 0), (12, 1)), Link((12, 0), (6, 0))]
    else:
        g.links.append(Link((10, 0), (6, 0)))
    return g


def golden_scene(name, atmosphere=None):
    """scenes/<name>.ron from its JSON copy, read by the package's scene-file reader;
    `atmosphere` overrides fields of the file's atmosphere."""
    from syfrack_gb300 import ron
    from syfrack_gb300.scene import scene_from_ron_value

    with open(os.path.join(GOLDEN, f"scene_{name}.json")) as f:
        d = json.load(f)

    def back(v):
        if isinstance(v, dict) and "nodes" in v and "links" in v:  # a texture's graph
            return _jsonish_to_ron(v)
        if isinstance(v, dict) and "__items__" in v:
            items = [back(x) for x in v["__items__"]]
            if v["__name__"] == "Graph":
                items = [_jsonish_to_ron(v["__items__"][0])]
            return ron.Tuple(v["__name__"], items)
        if isinstance(v, dict):
            return {k: back(x) for k, x in v.items()}
        if isinstance(v, list):
            return [back(x) for x in v]
        if isinstance(v, str) and v in ("None", "Smooth", "Linear"):
            return ron.Unit(v)
        return v

    if atmosphere:
        d["scene"].setdefault("atmosphere", {}).update(atmosphere)
    return scene_from_ron_value(back(d["scene"]))


def golden_film_blocks(name):
    with open(os.path.join(GOLDEN, f"film_{name}_blocks.json")) as f:
        d = json.load(f)
    return np.array(d["blocks"]).reshape(len(d["blocks"]), -1, 3), d

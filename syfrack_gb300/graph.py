"""The form graph: nodes, links and parameters, as in
crates/syfrack-core/src/scene/graph/mod.rs (Node :427-434, Link :436-441,
Graph :444-451, NodeKind :105-257), plus packing into the C ABI's sf_graph_desc.

A node kind is a `Kind(name, **fields)` with the reference's field names, e.g.
`Kind("Iterate", iterations=12, bailout=4.0, body=[2, 3, 4])`.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

from . import abi, ron


@dataclass
class Kind:
    name: str
    fields: dict = field(default_factory=dict)

    def __init__(self, name: str, **fields):
        if name not in abi.KIND_ID:
            raise ValueError(f"unknown node kind {name!r}")
        self.name = name
        self.fields = fields

    def __getitem__(self, k):
        return self.fields[k]

    def __repr__(self):
        if not self.fields:
            return self.name
        inner = ", ".join(f"{k}: {v!r}" for k, v in self.fields.items())
        return f"{self.name}({inner})"


@dataclass
class Node:
    id: int
    kind: Kind
    name: str = ""
    pos: tuple = (0.0, 0.0)
    enabled: bool = True


@dataclass
class Link:
    src: tuple  # (node, port)  -- `from` in the reference
    dst: tuple  # (node, port)  -- `to` in the reference


def _v3(x):
    return ron.vec(x)


# (float slots, uint slots) per kind, following the table in include/syfrack_gpu.h.
def _pack_params(k: Kind):
    f = [0.0] * 8
    u = [0, 0, 0]
    d = k.fields
    n = k.name
    if n == "Translate":
        f[0:3] = _v3(d["offset"])
    elif n == "Rotate":
        f[0:3] = _v3(d["angles"])
    elif n == "Scale":
        f[0] = d["factor"]
    elif n == "ScaleAxes":
        f[0:3] = _v3(d["factors"])
    elif n == "Mirror":
        f[0:3] = _v3(d["normal"])
        f[3] = d["offset"]
    elif n == "BoxFold":
        f[0] = d["limit"]
    elif n == "BoxFoldAxes":
        f[0:3] = _v3(d["limit"])
        u = [int(bool(d["x"])), int(bool(d["y"])), int(bool(d["z"]))]
    elif n == "SphereInversion":
        f[0], f[1] = d["radius"], d["min_radius"]
    elif n == "SphereFold":
        f[0], f[1] = d["min_radius"], d["fixed_radius"]
    elif n == "Abs":
        u = [int(bool(d["x"])), int(bool(d["y"])), int(bool(d["z"]))]
    elif n == "MengerFold":
        f[0] = d["scale"]
        f[1:4] = _v3(d["offset"])
    elif n == "Kaleido":
        u[0] = int(d["planes"])
        f[0] = d["phase"]
    elif n == "Power":
        f[0] = d["power"]
    elif n == "AddSeed":
        f[0:3] = _v3(d["multiplier"])
    elif n == "AddConstant":
        f[0:3] = _v3(d["multiplier"])
        f[3:6] = _v3(d["julia"])
    elif n in ("Twist", "Bend"):
        f[0] = d["rate"]
    elif n == "Tile":
        f[0:3] = _v3(d["period"])
    elif n == "RepeatFinite":
        f[0:3] = _v3(d["period"])
        u = [int(c) for c in d["count"]]
    elif n == "Iterate":
        u[0] = int(d["iterations"])
        f[0] = d["bailout"]
    elif n == "Trap":
        u = [int(d["slot"]), abi.MEASURES.index(d.get("measure", "Norm")),
             abi.TRAP_MODES.index(d.get("mode", "Minimum"))]
        f[0] = d["scale"]
    elif n == "Sphere":
        f[0] = d["radius"]
    elif n == "Torus":
        f[0], f[1] = d["radius"], d["tube"]
    elif n == "Cylinder":
        f[0], f[1] = d["radius"], d["half_height"]
    elif n == "Box":
        f[0:3] = _v3(d["half"])
    elif n == "RoundBox":
        f[0:3] = _v3(d["half"])
        f[3] = d["radius"]
    elif n == "Rock":
        f[0:3] = _v3(d["half"])
        f[3] = d["erosion"]
        u[0] = int(d["seed"])
    elif n == "Plane":
        f[0:3] = _v3(d["normal"])
        f[3] = d["offset"]
    elif n == "NormFence":
        f[0] = d["inset"]
    elif n == "MaterialTag":
        u[0] = int(d["index"])
    elif n in ("Bounded", "Instances"):
        f[0:3] = _v3(d["half"])
        f[3] = d["margin"]
    elif n in ("SmoothUnion", "SmoothIntersection"):
        f[0] = d["k"]
    return f, u


class Graph:
    """Graph{nodes, links, safety, bounding_radius_hint} (graph/mod.rs:444-451)."""

    def __init__(self, nodes, links, safety=1.0, bounding_radius_hint=2.0):
        self.nodes = list(nodes)
        self.links = list(links)
        self.safety = float(safety)
        self.bounding_radius_hint = float(bounding_radius_hint)

    def node(self, id):
        for n in self.nodes:
            if n.id == id:
                return n
        return None

    # -- RON interop -----------------------------------------------------------
    @classmethod
    def from_ron_value(cls, v) -> "Graph":
        nodes = []
        for nd in v["nodes"]:
            kv = nd["kind"]
            if isinstance(kv, ron.Unit):
                kind = Kind(kv.name)
            else:
                name = kv.pop("__name__")
                fields = {}
                for key, val in kv.items():
                    if isinstance(val, ron.Unit):
                        val = val.name
                    elif isinstance(val, ron.Tuple):
                        val = list(val.items)
                    fields[key] = val
                kind = Kind(name, **fields)
            pos = nd.get("pos", ron.Tuple(None, [0.0, 0.0]))
            nodes.append(Node(int(nd["id"]), kind, nd.get("name", ""),
                              tuple(ron.vec(pos)), bool(nd.get("enabled", True))))
        links = []
        for l in v["links"]:
            links.append(Link(tuple(int(a) for a in l["from"].items),
                              tuple(int(a) for a in l["to"].items)))
        return cls(nodes, links, v.get("safety", 1.0), v.get("bounding_radius_hint", 2.0))

    @classmethod
    def from_ron(cls, text: str) -> "Graph":
        return cls.from_ron_value(ron.loads(text))

    @classmethod
    def bundled(cls, name: str, **params) -> "Graph":
        """The reference's bundled forms (graph/bundled.rs:8-47), built in code."""
        builders = {"mandelbulb": mandelbulb, "mandelbox": mandelbox, "menger": menger,
                    "sphere": sphere}
        if name not in builders:
            raise KeyError(name)
        return builders[name](**params)

    def validate(self) -> dict:
        """Graph::validate (validate.rs:146-330) through the library, on the host only:
        raises SyfrackError for an invalid graph, else returns the derived constants."""
        from ._lib import check, load

        desc, keep = self.to_desc()
        info = abi.sf_graph_info()
        check(load().sf_graph_validate(C.byref(desc), C.byref(info)))
        return {"step_scale": info.step_scale, "lipschitz": info.lipschitz,
                "trap_scales": list(info.trap_scales), "iteration_product": info.iteration_product,
                "form": abi.FORMS.get(info.form, info.form), "op_count": info.op_count,
                "exact_union_leaves": info.exact_union_leaves}

    # -- C ABI packing -----------------------------------------------------------
    def to_desc(self):
        """Returns (sf_graph_desc, keepalive) -- keep `keepalive` referenced while
        the descriptor is in use."""
        n = len(self.nodes)
        nodes = (abi.sf_node * max(n, 1))()
        body_ids: list[int] = []
        placements: list = []
        for i, nd in enumerate(self.nodes):
            f, u = _pack_params(nd.kind)
            s = nodes[i]
            s.id = nd.id
            s.kind = abi.KIND_ID[nd.kind.name]
            s.enabled = 1 if nd.enabled else 0
            for j in range(8):
                s.f[j] = float(f[j])
            for j in range(3):
                s.u[j] = int(u[j])
            if nd.kind.name == "Iterate":
                body = [int(b) for b in nd.kind.fields["body"]]
                s.body_offset = len(body_ids)
                s.body_len = len(body)
                body_ids.extend(body)
            if nd.kind.name == "Instances":
                own = [placement_tuple(p) for p in nd.kind.fields.get("placements", [])]
                s.u[0] = len(placements)
                s.u[1] = len(own)
                placements.extend(own)
        links = (abi.sf_link * max(len(self.links), 1))()
        for i, l in enumerate(self.links):
            links[i].from_node, links[i].from_port = l.src
            links[i].to_node, links[i].to_port = l.dst
        bodies = (C.c_uint32 * max(len(body_ids), 1))(*body_ids)
        pl = (abi.sf_placement * max(len(placements), 1))()
        for i, (pos, ang, sc) in enumerate(placements):
            pl[i].position[:] = pos
            pl[i].angles[:] = ang
            pl[i].scale[:] = sc
        d = abi.sf_graph_desc(nodes, n, links, len(self.links), bodies, len(body_ids),
                              self.safety, self.bounding_radius_hint, pl, len(placements))
        return d, (nodes, links, bodies, pl)


def placement_tuple(p):
    """Placement{position, angles, scale} (graph/mod.rs:26-40) from a dict (RON or
    keyword form) or a (position, angles, scale) triple; missing fields take the
    defaults (origin, no rotation, unit scale)."""
    if isinstance(p, dict):
        get = lambda k, dflt: [float(x) for x in _v3(p.get(k, dflt))]
        return (get("position", [0.0, 0.0, 0.0]), get("angles", [0.0, 0.0, 0.0]), get("scale", [1.0, 1.0, 1.0]))
    pos, ang, sc = p
    return ([float(x) for x in pos], [float(x) for x in ang], [float(x) for x in sc])


def _chain_links(pairs):
    return [Link((a, 0), (b, port)) for a, b, port in pairs]


def mandelbulb(power=8.0, iterations=12, bailout=4.0, trap_scale=4.0, safety=0.7, hint=2.5):
    """graphs/mandelbulb.ron: Iterate{Trap, Power, AddOrigin} -> BulbFence."""
    nodes = [
        Node(0, Kind("Input")),
        Node(1, Kind("Iterate", iterations=iterations, bailout=bailout, body=[2, 3, 4])),
        Node(2, Kind("Trap", slot=0, measure="Norm", scale=trap_scale)),
        Node(3, Kind("Power", power=power)),
        Node(4, Kind("AddOrigin")),
        Node(5, Kind("BulbFence")),
        Node(6, Kind("Output")),
    ]
    return Graph(nodes, _chain_links([(0, 1, 0), (1, 5, 0), (5, 6, 0)]), safety, hint)


def mandelbox(scale=2.0, iterations=12, bailout=1000.0, limit=1.0, min_radius=0.5,
              fixed_radius=1.0, trap_scale=2.0, safety=0.6, hint=10.392304):
    """graphs/mandelbox.ron: Iterate{BoxFold, Trap, SphereFold, Scale, AddOrigin} -> NormFence."""
    nodes = [
        Node(0, Kind("Input")),
        Node(1, Kind("Iterate", iterations=iterations, bailout=bailout, body=[2, 3, 4, 5, 6])),
        Node(2, Kind("BoxFold", limit=limit)),
        Node(3, Kind("Trap", slot=0, measure="Norm", scale=trap_scale)),
        Node(4, Kind("SphereFold", min_radius=min_radius, fixed_radius=fixed_radius)),
        Node(5, Kind("Scale", factor=scale)),
        Node(6, Kind("AddOrigin")),
        Node(7, Kind("NormFence", inset=0.0)),
        Node(8, Kind("Output")),
    ]
    return Graph(nodes, _chain_links([(0, 1, 0), (1, 7, 0), (7, 8, 0)]), safety, hint)


def menger(scale=3.0, offset=(1.0, 1.0, 1.0), iterations=5, bailout=1.0e6, trap_scale=4.0,
           half=(1.0, 1.0, 1.0), safety=0.9, hint=4.464102):
    """graphs/menger.ron: Iterate{MengerFold, Trap} -> Box."""
    nodes = [
        Node(0, Kind("Input")),
        Node(1, Kind("Iterate", iterations=iterations, bailout=bailout, body=[2, 3])),
        Node(2, Kind("MengerFold", scale=scale, offset=list(offset))),
        Node(3, Kind("Trap", slot=0, measure="Norm", scale=trap_scale)),
        Node(4, Kind("Box", half=list(half))),
        Node(5, Kind("Output")),
    ]
    return Graph(nodes, _chain_links([(0, 1, 0), (1, 4, 0), (4, 5, 0)]), safety, hint)


def sphere(radius=1.0, ground=-1.0, safety=1.0, hint=100.0):
    """graphs/sphere.ron: Trap -> {Sphere, Plane} -> Union."""
    nodes = [
        Node(0, Kind("Input")),
        Node(1, Kind("Trap", slot=0, measure="Norm", scale=1.0)),
        Node(2, Kind("Sphere", radius=radius)),
        Node(3, Kind("Plane", normal=[0.0, 1.0, 0.0], offset=ground)),
        Node(4, Kind("Union")),
        Node(5, Kind("Output")),
    ]
    links = _chain_links([(0, 1, 0), (1, 2, 0), (1, 3, 0), (2, 4, 0), (3, 4, 1), (4, 5, 0)])
    return Graph(nodes, links, safety, hint)

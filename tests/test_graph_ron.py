"""RON reading, graph packing and the bundled graphs (CPU)."""
import numpy as np
import pytest

from helpers import FORMS, golden_graph
from syfrack_gb300 import abi, ron
from syfrack_gb300.graph import Graph


def test_ron_values():
    v = ron.loads('(a: 1, b: [1.5, -2e3], c: Some("x\\n"), d: None, e: Name(k: true), f: (1, 2), g: Unit)')
    assert v["a"] == 1 and v["b"] == [1.5, -2000.0] and v["c"] == "x\n" and v["d"] is None
    assert v["e"]["__name__"] == "Name" and v["e"]["k"] is True
    assert v["f"].items == [1, 2] and v["g"] == ron.Unit("Unit")


def test_ron_comments_and_trailing_commas():
    v = ron.loads("// header\n[\n (p: (1.0, 2.0, 3.0), x: 1,),  /* c */\n]\n")
    assert ron.vec(v[0]["p"]) == [1.0, 2.0, 3.0]


@pytest.mark.parametrize("name", FORMS)
def test_bundled_builders_match_reference_graphs(name):
    ref = golden_graph(name)
    mine = Graph.bundled(name)
    assert [n.id for n in mine.nodes] == [n.id for n in ref.nodes]
    for a, b in zip(mine.nodes, ref.nodes):
        assert a.kind.name == b.kind.name
        fa, ua = __import__("syfrack_gb300.graph", fromlist=["_pack_params"])._pack_params(a.kind)
        fb, ub = __import__("syfrack_gb300.graph", fromlist=["_pack_params"])._pack_params(b.kind)
        np.testing.assert_allclose(fa, fb, rtol=1e-6)
        assert ua == ub
    assert [(l.src, l.dst) for l in mine.links] == [(l.src, l.dst) for l in ref.links]
    assert mine.safety == pytest.approx(ref.safety)
    assert mine.bounding_radius_hint == pytest.approx(ref.bounding_radius_hint, rel=1e-6)


def test_desc_packing():
    g = Graph.bundled("mandelbox")
    d, keep = g.to_desc()
    assert d.node_count == 9 and d.link_count == 3 and d.body_id_count == 5
    it = d.nodes[1]
    assert it.kind == abi.KIND_ID["Iterate"] and it.u[0] == 12 and it.f[0] == 1000.0
    assert [d.body_ids[i] for i in range(it.body_offset, it.body_offset + it.body_len)] == [2, 3, 4, 5, 6]
    trap = d.nodes[3]
    assert trap.kind == abi.KIND_ID["Trap"] and list(trap.u) == [0, 0, 0] and trap.f[0] == 2.0

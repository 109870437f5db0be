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


def test_scene_reader_keeps_materials_lights_and_fog():
    """The scene files' material (finishes with their details, surface variation, a
    volumetric texture with its own graph), projector and tube lights, and fog reach
    the scene (scenes/eclosion-brume.ron, scenes/puits-des-eons.ron)."""
    from helpers import golden_scene
    from syfrack_gb300.scene import ProjectorLight, TubeLight

    s = golden_scene("eclosion-brume")
    kinds = [type(l).__name__ for l in s.lights]
    assert kinds == ["ProjectorLight", "ProjectorLight", "AreaLight", "AreaLight", "TubeLight", "TubeLight",
                     "EnvironmentLight"]
    p = s.lights[0]
    assert isinstance(p, ProjectorLight) and p.inner_angle < p.outer_angle
    assert isinstance(s.lights[4], TubeLight) and s.lights[4].radius > 0
    assert len(s.material.finishes) == 8 and sum(f.detail is not None for f in s.material.finishes) == 4
    assert s.material.finishes[0].detail.pattern == "BrushedMetal"
    assert s.fog is not None and s.fog.density > 0 and s.cavity_darkness > 0
    s = golden_scene("puits-des-eons")
    t = s.material.texture
    assert t is not None and t.channel == ("trap", 0) and len(t.graph.nodes) > 3
    assert t.graph.validate()["op_count"] > 0
    assert s.material.surface is not None and s.material.coloring is not None
    d = golden_scene("eclosion-brume").desc(64, 36)
    assert d.light_count == 7 and d.finish_count == 8 and sum(d.details[i].pattern > 0 for i in range(8)) == 4
    assert [d.lights[i].kind for i in range(7)] == [4, 4, 0, 0, 5, 5, 2]


def test_creation_scenes_are_refused():
    from syfrack_gb300.scene import scene_from_ron_value

    with pytest.raises(ValueError, match="creation"):
        scene_from_ron_value({"creation": {}, "camera": {}, "lights": [], "material": {}})

"""The interactive preview machine (ControlSession, control/mod.rs:172-530 and
control.wgsl:54-303) on the GPU: primary rays on the exact field with no step
budget, in resumable quanta (the image does not depend on the quantum), the fixed
preview shading, tick() that never waits, pick(), and edits that upload data and
restart without compiling anything (an edited preview equals a fresh one)."""
import time

import numpy as np
import pytest

from syfrack_gb300 import PreviewSession, workloads
from syfrack_gb300.graph import Graph
from syfrack_gb300.scene import Scene

pytestmark = pytest.mark.gpu
LIGHT = np.array([0.4, 0.7, 0.6]) / np.linalg.norm([0.4, 0.7, 0.6])


def bulb_scene(power=8.0):
    _, cam, *_ = workloads.mandelbulb_primary()
    g = Graph.bundled("mandelbulb", power=power, iterations=12, bailout=2.0, safety=0.7, hint=2.5)
    return Scene(graph=g, camera=cam)


def test_preview_against_the_oracle_march(renderer, oracle_mod):
    scene = bulb_scene()
    w = h = 128
    p = PreviewSession(renderer, scene, (w, h))
    p.wait_complete()
    img = p.readback()
    assert p.progress()["completed_pixels"] == w * h
    sd = scene.desc(w, h)
    ref = oracle_mod.OracleGraph(scene.graph).primary(sd.camera, w, h, 1 << 20, 0, 1e-4, 200.0, 1.0, 1,
                                                      precision=32)
    depth = img["depth"].reshape(-1)
    hit_p, hit_r = depth >= 0, ref["t"] >= 0
    assert (hit_p == hit_r).mean() >= 0.995 and hit_p.mean() > 0.2
    both = hit_p & hit_r
    assert (np.abs(depth[both] - ref["t"][both]) <= 1e-4 * ref["t"][both]).mean() >= 0.99
    aux = img["aux"].reshape(-1, 4)
    steps = aux[:, 3].astype(np.int64)
    assert (steps[both] == ref["steps"][both].astype(np.int64) - 1).mean() >= 0.9
    dots = (aux[both, :3] * ref["normal"][both]).sum(1)
    assert (dots >= 0.99985).mean() >= 0.98
    color = img["accum"].reshape(-1, 4)
    expect = np.array([0.68, 0.70, 0.73]) * (0.2 + 0.8 * np.maximum(ref["normal"] @ LIGHT, 0.0))[:, None]
    assert (np.abs(color[both, :3] - expect[both]).max(1) <= 2e-3).mean() >= 0.98
    assert np.all(color[~hit_p & ~hit_r, :3] == np.array([0.025, 0.035, 0.05], np.float32))
    # pick reads the same pixel
    u, v = 0.5, 0.5
    d = p.pick(u, v)
    assert d is not None and d[0] == img["depth"][int(v * h), int(u * w)]
    assert d[1] == list(img["aux"][int(v * h), int(u * w)])
    assert p.pick(0.0, 0.0) is None  # the corner sees the background
    p.close()


def test_quanta_do_not_change_the_image_and_tick_never_waits(renderer):
    scene = bulb_scene()
    a = PreviewSession(renderer, scene, (96, 96), quantum=1)
    t_max = 0.0
    ticks = 0
    while True:
        t0 = time.perf_counter()
        done = a.tick()
        t_max = max(t_max, time.perf_counter() - t0)
        ticks += 1
        if done:
            break
        assert ticks < 2_000_000
    assert a.progress()["dispatches"] > 20  # one DE evaluation per pixel per quantum
    assert t_max < 0.05  # polls and submits, never waits for the device
    b = PreviewSession(renderer, scene, (96, 96), quantum=4096)
    b.wait_complete()
    ia, ib = a.readback(), b.readback()
    for k in ("accum", "depth", "aux"):
        np.testing.assert_array_equal(ia[k], ib[k], err_msg=k)
    assert b.progress()["dispatches"] < a.progress()["dispatches"]
    a.close()
    b.close()


def test_edits_restart_without_compiling(renderer):
    p = PreviewSession(renderer, bulb_scene(8.0), (96, 96))
    p.wait_complete()
    eight = p.readback()
    p.update_graph(bulb_scene(6.0).graph)  # a value edit: same topology (graph/mod.rs:397-425)
    assert p.progress()["completed_pixels"] == 0
    p.wait_complete()
    six = p.readback()
    fresh = PreviewSession(renderer, bulb_scene(6.0), (96, 96))
    fresh.wait_complete()
    np.testing.assert_array_equal(six["accum"], fresh.readback()["accum"])
    assert np.abs(six["accum"] - eight["accum"]).max() > 0.05
    # another graph altogether: also data, the image restarts
    p.set_scene(Scene(graph=Graph.bundled("menger"), camera=bulb_scene().camera))
    p.wait_complete()
    assert (p.readback()["depth"] >= 0).mean() > 0.1
    p.close()
    fresh.close()

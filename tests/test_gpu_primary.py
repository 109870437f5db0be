"""Primary-ray sphere trace (t, steps, normal) against the FP64 oracle on all
65,536 pixels of the 256x256 Mandelbulb workload (GPU).

Tolerances: hit/miss classification equal on >= 99.5% of pixels; on common
hits |dt| <= 1e-3 * t for >= 99%; normals within 1 degree (dot >= 0.99985) for
>= 98%; step counts equal for >= 90% and within 2 for >= 99%."""
import numpy as np
import pytest

from syfrack_gb300 import workloads
from syfrack_gb300.scene import Scene

pytestmark = pytest.mark.gpu


def _camera_desc(cam, w, h):
    sd = Scene(graph=None, camera=cam).desc(w, h)
    return sd.camera


@pytest.mark.parametrize("rule", ["absolute", "cone"])
def test_primary_against_fp64_oracle(renderer, oracle_mod, rule):
    g, cam, w, h, steps, eps, far = workloads.mandelbulb_primary()
    gpu = renderer.primary(g, cam, w, h, max_steps=steps, rule=rule, eps=eps, t_far=far, normal="central")
    ref = oracle_mod.OracleGraph(g).primary(_camera_desc(cam, w, h), w, h, steps, 1 if rule == "absolute" else 0,
                                            eps, far, 1.0, 0, precision=64)
    hit_g, hit_r = gpu["t"] >= 0, ref["t"] >= 0
    assert (hit_g == hit_r).mean() >= 0.995
    both = hit_g & hit_r
    assert both.sum() > 10000
    dt = np.abs(gpu["t"][both] - ref["t"][both]) / ref["t"][both]
    assert (dt <= 1e-3).mean() >= 0.99
    dots = (gpu["normal"][both] * ref["normal"][both]).sum(1)
    assert (dots >= 0.99985).mean() >= 0.98
    ds = np.abs(gpu["steps"].astype(np.int64) - ref["steps"].astype(np.int64))
    assert (ds == 0).mean() >= 0.90 and (ds <= 2).mean() >= 0.99


def test_primary_tetrahedral_normals_are_unit(renderer):
    g, cam, w, h, steps, eps, far = workloads.mandelbulb_primary()
    gpu = renderer.primary(g, cam, 64, 64, max_steps=steps, rule="absolute", eps=eps, t_far=far,
                           normal="tetrahedral")
    hit = gpu["t"] >= 0
    assert hit.sum() > 500
    np.testing.assert_allclose(np.linalg.norm(gpu["normal"][hit], axis=1), 1.0, atol=1e-5)
    assert np.all(gpu["normal"][~hit] == 0)


@pytest.mark.parametrize("margin", [0.05, 10.0])
def test_primary_with_skippable_bound(renderer, oracle_mod, margin):
    """A Bounded branch the GPU skips outside its margin (graph_wgsl.rs:800-814): the
    march steps by the box bound, re-evaluates exactly within five hit cones
    (pathtrace.wgsl:100-106) and never accepts a flagged sample. The device follows
    the f32 oracle's march; margin 10 never skips inside the view."""
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from helpers import bounded_bulb

    _, cam, w, h, steps, eps, far = workloads.mandelbulb_primary()
    g = bounded_bulb(margin=margin)
    w = h = 128
    gpu = renderer.primary(g, cam, w, h, max_steps=steps, rule="cone", eps=eps, t_far=far, normal="central")
    og = oracle_mod.OracleGraph(g)
    ref = og.primary(_camera_desc(cam, w, h), w, h, steps, 0, eps, far, 1.0, 0, precision=32)
    hit_g, hit_r = gpu["t"] >= 0, ref["t"] >= 0
    assert (hit_g == hit_r).mean() >= 0.995
    both = hit_g & hit_r
    assert both.sum() > 2000
    assert (np.abs(gpu["t"][both] - ref["t"][both]) <= 1e-4 * ref["t"][both]).mean() >= 0.99
    ds = np.abs(gpu["steps"].astype(np.int64) - ref["steps"].astype(np.int64))
    assert (ds == 0).mean() >= 0.95 and (ds <= 2).mean() >= 0.99
    if margin < 1.0:
        wide = renderer.primary(bounded_bulb(margin=10.0), cam, w, h, max_steps=steps, rule="cone", eps=eps,
                                t_far=far, normal="central")
        # stepping by the bound far from the box takes more (cheaper) steps
        assert gpu["steps"].sum() > wide["steps"].sum()
        assert ((gpu["t"] >= 0) == (wide["t"] >= 0)).mean() >= 0.995

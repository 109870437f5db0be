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

"""Tiled export on the GPU (crates/syfrack-render/tests/gpu_export.rs:67-282 restated):
a tiled export of clipped 16-pixel tiles equals the resident session (camera and RNG
in image coordinates, samples in ascending order: here bit for bit), holds far fewer
device bytes, resumes from a checkpoint to the uninterrupted image exactly, and
refuses a changed export.bin ("checksum")."""
import os

import numpy as np
import pytest

from syfrack_gb300 import ExportSession, RenderSession, SyfrackError, workloads
from syfrack_gb300.scene import RenderConfig

pytestmark = pytest.mark.gpu


def cfg(integrator="wavefront", w=263, h=251, spp=3, tile=16, spd=2):
    return RenderConfig(width=w, height=h, samples_per_pixel=spp, max_bounces=2, max_steps=512, pixel_tolerance=1.0,
                        tile_size=tile, samples_per_dispatch=spd, integrator=integrator)


def finish(s):
    while not s.step(20):
        pass


@pytest.mark.parametrize("integrator", ["wavefront", "megakernel"])
def test_tiles_match_the_resident_session(renderer, integrator):
    scene = workloads.mandelbox_scene()
    c = cfg(integrator)
    ref = RenderSession(renderer, scene, c)
    finish(ref)
    expected = ref.film_planes()
    ref.close()
    ex = ExportSession(renderer, scene, c)
    finish(ex)
    got = ex.film_planes()
    for k in ("accum", "depth", "aux", "volume", "moments", "surface"):
        np.testing.assert_array_equal(got[k], expected[k], err_msg=k)
    p = ex.progress()
    assert (p["samples_min"], p["samples_max"]) == (3, 3)
    # one tile-sized film and path arena on the device: less than the image's film alone
    assert 0 < ex.device_bytes() < 263 * 251 * 36
    ex.close()


def test_checkpoint_resumes_exactly_and_rejects_corruption(renderer, tmp_path):
    scene = workloads.mandelbox_scene()
    c = cfg()
    d = str(tmp_path / "render.state")
    s = ExportSession(renderer, scene, c)
    while s.progress()["samples_max"] == 0:
        s.step(0)
    part = s.progress()
    assert 0 < part["pixel_samples_done"] < part["pixel_samples_total"]
    s.save(d)
    s.close()
    restored = ExportSession.resume(renderer, scene, c, d)
    assert restored.progress()["pixel_samples_done"] == part["pixel_samples_done"]
    finish(restored)
    full = ExportSession(renderer, scene, c)
    finish(full)
    a, b = full.film_planes(), restored.film_planes()
    for k in ("accum", "depth", "aux"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    restored.save(d)
    restored.close()
    with open(os.path.join(d, "export.bin"), "r+b") as f:
        f.seek(7)
        byte = f.read(1)
        f.seek(7)
        f.write(bytes([byte[0] ^ 1]))
    with pytest.raises(SyfrackError) as e:
        ExportSession.resume(renderer, scene, c, d)
    assert "checksum" in str(e.value)
    full.close()


def test_uncommitted_tiles_keep_cleared_planes(renderer):
    scene = workloads.mandelbox_scene()
    s = ExportSession(renderer, scene, cfg(w=64, h=48, tile=16))
    s.step(0)  # one tile
    p = s.film_planes()
    counts = p["accum"][..., 3]
    assert set(np.unique(counts)) <= {0.0, 3.0}
    assert (counts == 3.0).sum() == 16 * 16
    assert np.all(p["depth"][counts == 0] == -1.0)
    s.close()


def test_fog_export_keeps_the_volume_planes(renderer, tmp_path):
    """A fog scene exported tile by tile (with a checkpoint taken mid-export) equals the
    resident session on every plane, the volume layer split included."""
    from test_fog import fog_bulb_scene

    scene = fog_bulb_scene()
    c = cfg(w=70, h=45, spp=4, tile=16, spd=2)
    ref = RenderSession(renderer, scene, c)
    finish(ref)
    expected = ref.film_planes()
    ref.close()
    assert expected["volume"][..., :3].max() > 0
    ex = ExportSession(renderer, scene, c)
    while ex.progress()["samples_max"] == 0:
        ex.step(0)
    d = str(tmp_path / "fog.state")
    ex.save(d)
    ex.close()
    ex = ExportSession.resume(renderer, scene, c, d)
    finish(ex)
    got = ex.film_planes()
    ex.close()
    for k in ("accum", "depth", "aux", "volume", "moments", "surface"):
        np.testing.assert_array_equal(got[k], expected[k], err_msg=k)

"""The allocation-free deep zoom against the allocating one (GPU).

sf_deep_zoom_noalloc exists for callers that cannot let a library call cudaMalloc
(hosts that own all device memory through their own pool, threads that cannot take
cudaMalloc's implicit synchronisation): it writes into the caller's device buffers
and keeps the reference orbit in a file-scope device array. This test allocates the
output buffers itself (with torch), calls the entry point through the C ABI twice in
a row with different views -- the second call finds the first call's orbit still in
the shared array -- and requires the same iteration counts and smooth values as
sf_deep_zoom. It runs alone or after the other tests; the file name keeps it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

VIEWS = [
    # centre, width, image, max_iter
    ((-0.743, 0.131), 1e-3, 160, 90, 3000),
    ((0.27868532354762443, 0.5820921261345181), 1e-12, 128, 72, 20000),
]


def _desc(center, width, w, h, max_iter):
    from syfrack_gb300._lib import sf_deep_zoom_desc

    d = sf_deep_zoom_desc()
    d.center_hi[:] = list(center)
    d.center_lo[:] = [0.0, 0.0]
    d.width_units, d.width, d.height, d.max_iter, d.bailout = width, w, h, max_iter, 16.0
    return d


def test_noalloc_matches_allocating_entry_point(gpu_ctx):
    import torch

    from syfrack_gb300 import deep_zoom
    from syfrack_gb300._lib import check, load

    lib = load()
    for center, width, w, h, max_iter in VIEWS:
        ref = deep_zoom(gpu_ctx, center, (0.0, 0.0), width, w, h, max_iter, bailout=16.0)
        it = torch.empty(w * h, dtype=torch.int32, device="cuda")
        sm = torch.empty(w * h, dtype=torch.float32, device="cuda")
        stream = torch.cuda.current_stream()
        check(lib.sf_deep_zoom_noalloc(C.byref(_desc(center, width, w, h, max_iter)), C.c_void_p(it.data_ptr()),
                                       C.c_void_p(sm.data_ptr()), C.c_void_p(stream.cuda_stream)))
        stream.synchronize()
        got_it = it.cpu().numpy().view(np.uint32).reshape(h, w)
        got_sm = sm.cpu().numpy().reshape(h, w)
        np.testing.assert_array_equal(got_it, ref["iterations"])
        np.testing.assert_array_equal(got_sm, ref["smooth"])
        assert got_it.min() < max_iter  # the view is not empty


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu_ctx):
    import torch

    from syfrack_gb300._lib import SyfrackError, check, load

    lib = load()
    it = torch.empty(16, dtype=torch.int32, device="cuda")
    sm = torch.empty(16, dtype=torch.float32, device="cuda")
    with pytest.raises(SyfrackError) as e:
        check(lib.sf_deep_zoom_noalloc(C.byref(_desc((0.0, 0.0), 1.0, 4, 4, 65537)), C.c_void_p(it.data_ptr()),
                                       C.c_void_p(sm.data_ptr()), None))
    assert e.value.status == 1 and "65536" in str(e.value)

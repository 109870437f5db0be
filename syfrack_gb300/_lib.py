"""Loads libsyfrack_gpu.so (built in-tree by syfrack_gb300.build) and declares
the C ABI of include/syfrack_gpu.h for ctypes. There is no fallback: if the
library is missing or no CUDA device is usable, calls raise SyfrackError."""
from __future__ import annotations

import ctypes as C
import os

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsyfrack_gpu.so")


class SyfrackError(RuntimeError):
    def __init__(self, status: int, message: str):
        self.status = status
        name = abi.STATUS_NAMES.get(status, f"status {status}")
        super().__init__(f"{name}: {message}" if message else name)


_lib = None

P = C.POINTER
vp = C.c_void_p
st = C.c_int32
u32 = C.c_uint32
u64 = C.c_uint64
fp = P(C.c_float)
up = P(C.c_uint32)


class sf_primary_desc(C.Structure):
    _fields_ = [("camera", abi.sf_camera), ("width", u32), ("height", u32), ("max_steps", u32),
                ("rule", C.c_int32), ("normal_mode", C.c_int32), ("eps", C.c_float), ("t_far", C.c_float),
                ("pixel_tolerance", C.c_float)]


class sf_stats(C.Structure):
    _fields_ = [("de_evals", u64), ("de_iterations", u64), ("segments", u64), ("shadow_segments", u64),
                ("steps", u64), ("launches", u64), ("kernel_ms", C.c_double), ("trace_ms", C.c_double),
                ("trace_launches", u64), ("warp_de_calls", u64), ("iteration_slots", u64),
                ("warp_cycles", u64), ("tail_cycles", u64)]


class sf_progress(C.Structure):
    _fields_ = [("tiles", u32), ("dispatches", u32), ("samples_min", u32), ("samples_max", u32),
                ("target", u32), ("pixel_samples_done", u64), ("pixel_samples_total", u64),
                ("status_word", u32)]


class sf_film_planes(C.Structure):
    _fields_ = [("accum", fp), ("depth", fp), ("aux", fp), ("volume", fp), ("moments", fp), ("surface", fp),
                ("color", fp)]


class sf_planar_desc(C.Structure):
    _fields_ = [("family", u32), ("power", u32), ("iterations", u32), ("julia", C.c_float * 2),
                ("center", C.c_float * 2), ("zoom", C.c_float), ("angle", C.c_float),
                ("inversion", C.c_float), ("twist", C.c_float), ("relaxation", C.c_float),
                ("memory", C.c_float), ("bailout", C.c_float), ("trap_radius", C.c_float),
                ("stripes", C.c_float)]


class sf_canvas(C.Structure):
    _fields_ = [("center", C.c_float * 2), ("zoom", C.c_float), ("rotation_deg", C.c_float),
                ("width", u32), ("height", u32), ("seed", u64)]


class sf_batch_job(C.Structure):
    _fields_ = [("graph", vp), ("scene", abi.sf_scene_desc), ("cfg", abi.sf_render_config)]


class sf_deep_zoom_desc(C.Structure):
    _fields_ = [("center_hi", C.c_double * 2), ("center_lo", C.c_double * 2), ("width_units", C.c_double),
                ("width", u32), ("height", u32), ("max_iter", u32), ("bailout", C.c_float),
                ("orbit_mode", u32), ("orbit_len", u32), ("orbit", fp)]


class sf_server_config(C.Structure):
    _fields_ = [("hbm_budget", u64), ("host_result_bytes", u64), ("slots", u32), ("path_capacity", u32),
                ("max_jobs", u32), ("max_tile_pixels", u32), ("min_blocks", u32), ("quantum", u32),
                ("regen", u32), ("pad", u32)]


class sf_request(C.Structure):
    _fields_ = [("kind", u32), ("samples", u32), ("parent", u64), ("graph", vp), ("scene", abi.sf_scene_desc),
                ("cfg", abi.sf_render_config), ("planar", sf_planar_desc), ("canvas", sf_canvas),
                ("tile_outputs", u32), ("pad", u32)]


class sf_result(C.Structure):
    _fields_ = [("state", u32), ("status", st), ("kind", u32), ("width", u32), ("height", u32),
                ("samples", u32), ("batch_requests", u32), ("pad", u32), ("work", u64),
                ("submit_ms", C.c_double), ("start_ms", C.c_double), ("done_ms", C.c_double),
                ("accum", fp), ("iterations", up), ("smooth", fp), ("distance", fp), ("traps", fp)]


class sf_server_stats(C.Structure):
    _fields_ = [("submitted", u64), ("completed", u64), ("failed", u64), ("batches", u64),
                ("batched_requests", u64), ("admission_waits", u64), ("hbm_used", u64), ("hbm_peak", u64),
                ("hbm_reserved", u64), ("host_used", u64), ("launches", u64), ("now_ms", C.c_double)]


# name -> (argtypes); every function returns sf_status unless listed in _RESTYPES
SIGNATURES = {
    "sf_status_string": [st],
    "sf_last_error": [],
    "sf_abi_version": [],
    "sf_context_create": [C.c_int, u64, P(vp)],
    "sf_context_destroy": [vp],
    "sf_context_stream": [vp, P(vp)],
    "sf_context_memory": [vp, P(u64), P(u64)],
    "sf_context_set_profiling": [vp, C.c_int],
    "sf_context_stats": [vp, P(sf_stats)],
    "sf_context_reset_stats": [vp],
    "sf_context_sync": [vp, u32],
    "sf_device_fp32_peak": [vp, P(C.c_double)],
    "sf_graph_validate": [P(abi.sf_graph_desc), P(abi.sf_graph_info)],
    "sf_environment_build": [fp, u32, u32, fp, up, up, P(C.c_int)],
    "sf_environment_create": [vp, fp, u32, u32, P(vp)],
    "sf_environment_destroy": [vp],
    "sf_graph_compile": [vp, P(abi.sf_graph_desc), P(vp)],
    "sf_graph_info_get": [vp, P(abi.sf_graph_info)],
    "sf_graph_update": [vp, P(abi.sf_graph_desc)],
    "sf_graph_destroy": [vp],
    "sf_de_probe": [vp, fp, C.c_size_t, P(abi.sf_de_sample)],
    "sf_de_probe_device": [vp, vp, vp, vp, C.c_size_t, vp, vp, vp, vp],
    "sf_primary_trace": [vp, P(sf_primary_desc), fp, up, fp],
    "sf_session_create": [vp, vp, P(abi.sf_scene_desc), P(abi.sf_render_config), P(vp)],
    "sf_session_dispatch": [vp, abi.sf_tile, u32],
    "sf_session_step": [vp, u32, P(C.c_int)],
    "sf_session_sync": [vp, u32, up],
    "sf_session_progress": [vp, P(sf_progress)],
    "sf_session_tiles": [vp, P(abi.sf_tile), u32, up],
    "sf_session_readback": [vp, P(sf_film_planes)],
    "sf_session_stats": [vp, P(sf_stats)],
    "sf_session_save": [vp, C.c_char_p],
    "sf_session_resume": [vp, vp, C.c_char_p, P(vp)],
    "sf_session_destroy": [vp],
    "sf_session_set_launch": [vp, u32, u32, u32],
    "sf_batch_create": [vp, P(sf_batch_job), u32, P(vp)],
    "sf_batch_set_launch": [vp, u32, u32, u32],
    "sf_batch_autotune": [vp, up, up, up, P(C.c_float)],
    "sf_batch_run": [vp, u32, C.c_int],
    "sf_batch_sync": [vp, u32, up],
    "sf_batch_readback": [vp, u32, P(sf_film_planes)],
    "sf_batch_destroy": [vp],
    "sf_planar_probe": [vp, P(sf_planar_desc), fp, C.c_size_t, fp, fp, up],
    "sf_escape2d": [vp, P(sf_planar_desc), P(sf_canvas), abi.sf_tile, u32, fp, fp, up],
    "sf_deep_zoom": [vp, P(sf_deep_zoom_desc), up, fp, C.c_int, up, fp, P(u64)],
    "sf_deep_zoom_noalloc": [P(sf_deep_zoom_desc), vp, vp, vp],
    "sf_server_create": [vp, P(sf_server_config), P(vp)],
    "sf_serve_submit": [vp, P(sf_request), P(u64)],
    "sf_serve_poll": [vp, u64, P(sf_result)],
    "sf_serve_wait": [vp, u64, u32, P(sf_result)],
    "sf_serve_release": [vp, u64],
    "sf_server_stats_get": [vp, P(sf_server_stats)],
    "sf_server_destroy": [vp],
    "sf_export_create": [vp, vp, P(abi.sf_scene_desc), P(abi.sf_render_config), P(vp)],
    "sf_export_step": [vp, u32, P(C.c_int)],
    "sf_export_progress": [vp, P(sf_progress)],
    "sf_export_readback": [vp, P(sf_film_planes)],
    "sf_export_save": [vp, C.c_char_p],
    "sf_export_resume": [vp, vp, C.c_char_p, P(vp)],
    "sf_export_device_bytes": [vp, P(u64)],
    "sf_export_destroy": [vp],
    "sf_preview_create": [vp, vp, P(abi.sf_scene_desc), u32, u32, u32, P(vp)],
    "sf_preview_set": [vp, vp, P(abi.sf_scene_desc)],
    "sf_preview_tick": [vp, P(C.c_int)],
    "sf_preview_wait": [vp, u32],
    "sf_preview_progress": [vp, up, up],
    "sf_preview_readback": [vp, P(sf_film_planes)],
    "sf_preview_pick": [vp, C.c_float, C.c_float, fp, fp],
    "sf_preview_destroy": [vp],
}
_RESTYPES = {"sf_status_string": C.c_char_p, "sf_last_error": C.c_char_p, "sf_abi_version": u32}


def load(build_if_missing: bool = True):
    """Returns the loaded library; builds it in-tree first if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise SyfrackError(11, f"{LIB_PATH} is not built")
        from . import build
        build.build()
    lib = C.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, st)
    _lib = lib
    return lib


def check(status: int):
    if status != 0:
        msg = load().sf_last_error()
        raise SyfrackError(status, msg.decode() if msg else "")

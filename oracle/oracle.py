"""TEST INFRASTRUCTURE -- NOT THE PRODUCT.

ctypes wrapper of liboracle.so, the CPU restatement of SyFrack's DE, sphere
trace, path tracer subset and escape-time sampler (oracle_core.cpp). Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "liboracle.so")
SOURCES = ["oracle_core.cpp", "oracle_api.cpp"]

sys.path.insert(0, ROOT)
from syfrack_gb300 import abi  # noqa: E402


def build(force: bool = False) -> str:
    """Compiles liboracle.so with strict binary32 semantics (no FP contraction)."""
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    hdrs = [os.path.join(HERE, "oracle_core.hpp"), os.path.join(ROOT, "include", "syfrack_gpu.h")]
    if not force and os.path.exists(LIB_PATH):
        t = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(p) <= t for p in srcs + hdrs):
            return LIB_PATH
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-pthread", *srcs, "-o", LIB_PATH + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


class PlanarParams(C.Structure):
    _fields_ = [("family", C.c_uint32), ("power", C.c_uint32), ("iterations", C.c_uint32),
                ("julia", C.c_double * 2), ("center", C.c_double * 2),
                ("zoom", C.c_double), ("angle", C.c_double), ("inversion", C.c_double),
                ("twist", C.c_double), ("relaxation", C.c_double), ("memory", C.c_double),
                ("bailout", C.c_double), ("trap_radius", C.c_double), ("stripes", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.or_graph_new.restype = C.c_void_p
        L.or_graph_new.argtypes = [C.POINTER(abi.sf_graph_desc)]
        L.or_graph_free.argtypes = [C.c_void_p]
        L.or_graph_info.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                    C.POINTER(C.c_float), C.POINTER(C.c_uint32)]
        dp = C.POINTER(C.c_double)
        up = C.POINTER(C.c_uint32)
        L.or_de_eval.argtypes = [C.c_void_p, C.c_int, dp, C.c_size_t, dp, dp, up, up, C.c_int]
        L.or_de_eval_fast.argtypes = [C.c_void_p, C.c_int, dp, C.c_size_t, dp, up, C.c_int]
        L.or_de_eval_search.argtypes = [C.c_void_p, C.c_int, dp, C.c_size_t, dp, dp, up, up, up, C.c_int]
        L.or_union_leaves.argtypes = [C.c_void_p, up]
        L.or_union_leaves.restype = C.c_uint32
        L.or_panorama.argtypes = [C.c_uint64, C.POINTER(C.c_float), C.c_uint32, C.c_uint32, C.POINTER(C.c_float),
                                  up, up]
        L.or_panorama.restype = C.c_int
        L.or_bvh_build.argtypes = [C.POINTER(abi.sf_placement), C.c_uint32, C.POINTER(C.c_float),
                                   C.POINTER(C.c_float)]
        L.or_primary.restype = C.c_uint64
        L.or_primary.argtypes = [C.c_void_p, C.c_int, C.POINTER(abi.sf_camera), C.c_uint32, C.c_uint32,
                                 C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, C.c_double, C.c_double,
                                 C.c_double, C.c_int, dp, up, dp, C.c_int]
        L.or_render.restype = C.c_uint64
        L.or_render.argtypes = [C.c_void_p, C.c_int, C.POINTER(abi.sf_scene_desc),
                                C.POINTER(abi.sf_render_config), up, C.c_size_t, C.c_uint32, C.c_uint32,
                                dp, dp, dp, C.POINTER(C.c_uint64), C.c_int, dp, dp, dp]
        L.or_planar.argtypes = [C.c_int, C.POINTER(PlanarParams), dp, C.c_size_t, dp, dp, up, C.c_int]
        L.or_mandel_escape.argtypes = [C.c_int, dp, dp, dp, C.c_size_t, C.c_uint32, C.c_double, up, dp,
                                       C.c_int]
        L.or_mandel_orbit.restype = C.c_uint32
        L.or_mandel_orbit.argtypes = [C.c_int, C.c_double, C.c_double, C.c_uint32, C.c_double,
                                      C.POINTER(C.c_float)]
        L.or_mandel_escapes.restype = C.c_int
        L.or_mandel_escapes.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                        C.c_uint32]
        L.or_texture_values.argtypes = [C.POINTER(abi.sf_scene_desc), C.c_int, dp, C.c_size_t, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _up(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


def panorama(rgb, key=0):
    """The oracle's panorama tables (environment.rs:271-366): texels[h, w, 4]; with a key
    (a Panorama handle value) scenes whose HDRI light carries it render with them."""
    rgb = np.ascontiguousarray(rgb, dtype=np.float32)
    h, w = rgb.shape[:2]
    fpp = C.POINTER(C.c_float)
    ow, oh = C.c_uint32(), C.c_uint32()
    if not lib().or_panorama(0, rgb.ctypes.data_as(fpp), w, h, None, C.byref(ow), C.byref(oh)):
        raise ValueError("invalid panorama")
    out = np.zeros((oh.value, ow.value, 4), np.float32)
    lib().or_panorama(key, rgb.ctypes.data_as(fpp), w, h, out.ctypes.data_as(fpp), C.byref(ow), C.byref(oh))
    return out


def bvh_build(placements, half):
    """The fence hierarchy of bvh.rs:26-102: (2n-1, 8) float32 rows (centre, half,
    escape, placement or -1)."""
    n = len(placements)
    pl = (abi.sf_placement * n)()
    for i, (pos, ang, sc) in enumerate(placements):
        pl[i].position[:] = pos
        pl[i].angles[:] = ang
        pl[i].scale[:] = sc
    h = (C.c_float * 3)(*half)
    out = np.zeros((2 * n - 1, 8), np.float32)
    lib().or_bvh_build(pl, n, h, out.ctypes.data_as(C.POINTER(C.c_float)))
    return out


class OracleGraph:
    def __init__(self, graph):
        desc, self._keep = graph.to_desc()
        self._desc = desc
        self.h = lib().or_graph_new(C.byref(desc))
        if not self.h:
            raise ValueError("graph rejected by the oracle (cycle)")

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_graph_free(self.h)
            self.h = None

    def info(self):
        ss, lp = C.c_float(), C.c_float()
        ts = (C.c_float * 4)()
        ip = C.c_uint32()
        lib().or_graph_info(self.h, C.byref(ss), C.byref(lp), ts, C.byref(ip))
        return {"step_scale": ss.value, "lipschitz": lp.value, "trap_scales": list(ts),
                "iteration_product": ip.value}

    def de(self, points, precision=64, threads=None):
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        n = len(pts)
        dist = np.zeros(n)
        traps = np.zeros((n, 4))
        iters = np.zeros(n, dtype=np.uint32)
        mats = np.zeros(n, dtype=np.uint32)
        lib().or_de_eval(self.h, precision, _dp(pts), n, _dp(dist), _dp(traps), _up(iters), _up(mats),
                         threads or default_threads())
        return {"distance": dist, "traps": traps, "iterations": iters, "material": mats}

    def de_search(self, points, precision=64, threads=None):
        """The exact sample through the union search (graph_wgsl.rs:1112-1154): the
        leaves probed for their bounds, then evaluated exactly while a bound can beat
        the best; the same fields as de(), and per point the leaves evaluated exactly
        after the probes."""
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        n = len(pts)
        dist = np.zeros(n)
        traps = np.zeros((n, 4))
        iters = np.zeros(n, dtype=np.uint32)
        mats = np.zeros(n, dtype=np.uint32)
        exact = np.zeros(n, dtype=np.uint32)
        lib().or_de_eval_search(self.h, precision, _dp(pts), n, _dp(dist), _dp(traps), _up(iters), _up(mats),
                                _up(exact), threads or default_threads())
        return {"distance": dist, "traps": traps, "iterations": iters, "material": mats, "exact_leaves": exact}

    def union_leaves(self):
        """(leaves of the union search, whether the graph has a skippable node)."""
        fast = C.c_uint32()
        n = lib().or_union_leaves(self.h, C.byref(fast))
        return int(n), bool(fast.value)

    def de_fast(self, points, precision=64, threads=None):
        """The GPU's march sample: skippable Bounded branches outside their margin
        give their bound with flags = 1 (graph_wgsl.rs:800-814)."""
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        n = len(pts)
        dist = np.zeros(n)
        flags = np.zeros(n, dtype=np.uint32)
        lib().or_de_eval_fast(self.h, precision, _dp(pts), n, _dp(dist), _up(flags), threads or default_threads())
        return {"distance": dist, "flags": flags}

    def primary(self, camera: abi.sf_camera, width, height, max_steps, rule, eps, t_far, tol=1.0,
                normal_mode=0, precision=64, first=0, count=None, threads=None):
        count = width * height - first if count is None else count
        n = width * height
        t = np.full(n, np.nan)
        steps = np.zeros(n, dtype=np.uint32)
        nrm = np.zeros((n, 3))
        evals = lib().or_primary(self.h, precision, C.byref(camera), width, height, first, count,
                                 max_steps, rule, eps, t_far, tol, normal_mode, _dp(t), _up(steps),
                                 _dp(nrm), threads or default_threads())
        return {"t": t, "steps": steps, "normal": nrm, "de_evals": int(evals)}

    def render(self, scene: abi.sf_scene_desc, cfg: abi.sf_render_config, pixels, sample_start,
               samples, precision=64, threads=None, planes=False):
        """Radiance sums of `samples` samples per pixel; planes=True adds the volume,
        moments and surface planes (sums and counts, each pixel's starting at zero)."""
        px = np.ascontiguousarray(pixels, dtype=np.uint32).reshape(-1, 2)
        n = len(px)
        accum = np.zeros((n, 3))
        depth = np.full(n, np.nan)
        aux = np.full((n, 4), np.nan)
        extra = {k: np.zeros((n, 4)) for k in ("volume", "moments", "surface")} if planes else {}
        evals = C.c_uint64()
        segs = lib().or_render(self.h, precision, C.byref(scene), C.byref(cfg), _up(px), n,
                               sample_start, samples, _dp(accum), _dp(depth), _dp(aux), C.byref(evals),
                               threads or default_threads(),
                               *((_dp(extra[k]) for k in ("volume", "moments", "surface")) if planes
                                 else (None, None, None)))
        return {"accum": accum, "depth": depth, "aux": aux, "segments": int(segs),
                "de_evals": int(evals.value), **extra}


def planar(params: PlanarParams, xy, precision=64, threads=None):
    pts = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
    n = len(pts)
    dist = np.zeros(n)
    traps = np.zeros((n, 4))
    iters = np.zeros(n, dtype=np.uint32)
    lib().or_planar(precision, C.byref(params), _dp(pts), n, _dp(dist), _dp(traps), _up(iters),
                    threads or default_threads())
    return {"distance": dist, "traps": traps, "iterations": iters}


def mandel_escape(center_hi, center_lo, offsets, max_iter, bailout=2.0, precision=64, threads=None):
    off = np.ascontiguousarray(offsets, dtype=np.float64).reshape(-1, 2)
    n = len(off)
    hi = np.ascontiguousarray(center_hi, dtype=np.float64)
    lo = np.ascontiguousarray(center_lo, dtype=np.float64)
    iters = np.zeros(n, dtype=np.uint32)
    mag2 = np.zeros(n)
    lib().or_mandel_escape(precision, _dp(hi), _dp(lo), _dp(off), n, max_iter, bailout, _up(iters),
                           _dp(mag2), threads or default_threads())
    return iters, mag2


def mandel_orbit(c_ref, max_iter, bailout=2.0, precision=128):
    """Reference orbit of c_ref as (n, 4) float32 rows (Re hi, Im hi, Re lo, Im lo),
    computed in binary128 (or binary64), through its escape or max_iter."""
    out = np.zeros((max_iter + 1, 4), np.float32)
    n = lib().or_mandel_orbit(precision, float(c_ref[0]), float(c_ref[1]), max_iter, bailout,
                              out.ctypes.data_as(C.POINTER(C.c_float)))
    return out[:n].copy()


def texture_values(scene_desc, texture_graph, points, precision=32):
    """pattern_value (pattern.wgsl:2-49) of the descriptor's texture at points[n, 3]; the
    texture's graph is given as an OracleGraph."""
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    scene_desc.texture.graph = texture_graph.h
    out = np.zeros(len(pts))
    lib().or_texture_values(C.byref(scene_desc), precision, _dp(pts), len(pts), _dp(out))
    return out

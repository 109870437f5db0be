"""Renderer API over the C ABI, mirroring crates/syfrack-render:
GpuContext (gpu.rs:15-36), Renderer::{probe_distances, render} (renderer.rs:645-693),
RenderSession::{new, step, progress, readback, save, resume} (session.rs:165-1346),
RenderOutput (renderer.rs:151-164), plus the escape-time sampler
(PlanarFractal::sample, syfrack-core/src/scene/planar.rs:77-194) and deep zoom.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass

import numpy as np

from . import abi
from ._lib import (SyfrackError, check, load, sf_canvas, sf_deep_zoom_desc, sf_film_planes,
                   sf_planar_desc, sf_primary_desc, sf_progress, sf_stats)
from .graph import Graph
from .scene import Camera, RenderConfig, Scene


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _up(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


@dataclass
class DeSample:
    """crates/syfrack-core/src/scene/fractal.rs:18-27."""
    distance: float
    traps: tuple
    iterations: int
    material: int


class GpuContext:
    """One CUDA device, its stream and HBM admission budget (bytes; 0 = 90% of free)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.sf_context_create(device, hbm_budget, C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.sf_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        check(self.lib.sf_context_stream(self.h, C.byref(s)))
        return s.value or 0

    def memory(self):
        used, budget = C.c_uint64(), C.c_uint64()
        check(self.lib.sf_context_memory(self.h, C.byref(used), C.byref(budget)))
        return used.value, budget.value

    def set_profiling(self, on, lane_stats: bool = False):
        """Per-kernel CUDA-event timing; lane_stats also counts the trace kernel's
        warp-level DE calls and iteration slots (a slower diagnostic kernel)."""
        check(self.lib.sf_context_set_profiling(self.h, (2 if lane_stats else 1) if on else 0))

    def stats(self) -> dict:
        s = sf_stats()
        check(self.lib.sf_context_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in sf_stats._fields_}

    def reset_stats(self):
        check(self.lib.sf_context_reset_stats(self.h))

    def sync(self, timeout_ms: int = 0):
        check(self.lib.sf_context_sync(self.h, timeout_ms))


class CompiledGraph:
    """A graph lowered to the device program (graph_wgsl::compile's counterpart)."""

    def __init__(self, ctx: GpuContext, graph: Graph):
        self.ctx = ctx
        self.graph = graph
        desc, keep = graph.to_desc()
        h = C.c_void_p()
        check(ctx.lib.sf_graph_compile(ctx.h, C.byref(desc), C.byref(h)))
        self.h = h

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.ctx.lib.sf_graph_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def info(self) -> dict:
        i = abi.sf_graph_info()
        check(self.ctx.lib.sf_graph_info_get(self.h, C.byref(i)))
        return {"step_scale": i.step_scale, "lipschitz": i.lipschitz, "trap_scales": list(i.trap_scales),
                "iteration_product": i.iteration_product, "form": abi.FORMS.get(i.form, i.form),
                "op_count": i.op_count, "bounding_radius_hint": i.bounding_radius_hint,
                "exact_union_leaves": i.exact_union_leaves}

    def update(self, graph: Graph):
        desc, keep = graph.to_desc()
        check(self.ctx.lib.sf_graph_update(self.h, C.byref(desc)))
        self.graph = graph
        cache = getattr(self, "_cache", None)
        if cache is not None:  # the renderer's cache now finds this handle under the new values
            if cache.get(self._key) is self:
                del cache[self._key]
            self._key = Renderer.cache_key(graph)
            cache.setdefault(self._key, self)

    def probe(self, points) -> dict:
        """Batched DE at points (n, 3) -> arrays distance, traps (n, 4), iterations, material."""
        pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        n = len(pts)
        out = (abi.sf_de_sample * max(n, 1))()
        check(self.ctx.lib.sf_de_probe(self.h, _fp(pts), n, out))
        arr = np.ctypeslib.as_array(out)[:n] if n else np.zeros(0)
        if n == 0:
            return {"distance": np.zeros(0, np.float32), "traps": np.zeros((0, 4), np.float32),
                    "iterations": np.zeros(0, np.uint32), "material": np.zeros(0, np.uint32)}
        return {"distance": np.array([s.distance for s in out[:n]], dtype=np.float32),
                "traps": np.array([list(s.traps) for s in out[:n]], dtype=np.float32),
                "iterations": np.array([s.iterations for s in out[:n]], dtype=np.uint32),
                "material": np.array([s.material for s in out[:n]], dtype=np.uint32)}


@dataclass
class RenderOutput:
    """RenderOutput (renderer.rs:151-164): mean radiance, first-hit depth and aux."""
    color: np.ndarray       # (h, w, 4) mean linear radiance, alpha 1
    accum: np.ndarray       # (h, w, 4) sample sums and counts
    depth: np.ndarray       # (h, w), -1 on a miss
    normals: np.ndarray     # (h, w, 4): normal xyz and march steps, (0,0,0,-1) on a miss
    samples_min: int
    samples_max: int
    elapsed: float


class Renderer:
    """Renderer (renderer.rs:328): a device context plus a cache of compiled graphs."""

    def __init__(self, ctx: GpuContext | None = None):
        self.ctx = ctx or GpuContext()
        self._cache: dict = {}

    @staticmethod
    def cache_key(graph: Graph):
        desc, keep = graph.to_desc()
        return (bytes(C.string_at(desc.nodes, C.sizeof(abi.sf_node) * desc.node_count)),
                bytes(C.string_at(desc.links, C.sizeof(abi.sf_link) * desc.link_count)),
                bytes(C.string_at(desc.body_ids, 4 * desc.body_id_count)),
                bytes(C.string_at(desc.placements, C.sizeof(abi.sf_placement) * desc.placement_count)),
                desc.safety, desc.bounding_radius_hint)

    def compile(self, graph: Graph) -> CompiledGraph:
        key = self.cache_key(graph)
        g = self._cache.get(key)
        if g is None:
            g = CompiledGraph(self.ctx, graph)
            g._cache, g._key = self._cache, key
            self._cache[key] = g
        return g

    def probe_distances(self, scene_or_graph, points) -> list:
        """Renderer::probe_distances (renderer.rs:645-648)."""
        graph = scene_or_graph.graph if isinstance(scene_or_graph, Scene) else scene_or_graph
        r = self.compile(graph).probe(points)
        return [DeSample(float(r["distance"][i]), tuple(float(x) for x in r["traps"][i]),
                         int(r["iterations"][i]), int(r["material"][i])) for i in range(len(r["distance"]))]

    def render(self, scene: Scene, cfg: RenderConfig, progress=None) -> RenderOutput:
        """Renderer::render (renderer.rs:668-693): a session stepped to completion."""
        s = RenderSession(self, scene, cfg)
        while not s.step(250):
            if progress:
                progress(s.progress())
        return s.readback()

    def primary(self, graph: Graph, camera: Camera, width: int, height: int, max_steps: int = 256,
                rule: str = "absolute", eps: float = 1e-4, t_far: float = 10.0, normal: str = "central",
                pixel_tolerance: float = 1.0) -> dict:
        """Primary-ray trace (t, steps, normal) through pixel centres."""
        g = self.compile(graph)
        b = camera.basis()
        d = sf_primary_desc()
        d.camera.origin[:] = [float(x) for x in b.origin]
        d.camera.forward[:] = [float(x) for x in b.forward]
        d.camera.right[:] = [float(x) for x in b.right]
        d.camera.up[:] = [float(x) for x in b.up]
        d.camera.tan_half_fov = b.tan_half_fov
        d.camera.aspect = float(np.float32(width) / np.float32(height))
        d.width, d.height, d.max_steps = width, height, max_steps
        d.rule = 1 if rule == "absolute" else 0
        d.normal_mode = 0 if normal == "central" else 1
        d.eps, d.t_far, d.pixel_tolerance = eps, t_far, pixel_tolerance
        n = width * height
        t = np.zeros(n, np.float32)
        steps = np.zeros(n, np.uint32)
        nrm = np.zeros((3, n), np.float32)
        check(self.ctx.lib.sf_primary_trace(g.h, C.byref(d), _fp(t), _up(steps), _fp(nrm)))
        return {"t": t, "steps": steps, "normal": nrm.T.copy()}


class RenderSession:
    """Progressive render over a tile grid (session.rs:113-877)."""

    def __init__(self, renderer: Renderer, scene: Scene, cfg: RenderConfig, _handle=None):
        self.renderer = renderer
        self.ctx = renderer.ctx
        self.scene = scene
        self.cfg = cfg
        self.graph = renderer.compile(scene.graph)
        tex = scene.material.texture
        # the texture's graph is compiled like the form's and kept alive with the session
        self.tex_graph = renderer.compile(tex.graph) if tex is not None else None
        self.t0 = time.perf_counter()
        if _handle is not None:
            self.h = _handle
            return
        sd = scene.desc(cfg.width, cfg.height, self.tex_graph.h.value if self.tex_graph else None)
        rc = cfg.desc()
        h = C.c_void_p()
        check(self.ctx.lib.sf_session_create(self.ctx.h, self.graph.h, C.byref(sd), C.byref(rc), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.sf_session_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_launch(self, min_blocks_per_sm: int = 7, quantum: int = 0, regen: int = 4):
        """Trace-kernel shape: resident blocks per SM (2-4 of 256 threads, or 6-7 of 128),
        step quantum, regeneration threshold (idle lanes a warp waits for before taking
        new segments)."""
        check(self.ctx.lib.sf_session_set_launch(self.h, min_blocks_per_sm, quantum, regen))

    def dispatch(self, tile, samples: int):
        """One tile, `samples` samples starting at tile.done; asynchronous."""
        t = tile if isinstance(tile, abi.sf_tile) else abi.sf_tile(*tile)
        check(self.ctx.lib.sf_session_dispatch(self.h, t, samples))

    def sync(self, timeout_ms: int = 10000) -> int:
        w = C.c_uint32()
        check(self.ctx.lib.sf_session_sync(self.h, timeout_ms, C.byref(w)))
        return w.value

    def step(self, budget_ms: int = 250) -> bool:
        done = C.c_int()
        check(self.ctx.lib.sf_session_step(self.h, budget_ms, C.byref(done)))
        return bool(done.value)

    def progress(self) -> dict:
        p = sf_progress()
        check(self.ctx.lib.sf_session_progress(self.h, C.byref(p)))
        return {k: getattr(p, k) for k, _ in sf_progress._fields_}

    def tiles(self) -> list:
        n = C.c_uint32()
        check(self.ctx.lib.sf_session_tiles(self.h, None, 0, C.byref(n)))
        arr = (abi.sf_tile * max(n.value, 1))()
        check(self.ctx.lib.sf_session_tiles(self.h, arr, n.value, C.byref(n)))
        return [(t.x, t.y, t.w, t.h, t.done) for t in arr[:n.value]]

    def readback(self) -> RenderOutput:
        w, h = self.cfg.width, self.cfg.height
        acc, aux, color = (np.empty((h, w, 4), np.float32) for _ in range(3))
        depth = np.empty((h, w), np.float32)
        # the library fills every plane, the mean colour included (pinned staging, host threads)
        planes = sf_film_planes(_fp(acc), _fp(depth), _fp(aux), None, None, None, _fp(color))
        check(self.ctx.lib.sf_session_readback(self.h, C.byref(planes)))
        p = self.progress()
        return RenderOutput(color, acc, depth, aux, p["samples_min"], p["samples_max"],
                            time.perf_counter() - self.t0)

    def film_planes(self) -> dict:
        """Every plane of the film (wf_commit's order): accum, depth, aux, volume,
        moments, surface."""
        w, h = self.cfg.width, self.cfg.height
        out = {k: np.zeros((h, w, 4), np.float32) for k in ("accum", "aux", "volume", "moments", "surface")}
        out["depth"] = np.zeros((h, w), np.float32)
        planes = sf_film_planes(*(_fp(out[k]) for k in ("accum", "depth", "aux", "volume", "moments", "surface")))
        check(self.ctx.lib.sf_session_readback(self.h, C.byref(planes)))
        return out

    def stats(self) -> dict:
        return self.ctx.stats()

    def save(self, directory: str):
        check(self.ctx.lib.sf_session_save(self.h, directory.encode()))

    @classmethod
    def resume(cls, renderer: Renderer, scene: Scene, cfg: RenderConfig, directory: str) -> "RenderSession":
        """RenderSession::resume (session.rs:1319): refuses corrupt or foreign checkpoints."""
        g = renderer.compile(scene.graph)
        h = C.c_void_p()
        check(renderer.ctx.lib.sf_session_resume(renderer.ctx.h, g.h, directory.encode(), C.byref(h)))
        return cls(renderer, scene, cfg, _handle=h)


class PreviewSession:
    """Interactive preview (ControlSession, control/mod.rs:172-530): primary rays on
    the exact field in resumable quanta, no step budget; tick() never waits; edits
    upload data and restart the image."""

    def __init__(self, renderer: Renderer, scene: Scene, size, quantum: int = 128):
        self.renderer = renderer
        self.ctx = renderer.ctx
        self.scene = scene
        self.size = (int(size[0]), int(size[1]))
        self.graph = renderer.compile(scene.graph)
        sd = scene.desc(*self.size)
        h = C.c_void_p()
        check(self.ctx.lib.sf_preview_create(self.ctx.h, self.graph.h, C.byref(sd), self.size[0], self.size[1],
                                             quantum, C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.sf_preview_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_scene(self, scene: Scene):
        """A new scene (graph and camera): uploaded, nothing compiled; the image restarts."""
        g = self.renderer.compile(scene.graph)
        sd = scene.desc(*self.size)
        check(self.ctx.lib.sf_preview_set(self.h, g.h, C.byref(sd)))
        self.scene, self.graph = scene, g

    def update_graph(self, graph):
        """A value edit of the current graph (same topology): sf_graph_update, then restart."""
        self.graph.update(graph)
        check(self.ctx.lib.sf_preview_set(self.h, None, None))

    def tick(self) -> bool:
        done = C.c_int()
        check(self.ctx.lib.sf_preview_tick(self.h, C.byref(done)))
        return bool(done.value)

    def wait_complete(self, timeout_ms: int = 120000):
        check(self.ctx.lib.sf_preview_wait(self.h, timeout_ms))

    def progress(self) -> dict:
        px, d = C.c_uint32(), C.c_uint32()
        check(self.ctx.lib.sf_preview_progress(self.h, C.byref(px), C.byref(d)))
        return {"completed_pixels": px.value, "dispatches": d.value}

    def readback(self) -> dict:
        w, h = self.size
        out = {"accum": np.zeros((h, w, 4), np.float32), "depth": np.zeros((h, w), np.float32),
               "aux": np.zeros((h, w, 4), np.float32)}
        planes = sf_film_planes(_fp(out["accum"]), _fp(out["depth"]), _fp(out["aux"]))
        check(self.ctx.lib.sf_preview_readback(self.h, C.byref(planes)))
        return out

    def pick(self, u: float, v: float):
        """(depth, aux) at (u, v) in [0, 1]^2, or None where nothing was hit."""
        d = C.c_float()
        a = (C.c_float * 4)()
        check(self.ctx.lib.sf_preview_pick(self.h, u, v, C.byref(d), a))
        return None if d.value <= 0.0 else (d.value, list(a))


class ExportSession:
    """Tiled export (ExportSession / TiledExport, export.rs:95-300, :830-900): the image
    in host memory, one tile-sized film on the device; tiles are committed whole."""

    def __init__(self, renderer: Renderer, scene: Scene, cfg: RenderConfig, _handle=None):
        self.renderer = renderer
        self.ctx = renderer.ctx
        self.scene = scene
        self.cfg = cfg
        self.graph = renderer.compile(scene.graph)
        tex = scene.material.texture
        # the texture's graph is compiled like the form's and kept alive with the session
        self.tex_graph = renderer.compile(tex.graph) if tex is not None else None
        self.t0 = time.perf_counter()
        if _handle is not None:
            self.h = _handle
            return
        sd = scene.desc(cfg.width, cfg.height, self.tex_graph.h.value if self.tex_graph else None)
        rc = cfg.desc()
        h = C.c_void_p()
        check(self.ctx.lib.sf_export_create(self.ctx.h, self.graph.h, C.byref(sd), C.byref(rc), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.sf_export_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, budget_ms: int = 250) -> bool:
        done = C.c_int()
        check(self.ctx.lib.sf_export_step(self.h, budget_ms, C.byref(done)))
        return bool(done.value)

    def progress(self) -> dict:
        p = sf_progress()
        check(self.ctx.lib.sf_export_progress(self.h, C.byref(p)))
        return {k: getattr(p, k) for k, _ in sf_progress._fields_}

    def device_bytes(self) -> int:
        n = C.c_uint64()
        check(self.ctx.lib.sf_export_device_bytes(self.h, C.byref(n)))
        return n.value

    def film_planes(self) -> dict:
        w, h = self.cfg.width, self.cfg.height
        out = {k: np.zeros((h, w, 4), np.float32) for k in ("accum", "aux", "volume", "moments", "surface")}
        out["depth"] = np.zeros((h, w), np.float32)
        planes = sf_film_planes(*(_fp(out[k]) for k in ("accum", "depth", "aux", "volume", "moments", "surface")))
        check(self.ctx.lib.sf_export_readback(self.h, C.byref(planes)))
        return out

    def readback(self) -> RenderOutput:
        p = self.film_planes()
        acc = p["accum"]
        color = np.ones_like(acc)
        color[..., :3] = acc[..., :3] / np.maximum(acc[..., 3:4], 1.0)
        pr = self.progress()
        return RenderOutput(color, acc, p["depth"], p["aux"], pr["samples_min"], pr["samples_max"],
                            time.perf_counter() - self.t0)

    def save(self, directory: str):
        check(self.ctx.lib.sf_export_save(self.h, directory.encode()))

    @classmethod
    def resume(cls, renderer: Renderer, scene: Scene, cfg: RenderConfig, directory: str) -> "ExportSession":
        """ExportSession::resume (export.rs:135-190): refuses a changed export.bin."""
        g = renderer.compile(scene.graph)
        h = C.c_void_p()
        check(renderer.ctx.lib.sf_export_resume(renderer.ctx.h, g.h, directory.encode(), C.byref(h)))
        return cls(renderer, scene, cfg, _handle=h)


class Batch:
    """Many (scene, config) jobs rendered by one wavefront (sf_batch_*): one set of
    persistent launches per round over all jobs' paths, captured in a CUDA graph."""

    def __init__(self, renderer: Renderer, jobs):
        from ._lib import sf_batch_job

        self.renderer = renderer
        self.ctx = renderer.ctx
        self.jobs = list(jobs)
        self._graphs = [renderer.compile(sc.graph) for sc, _ in self.jobs]
        # textured jobs: their texture graphs, compiled and kept alive with the batch
        self._tex = [renderer.compile(sc.material.texture.graph) if sc.material.texture else None
                     for sc, _ in self.jobs]
        arr = (sf_batch_job * len(self.jobs))()
        # the descriptors stay alive with the batch: a light list is referenced, not copied
        self._descs = [sc.desc(cfg.width, cfg.height, self._tex[i].h.value if self._tex[i] else None)
                       for i, (sc, cfg) in enumerate(self.jobs)]
        for i, (sc, cfg) in enumerate(self.jobs):
            arr[i].graph = self._graphs[i].h
            arr[i].scene = self._descs[i]
            arr[i].cfg = cfg.desc()
        h = C.c_void_p()
        check(self.ctx.lib.sf_batch_create(self.ctx.h, arr, len(self.jobs), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.sf_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_launch(self, min_blocks_per_sm: int = 3, quantum: int = 128, regen: int = 4):
        check(self.ctx.lib.sf_batch_set_launch(self.h, min_blocks_per_sm, quantum, regen))

    def autotune(self):
        """Returns (min_blocks_per_sm, quantum, regen, best pass ms)."""
        mb, q, rg, ms = C.c_uint32(), C.c_uint32(), C.c_uint32(), C.c_float()
        check(self.ctx.lib.sf_batch_autotune(self.h, C.byref(mb), C.byref(q), C.byref(rg), C.byref(ms)))
        return mb.value, q.value, rg.value, ms.value

    def run(self, passes: int = 1, use_graph: bool = True):
        check(self.ctx.lib.sf_batch_run(self.h, passes, 1 if use_graph else 0))

    def sync(self, timeout_ms: int = 60000) -> int:
        w = C.c_uint32()
        check(self.ctx.lib.sf_batch_sync(self.h, timeout_ms, C.byref(w)))
        return w.value

    def readback(self, job: int) -> RenderOutput:
        cfg = self.jobs[job][1]
        w, h = cfg.width, cfg.height
        acc, aux, color = (np.empty((h, w, 4), np.float32) for _ in range(3))
        depth = np.empty((h, w), np.float32)
        planes = sf_film_planes(_fp(acc), _fp(depth), _fp(aux), None, None, None, _fp(color))
        check(self.ctx.lib.sf_batch_readback(self.h, job, C.byref(planes)))
        n = int(acc[..., 3].min()) if acc.size else 0
        return RenderOutput(color, acc, depth, aux, n, int(acc[..., 3].max()) if acc.size else 0, 0.0)

    def film_planes(self, job: int) -> dict:
        """Every plane of a job's film: accum, depth, aux, volume, moments, surface."""
        cfg = self.jobs[job][1]
        w, h = cfg.width, cfg.height
        out = {k: np.zeros((h, w, 4), np.float32) for k in ("accum", "aux", "volume", "moments", "surface")}
        out["depth"] = np.zeros((h, w), np.float32)
        planes = sf_film_planes(*(_fp(out[k]) for k in ("accum", "depth", "aux", "volume", "moments", "surface")))
        check(self.ctx.lib.sf_batch_readback(self.h, job, C.byref(planes)))
        return out


# ---------------------------------------------------------------------- escape time
FAMILIES = ["Julia", "Mandelbrot", "BurningShip", "Newton", "Nova", "Phoenix"]


@dataclass
class PlanarFractal:
    """PlanarFractal (planar.rs:20-59) with its defaults."""
    family: str = "Julia"
    power: int = 2
    iterations: int = 128
    julia: tuple = (-0.74543, 0.11301)
    center: tuple = (0.0, 0.0)
    zoom: float = 1.0
    angle: float = 0.0
    inversion: float = 0.0
    twist: float = 0.0
    relaxation: float = 1.0
    memory: float = -0.5
    bailout: float = 16.0
    trap_radius: float = 0.5
    stripes: float = 12.0

    def desc(self) -> sf_planar_desc:
        d = sf_planar_desc()
        d.family = FAMILIES.index(self.family)
        d.power, d.iterations = self.power, self.iterations
        d.julia[:] = list(self.julia)
        d.center[:] = list(self.center)
        for k in ("zoom", "angle", "inversion", "twist", "relaxation", "memory", "bailout", "trap_radius",
                  "stripes"):
            setattr(d, k, getattr(self, k))
        return d

    def sample(self, ctx: GpuContext, points) -> dict:
        """PlanarFractal::sample at points (n, 2) on the GPU."""
        pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 2)
        n = len(pts)
        dist = np.zeros(n, np.float32)
        traps = np.zeros((4, n), np.float32)
        iters = np.zeros(n, np.uint32)
        d = self.desc()
        check(ctx.lib.sf_planar_probe(ctx.h, C.byref(d), _fp(pts), n, _fp(dist), _fp(traps), _up(iters)))
        return {"distance": dist, "traps": traps.T.copy(), "iterations": iters}


@dataclass
class Canvas:
    """The 2D canvas mapping (pathtrace.wgsl:1226-1239)."""
    width: int
    height: int
    center: tuple = (0.0, 0.0)
    zoom: float = 1.0
    rotation: float = 0.0
    seed: int = 0

    def desc(self) -> sf_canvas:
        c = sf_canvas()
        c.center[:] = list(self.center)
        c.zoom, c.rotation_deg = self.zoom, self.rotation
        c.width, c.height, c.seed = self.width, self.height, self.seed
        return c


def escape2d(ctx: GpuContext, fractal: PlanarFractal, canvas: Canvas, tile=None, sample: int = 0xFFFFFFFF) -> dict:
    x, y, w, h = tile if tile else (0, 0, canvas.width, canvas.height)
    n = w * h
    dist = np.zeros(n, np.float32)
    traps = np.zeros((4, n), np.float32)
    iters = np.zeros(n, np.uint32)
    d, c = fractal.desc(), canvas.desc()
    check(ctx.lib.sf_escape2d(ctx.h, C.byref(d), C.byref(c), abi.sf_tile(x, y, w, h, 0), sample, _fp(dist),
                              _fp(traps), _up(iters)))
    return {"distance": dist.reshape(h, w), "traps": traps.reshape(4, h, w), "iterations": iters.reshape(h, w)}


ORBIT_MODES = {"device": 0, "host": 1, "given": 2}


def deep_zoom(ctx: GpuContext, center_hi, center_lo, width_units: float, width: int, height: int,
              max_iter: int, bailout: float = 16.0, reference_f64: bool = False, orbit: str = "device",
              given_orbit=None) -> dict:
    """sf_deep_zoom. orbit: "device" (FP64 on the GPU), "host" (FP64 on a host core) or
    "given" (given_orbit: (n, 4) float32 rows Re hi, Im hi, Re lo, Im lo of Z_0..Z_(n-1)
    for c_ref = center_hi)."""
    d = sf_deep_zoom_desc()
    d.center_hi[:] = list(center_hi)
    d.center_lo[:] = list(center_lo)
    d.width_units, d.width, d.height, d.max_iter, d.bailout = width_units, width, height, max_iter, bailout
    d.orbit_mode = ORBIT_MODES[orbit]
    keep = None
    if orbit == "given":
        keep = np.ascontiguousarray(given_orbit, dtype=np.float32).reshape(-1, 4)
        d.orbit_len, d.orbit = len(keep), _fp(keep)
    n = width * height
    it = np.zeros(n, np.uint32)
    sm = np.zeros(n, np.float32)
    it64 = np.zeros(n if reference_f64 else 1, np.uint32)
    sm64 = np.zeros(n if reference_f64 else 1, np.float32)
    reb = C.c_uint64()
    check(ctx.lib.sf_deep_zoom(ctx.h, C.byref(d), _up(it), _fp(sm), 1 if reference_f64 else 0, _up(it64),
                               _fp(sm64), C.byref(reb)))
    out = {"iterations": it.reshape(height, width), "smooth": sm.reshape(height, width), "rebases": reb.value}
    if reference_f64:
        out["iterations_f64"] = it64.reshape(height, width)
        out["smooth_f64"] = sm64.reshape(height, width)
    return out


__all__ = ["GpuContext", "CompiledGraph", "Renderer", "RenderSession", "RenderOutput", "DeSample", "Batch",
           "PlanarFractal", "Canvas", "escape2d", "deep_zoom", "SyfrackError"]

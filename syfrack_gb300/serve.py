"""Serving: previews, progressive refinements and 2D escape-time tiles behind one
request queue (sf_server_* / sf_serve_* in include/syfrack_gpu.h).

The reference serves an interactive client with one RenderSession per view, driven
by RenderSession::step (crates/syfrack-render/src/session.rs:694) one dispatch at a
time, and samples 2D fractals with PlanarFractal::sample
(crates/syfrack-core/src/scene/planar.rs:77). A Server queues the same three kinds
of work and lets the library's scheduler thread batch them: requests that arrive
while others run start as soon as a slot and memory are free, and films stay on the
device from a preview to its last refinement.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from ._lib import check, sf_request, sf_result, sf_server_config, sf_server_stats
from .render import Canvas, PlanarFractal, Renderer
from .scene import RenderConfig, Scene

PREVIEW, REFINE, TILE_2D = 0, 1, 2
QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, 3


@dataclass
class ServeResult:
    ticket: int
    kind: int
    state: int
    status: int
    width: int
    height: int
    samples: int
    batch_requests: int
    work: int
    submit_ms: float
    start_ms: float
    done_ms: float
    accum: Optional[np.ndarray] = None       # 3D: (h, w, 4) sample sums
    iterations: Optional[np.ndarray] = None  # 2D: (h, w) uint32
    smooth: Optional[np.ndarray] = None      # 2D: (h, w) trap 0
    distance: Optional[np.ndarray] = None    # 2D with traps: (h, w)
    traps: Optional[np.ndarray] = None       # 2D with traps: (4, h, w)

    @property
    def latency_ms(self) -> float:
        return self.done_ms - self.submit_ms


class Server:
    """A serving loop on one device (sf_server_create). hbm_budget bounds the
    device bytes of films and tile outputs held at once; requests wait in the queue
    until they fit."""

    def __init__(self, renderer: Renderer, hbm_budget: int, slots: int = 4, path_capacity: int = 1 << 22,
                 max_jobs: int = 256, max_tile_pixels: int = 1 << 25, host_result_bytes: int = 1 << 30,
                 min_blocks: int = 3, quantum: int = 128, regen: int = 4):
        self.renderer = renderer
        self.ctx = renderer.ctx
        k = sf_server_config(hbm_budget=hbm_budget, host_result_bytes=host_result_bytes, slots=slots,
                             path_capacity=path_capacity, max_jobs=max_jobs, max_tile_pixels=max_tile_pixels,
                             min_blocks=min_blocks, quantum=quantum, regen=regen)
        h = C.c_void_p()
        check(self.ctx.lib.sf_server_create(self.ctx.h, C.byref(k), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.sf_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _submit(self, req: sf_request) -> int:
        t = C.c_uint64()
        check(self.ctx.lib.sf_serve_submit(self.h, C.byref(req), C.byref(t)))
        return t.value

    def preview(self, scene: Scene, cfg: RenderConfig) -> int:
        """Queues the first pass of a view: cfg.samples_per_pixel samples into a new
        device film. Returns the ticket."""
        g = self.renderer.compile(scene.graph)  # the film holds its own reference
        # a textured scene's texture graph: compiled and kept by the renderer's cache
        tex = self.renderer.compile(scene.material.texture.graph) if scene.material.texture else None
        r = sf_request(kind=PREVIEW)
        r.graph = g.h
        r.scene = scene.desc(cfg.width, cfg.height, tex.h.value if tex else None)
        r.cfg = cfg.desc()
        return self._submit(r)

    def refine(self, preview_ticket: int, samples: int) -> int:
        """Queues `samples` more samples into the film of an earlier preview."""
        r = sf_request(kind=REFINE, samples=samples, parent=preview_ticket)
        return self._submit(r)

    def tile(self, fractal: PlanarFractal, canvas: Canvas, traps: bool = True) -> int:
        """Queues a 2D escape-time tile: the whole canvas at pixel centres. With
        traps=False only iterations and the smooth time are computed and returned."""
        r = sf_request(kind=TILE_2D, tile_outputs=0 if traps else 1)
        r.planar = fractal.desc()
        r.canvas = canvas.desc()
        return self._submit(r)

    def _result(self, ticket: int, r: sf_result, copy: bool) -> ServeResult:
        out = ServeResult(ticket, r.kind, r.state, r.status, r.width, r.height, r.samples, r.batch_requests,
                          r.work, r.submit_ms, r.start_ms, r.done_ms)
        if copy and r.state == DONE:
            n = r.width * r.height
            if r.kind == TILE_2D:
                out.iterations = np.ctypeslib.as_array(r.iterations, (n,)).reshape(r.height, r.width).copy()
                out.smooth = np.ctypeslib.as_array(r.smooth, (n,)).reshape(r.height, r.width).copy()
                if r.traps:
                    out.distance = np.ctypeslib.as_array(r.distance, (n,)).reshape(r.height, r.width).copy()
                    out.traps = np.ctypeslib.as_array(r.traps, (4 * n,)).reshape(4, r.height, r.width).copy()
            else:
                out.accum = np.ctypeslib.as_array(r.accum, (n * 4,)).reshape(r.height, r.width, 4).copy()
        return out

    def poll(self, ticket: int, copy: bool = True) -> ServeResult:
        r = sf_result()
        check(self.ctx.lib.sf_serve_poll(self.h, ticket, C.byref(r)))
        return self._result(ticket, r, copy)

    def wait(self, ticket: int, timeout_ms: int = 60000, copy: bool = True) -> ServeResult:
        r = sf_result()
        check(self.ctx.lib.sf_serve_wait(self.h, ticket, timeout_ms, C.byref(r)))
        return self._result(ticket, r, copy)

    def release(self, ticket: int):
        check(self.ctx.lib.sf_serve_release(self.h, ticket))

    def stats(self) -> dict:
        s = sf_server_stats()
        check(self.ctx.lib.sf_server_stats_get(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}


__all__ = ["Server", "ServeResult", "PREVIEW", "REFINE", "TILE_2D", "QUEUED", "RUNNING", "DONE", "FAILED"]

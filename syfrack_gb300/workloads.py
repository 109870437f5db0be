"""Seeded synthetic workloads of the DE path (the reference publishes no
benchmark inputs; these restate the measured configurations' shapes, sizes
and parameter ranges).

mandelbulb_primary : 256x256 primary rays, Mandelbulb power 8, 12 iterations,
                     bailout 2.0, pinhole at (0,0,-3) looking at the origin with a
                     60 degree horizontal field of view, 256 steps, epsilon 1e-4, far 10.
mandelbox_pathtrace: 1280x720, 64 spp, 4 bounces, 512 steps; Mandelbox scale -1.5
                     (box fold 1, min radius 0.5, fixed radius 1, 15 iterations,
                     bailout 1000, NormFence); Lambert albedo 0.7 blending into a
                     metal of roughness 0.2 by orbit trap 0; one 1x1 area light of
                     radiance 10 above the form's front-top edge, facing
                     down towards its centre.
mixed_batch        : 64 seeded jobs (Mandelbulb powers 2-12, Mandelbox scales
                     -2.5..2.5, Menger levels 3-7), tiles log-uniform 64..512,
                     1-16 spp, 2 bounces, camera distance 2.5-4, random orientation.
deep_zoom_center   : a seeded point on the Mandelbrot set boundary found by
                     bisection of the escape label along a random ray from c = 0.
"""
from __future__ import annotations

import math

import numpy as np

from .graph import Graph
from .scene import AreaLight, Camera, Material, RenderConfig, Scene, SurfaceVariation


def mandelbulb_primary_graph() -> Graph:
    return Graph.bundled("mandelbulb", power=8.0, iterations=12, bailout=2.0, safety=0.7, hint=2.5)


def mandelbulb_primary():
    """(graph, camera, width, height, max_steps, eps, t_far)."""
    cam = Camera.look_at((0.0, 0.0, -3.0), (0.0, 0.0, 0.0), 60.0)
    return mandelbulb_primary_graph(), cam, 256, 256, 256, 1e-4, 10.0


def mandelbox_graph(scale=-1.5, iterations=15) -> Graph:
    # |scale| < 2 fills the cube [-2, 2]^3: enclosing radius 2*sqrt(3)
    return Graph.bundled("mandelbox", scale=scale, iterations=iterations, bailout=1000.0, limit=1.0,
                         min_radius=0.5, fixed_radius=1.0, trap_scale=2.0, safety=0.6, hint=3.5)


def mandelbox_scene(seed: int = 20261203) -> Scene:
    mat = Material(albedo=(0.7, 0.7, 0.7), roughness=0.2, metallic=0.0, specular=0.04,
                   surface=SurfaceVariation(slot=0, roughness=(0.2, 0.2), metallic=(0.0, 1.0)))
    # above the form's front-top edge, facing down towards its centre
    light = AreaLight(position=(1.0, 3.5, -3.5), normal=(-1.0, -3.5, 3.5), size=(1.0, 1.0),
                      color=(1.0, 1.0, 1.0), intensity=10.0)
    cam = Camera.look_at((3.2, 2.6, -5.5), (0.0, 0.0, 0.0), 45.0)
    return Scene(graph=mandelbox_graph(), camera=cam, material=mat, lights=[light], seed=seed)


def mandelbox_pathtrace_config(integrator="wavefront", width=1280, height=720, spp=64,
                               samples_per_dispatch=8) -> RenderConfig:
    return RenderConfig(width=width, height=height, samples_per_pixel=spp, max_bounces=4, max_steps=512,
                        pixel_tolerance=1.0, tile_size=max(width, height),
                        samples_per_dispatch=samples_per_dispatch, integrator=integrator)


def mixed_batch(seed: int = 7, jobs: int = 64):
    """Seeded list of (scene, config) for the uneven batch."""
    rng = np.random.default_rng(seed)
    out = []
    for j in range(jobs):
        kind = j % 3
        if kind == 0:
            g = Graph.bundled("mandelbulb", power=float(rng.integers(2, 13)), iterations=10, bailout=4.0,
                              safety=0.7, hint=2.5)
        elif kind == 1:
            s = float(rng.uniform(-2.5, 2.5))
            if abs(s) < 1.05:
                s = math.copysign(1.05, s if s != 0 else 1.0)
            g = mandelbox_graph(scale=s, iterations=12)
            if abs(s) > 2.0:
                g.bounding_radius_hint = 2.0 * (abs(s) + 1.0) / (abs(s) - 1.0) * math.sqrt(3.0)
        else:
            g = Graph.bundled("menger", iterations=int(rng.integers(3, 8)))
        dist = float(rng.uniform(2.5, 4.0))
        if kind == 1:
            dist *= g.bounding_radius_hint / 2.0
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        cam = Camera.look_at(tuple((v * dist).tolist()), (0.0, 0.0, 0.0), 50.0)
        side = int(round(math.exp(rng.uniform(math.log(64), math.log(512)))))
        spp = int(rng.integers(1, 17))
        light = AreaLight(position=tuple((v * dist * 0.5 + np.array([0, dist * 0.6, 0])).tolist()),
                          normal=(0.0, -1.0, 0.0), size=(1.0, 1.0), intensity=10.0)
        scene = Scene(graph=g, camera=cam, material=Material(albedo=(0.7, 0.7, 0.7), roughness=0.4),
                      lights=[light], seed=int(rng.integers(0, 2**31)))
        cfg = RenderConfig(width=side, height=side, samples_per_pixel=spp, max_bounces=2, max_steps=512,
                           tile_size=side, samples_per_dispatch=spp, integrator="wavefront")
        out.append((scene, cfg))
    return out


def mandelbrot_escapes(cx: float, cy: float, max_iter: int, bailout: float = 2.0) -> bool:
    """Direct FP64 escape label of c (z <- z^2 + c)."""
    zx = zy = 0.0
    b2 = bailout * bailout
    for _ in range(max_iter):
        x2, y2 = zx * zx, zy * zy
        if x2 + y2 > b2:
            return True
        zy = 2.0 * zx * zy + cy
        zx = x2 - y2 + cx
    return False


def deep_zoom_center(seed: int = 2026, max_iter: int = 50000, steps: int = 64):
    """Bisects the FP64 escape label of c along a seeded ray from c = 0 (inside)
    to |c| = 2.5 (outside). Returns the last non-escaping point (cx, cy)."""
    rng = np.random.default_rng(seed)
    ang = float(rng.uniform(0, 2 * math.pi))
    dx, dy = math.cos(ang), math.sin(ang)
    lo_t, hi_t = 0.0, 2.5
    for _ in range(steps):
        mid = 0.5 * (lo_t + hi_t)
        if mid in (lo_t, hi_t):
            break
        if mandelbrot_escapes(mid * dx, mid * dy, max_iter):
            hi_t = mid
        else:
            lo_t = mid
    return (lo_t * dx, lo_t * dy)

"""Seeded synthetic workloads of the DE path (the reference publishes no
benchmark inputs; these restate the measured configurations' shapes, sizes
and parameter ranges).

mandelbulb_primary : 256x256 primary rays, Mandelbulb power 8, 12 iterations,
                     bailout 2.0, pinhole at (0,0,-3) looking at the origin with a
                     60 degree horizontal field of view, 256 steps, epsilon 1e-4, far 10.
mandelbox_pathtrace: 1280x720, 64 spp, 4 bounces, 512 steps, hit epsilon 1e-4
                     (fixed-epsilon hit test; rule="cone" gives the reference's
                     cone-relative test at pixel tolerance 1); Mandelbox scale -1.5
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


PATHTRACE_EPSILON = 1e-4


def mandelbox_pathtrace_config(integrator="wavefront", width=1280, height=720, spp=64,
                               samples_per_dispatch=8, rule="epsilon") -> RenderConfig:
    """rule "epsilon": hits at radius <= 1e-4 (the stated march epsilon); "cone": the
    reference's cone-relative test radius / t < pixel_cone at pixel tolerance 1."""
    eps = {"epsilon": PATHTRACE_EPSILON, "cone": 0.0}[rule]
    return RenderConfig(width=width, height=height, samples_per_pixel=spp, max_bounces=4, max_steps=512,
                        pixel_tolerance=1.0, tile_size=max(width, height),
                        samples_per_dispatch=samples_per_dispatch, integrator=integrator, hit_epsilon=eps)


def mandelbox_radius(scale: float) -> float:
    """Radius of a sphere enclosing the Mandelbox of this scale: scales <= 1 stay in
    the cube [-2, 2]^3, scales s > 1 reach 2(s+1)/(s-1) along each axis (the band near
    s = 1 is capped at 12, beyond which the form is thin shells)."""
    half = 2.0 if scale <= 1.0 else min(2.0 * (scale + 1.0) / (scale - 1.0), 12.0)
    return half * math.sqrt(3.0)


def mixed_batch_graph(kind: str, value) -> Graph:
    """One form of the uneven batch: ("mandelbulb", power), ("mandelbox", scale) or
    ("menger", level)."""
    if kind == "mandelbulb":
        return Graph.bundled("mandelbulb", power=float(value), iterations=10, bailout=4.0, safety=0.7, hint=2.5)
    if kind == "mandelbox":
        g = mandelbox_graph(scale=float(value), iterations=12)
        g.bounding_radius_hint = mandelbox_radius(float(value))
        return g
    return Graph.bundled("menger", iterations=int(value))


def mixed_batch(seed: int = 7, jobs: int = 64):
    """Seeded list of (scene, config) for the uneven batch: Mandelbulb powers U{2..12},
    Mandelbox scales U[-2.5, 2.5] (the whole range), Menger levels U{3..7}; the camera
    at 2.5-4 units (Mandelbulb, Menger) or 2.5-4 half-radii of the Mandelbox's
    enclosing sphere from the origin, in a uniform random direction."""
    rng = np.random.default_rng(seed)
    out = []
    for j in range(jobs):
        kind = j % 3
        if kind == 0:
            g = mixed_batch_graph("mandelbulb", int(rng.integers(2, 13)))
        elif kind == 1:
            s = float(rng.uniform(-2.5, 2.5))
            while abs(s) < 1e-3:  # Scale factors below 1e-3 fail validation (validate.rs:187-196)
                s = float(rng.uniform(-2.5, 2.5))
            g = mixed_batch_graph("mandelbox", s)
        else:
            g = mixed_batch_graph("menger", int(rng.integers(3, 8)))
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


# ---------------------------------------------------------------------- serving stream
SERVE_PREVIEW = dict(width=480, height=270, spp=1, bounces=1, steps=512)
SERVE_REFINE_SPP = 8
SERVE_REFINE_WINDOW = 16  # a refinement picks one of the 16 latest previews


def serving_graphs():
    """The forms a serving client orbits: Mandelbulb powers 6, 8, 10 and Mandelbox
    scales -1.5, -2, 2 (compiled once, then cached by the renderer)."""
    bulbs = [Graph.bundled("mandelbulb", power=p, iterations=10, bailout=4.0, safety=0.7, hint=2.5)
             for p in (6.0, 8.0, 10.0)]
    boxes = [mandelbox_graph(scale=s, iterations=12) for s in (-1.5, -2.0, 2.0)]
    return bulbs + boxes


def _preview_scene(rng, graphs):
    g = graphs[int(rng.integers(0, len(graphs)))]
    dist = float(rng.uniform(2.5, 4.0)) * max(1.0, g.bounding_radius_hint / 2.5)
    v = rng.normal(size=3)
    v /= np.linalg.norm(v)
    cam = Camera.look_at(tuple((v * dist).tolist()), (0.0, 0.0, 0.0), 50.0)
    light = AreaLight(position=tuple((v * dist * 0.5 + np.array([0, dist * 0.6, 0])).tolist()),
                      normal=(0.0, -1.0, 0.0), size=(1.0, 1.0), intensity=10.0)
    scene = Scene(graph=g, camera=cam, material=Material(albedo=(0.7, 0.7, 0.7), roughness=0.4),
                  lights=[light], seed=int(rng.integers(0, 2**31)))
    p = SERVE_PREVIEW
    cfg = RenderConfig(width=p["width"], height=p["height"], samples_per_pixel=p["spp"], max_bounces=p["bounces"],
                       max_steps=p["steps"], tile_size=max(p["width"], p["height"]),
                       samples_per_dispatch=p["spp"], integrator="wavefront")
    return scene, cfg


def _tile(rng, side_range=(256, 2048), iter_range=(1000, 20000)):
    from .render import Canvas, PlanarFractal

    side = int(rng.integers(side_range[0], side_range[1] + 1))
    iters = int(rng.integers(iter_range[0], iter_range[1] + 1))
    if rng.random() < 0.5:
        a = float(rng.uniform(0.0, 2.0 * math.pi))
        f = PlanarFractal(family="Julia", iterations=iters, julia=(0.7885 * math.cos(a), 0.7885 * math.sin(a)))
        canvas = Canvas(width=side, height=side, center=(0.0, 0.0), zoom=2.0)
    else:
        f = PlanarFractal(family="BurningShip", iterations=iters)
        cx, cy = -0.45 + float(rng.uniform(-0.2, 0.2)), -0.5 + float(rng.uniform(-0.2, 0.2))
        canvas = Canvas(width=side, height=side, center=(cx, cy), zoom=float(rng.uniform(1.5, 3.0)))
    return f, canvas


def serving_stream(seed: int = 5, rate: float = 200.0, duration: float = 60.0, tile_side=(256, 2048),
                   tile_iters=(1000, 20000)):
    """Seeded Poisson request stream: list of (arrival_s, kind, payload). Kinds:
    'tile' 40% (Julia with c = 0.7885 e^{ia}, or a Burning Ship view; side and
    iterations uniform in the given ranges), 'preview' 40% (480x270, 1 spp, 1
    bounce, a random orbit of one of serving_graphs()), 'refine' 20% (+8 spp to one
    of the 16 latest previews; payload = index of that preview's event)."""
    rng = np.random.default_rng(seed)
    graphs = serving_graphs()
    out, previews = [], []
    t = 0.0
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= duration:
            break
        u = float(rng.random())
        if u < 0.4:
            out.append((t, "tile", _tile(rng, tile_side, tile_iters)))
        elif u < 0.8 or not previews:
            previews.append(len(out))
            out.append((t, "preview", _preview_scene(rng, graphs)))
        else:
            k = previews[-SERVE_REFINE_WINDOW:]
            out.append((t, "refine", k[int(rng.integers(0, len(k)))]))
    return out

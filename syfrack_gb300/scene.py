"""Scene-side types of the DE path, mirroring syfrack-core:
Camera / CameraBasis (crates/syfrack-core/src/scene/camera.rs:6-104),
Light::Area (light.rs:79-85) and its GPU packing (syfrack-render/src/uniforms.rs:671-713),
Material / Finish (material.rs:136-170), RenderConfig (syfrack-render/src/renderer.rs:17-76).
Vector arithmetic is binary32 (numpy float32), like glam's Vec3.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .graph import Graph

f32 = np.float32


def _v(x):
    return np.asarray(x, dtype=f32).reshape(3)


def _normalize(v):
    return (v / f32(math.sqrt(float(np.dot(v, v).astype(f32))))).astype(f32)


def _normalize_or(v, fallback):
    n = float(np.dot(v, v).astype(f32))
    if not (n > 0.0) or not math.isfinite(n):
        return _v(fallback)
    r = f32(1.0) / f32(math.sqrt(n))
    if not (r > 0) or not math.isfinite(float(r)):
        return _v(fallback)
    return (v * r).astype(f32)


@dataclass
class CameraBasis:
    origin: np.ndarray
    forward: np.ndarray
    right: np.ndarray
    up: np.ndarray
    tan_half_fov: float
    lens_radius: float
    focus_distance: float


@dataclass
class Camera:
    """CameraMode::Free{position, target, roll}; focal_mm (36 mm sensor), f_number, focus."""
    position: tuple = (0.0, 0.0, -3.0)
    target: tuple = (0.0, 0.0, 0.0)
    roll: float = 0.0
    focal_mm: float = 35.0
    f_number: float = 0.0
    focus_distance: float = 3.0

    @classmethod
    def look_at(cls, position, target, fov_deg: float, roll: float = 0.0):
        """A pinhole camera with a horizontal field of view (tan_half_fov = 18 / focal_mm)."""
        focal = 18.0 / math.tan(math.radians(fov_deg) * 0.5)
        return cls(tuple(position), tuple(target), roll, focal, 0.0, 3.0)

    @classmethod
    def orbit(cls, point, distance, azimuth, elevation, roll=0.0, focal_mm=35.0):
        """CameraMode::Orbit: azimuth/elevation in degrees around `point`."""
        az, el = math.radians(azimuth), math.radians(elevation)
        off = np.array([math.cos(el) * math.sin(az), math.sin(el), math.cos(el) * math.cos(az)]) * distance
        pos = tuple((np.asarray(point, dtype=np.float64) + off).tolist())
        return cls(pos, tuple(point), roll, focal_mm)

    def basis(self) -> CameraBasis:
        """Camera::basis (camera.rs:58-104)."""
        origin = _v(self.position)
        target = _v(self.target)
        forward = _normalize_or((target - origin).astype(f32), (0.0, 0.0, -1.0))
        world_up = _v((0, 0, 1)) if abs(float(forward[1])) > 0.9999 else _v((0, 1, 0))
        right0 = _normalize(np.cross(forward, world_up).astype(f32))
        up0 = np.cross(right0, forward).astype(f32)
        r = f32(self.roll) * f32(math.pi / 180.0)
        s, c = f32(math.sin(r)), f32(math.cos(r))
        right = (right0 * c + up0 * s).astype(f32)
        up = (up0 * c - right0 * s).astype(f32)
        lens = (self.focal_mm / 1000.0) / (2.0 * self.f_number) if self.f_number > 0 else 0.0
        return CameraBasis(origin, forward, right, up, float(f32(18.0) / f32(self.focal_mm)), lens,
                           self.focus_distance)


@dataclass
class AreaLight:
    """Light::Area{position, normal, size, color, intensity}; color is linear RGB."""
    position: tuple = (0.0, 4.0, 0.0)
    normal: tuple = (0.0, -1.0, 0.0)
    size: tuple = (1.0, 1.0)
    color: tuple = (1.0, 1.0, 1.0)
    intensity: float = 10.0

    def packed(self) -> abi.sf_area_light:
        """GpuLight::from_light for Area (uniforms.rs:671-713): a = centre, b/c = full edges."""
        n = _normalize_or(_v(self.normal), (0, 1, 0))
        helper = _v((0, 0, 1)) if abs(float(n[1])) > 0.999 else _v((0, 1, 0))
        u = _normalize(np.cross(helper, n).astype(f32))
        v = np.cross(n, u).astype(f32)
        out = abi.sf_area_light()
        out.center[:] = [float(x) for x in _v(self.position)]
        out.edge_u[:] = [float(x) for x in (u * f32(self.size[0])).astype(f32)]
        out.edge_v[:] = [float(x) for x in (v * f32(self.size[1])).astype(f32)]
        out.radiance[:] = [float(f32(c) * f32(self.intensity)) for c in self.color]
        return out


@dataclass
class Finish:
    albedo: tuple = (0.7, 0.7, 0.7)
    roughness: float = 0.5
    metallic: float = 0.0
    specular: float = 0.04
    emission: tuple = (0.0, 0.0, 0.0)

    def packed(self) -> abi.sf_material:
        m = abi.sf_material()
        m.albedo[:] = list(self.albedo)
        m.roughness, m.metallic, m.specular = self.roughness, self.metallic, self.specular
        m.emission[:] = list(self.emission)
        return m


@dataclass
class SurfaceVariation:
    """Trap-driven roughness/metallic ramp (uniforms.rs:485-495)."""
    slot: int = 0
    roughness: tuple = (0.2, 0.2)
    metallic: tuple = (0.0, 1.0)


@dataclass
class Material(Finish):
    finishes: list = field(default_factory=list)
    surface: SurfaceVariation | None = None


@dataclass
class Scene:
    graph: Graph
    camera: Camera = field(default_factory=Camera)
    material: Material = field(default_factory=Material)
    lights: list = field(default_factory=list)
    seed: int = 0
    cavity_darkness: float = 0.0

    def desc(self, width: int, height: int) -> abi.sf_scene_desc:
        """The scene half of Uniforms::from_scene (uniforms.rs:748-830)."""
        b = self.camera.basis()
        d = abi.sf_scene_desc()
        cam = d.camera
        cam.origin[:] = [float(x) for x in b.origin]
        cam.forward[:] = [float(x) for x in b.forward]
        cam.right[:] = [float(x) for x in b.right]
        cam.up[:] = [float(x) for x in b.up]
        cam.tan_half_fov = b.tan_half_fov
        cam.aspect = float(f32(width) / f32(height))
        cam.lens_radius = b.lens_radius
        cam.focus_distance = b.focus_distance
        d.material = self.material.packed()
        if len(self.material.finishes) > abi.SF_MAX_FINISHES:
            raise ValueError("at most 8 finishes")
        for i, f in enumerate(self.material.finishes):
            d.finishes[i] = f.packed()
        d.finish_count = len(self.material.finishes)
        if len(self.lights) > abi.SF_MAX_LIGHTS:
            raise ValueError("at most 8 area lights on the device path")
        for i, l in enumerate(self.lights):
            d.lights[i] = l.packed()
        d.light_count = len(self.lights)
        sv = self.material.surface
        if sv is not None:
            d.variation_slot = sv.slot
            d.variation_enabled = 1
            d.variation_roughness[:] = list(sv.roughness)
            d.variation_metallic[:] = list(sv.metallic)
        d.cavity_darkness = self.cavity_darkness
        d.seed = self.seed & 0xFFFFFFFFFFFFFFFF
        return d


@dataclass
class RenderConfig:
    """RenderConfig (renderer.rs:17-43); defaults of RenderConfig::new (:58-76)."""
    width: int
    height: int
    samples_per_pixel: int
    max_bounces: int = 4
    max_steps: int = 256
    pixel_tolerance: float = 1.0
    tile_size: int = 256
    samples_per_dispatch: int = 8
    integrator: str = "megakernel"  # or "wavefront"

    def desc(self) -> abi.sf_render_config:
        c = abi.sf_render_config()
        c.integrator = {"megakernel": 0, "wavefront": 1}[self.integrator]
        c.width, c.height, c.samples_per_pixel = self.width, self.height, self.samples_per_pixel
        c.max_bounces, c.max_steps = self.max_bounces, self.max_steps
        c.pixel_tolerance = self.pixel_tolerance
        c.tile_size, c.samples_per_dispatch = self.tile_size, self.samples_per_dispatch
        return c

"""Scene-side types of the DE path, mirroring syfrack-core:
Camera / CameraBasis (crates/syfrack-core/src/scene/camera.rs:6-104),
Light::Area (light.rs:79-85) and its GPU packing (syfrack-render/src/uniforms.rs:671-713),
Material / Finish (material.rs:136-170), RenderConfig (syfrack-render/src/renderer.rs:17-76).
Vector arithmetic is binary32 (numpy float32), like glam's Vec3.
"""
from __future__ import annotations

import ctypes as C
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
class ProjectorLight(AreaLight):
    """Light::Projector{position, normal, size, color, intensity, inner_angle, outer_angle}:
    an area light whose emission about its normal is full within inner_angle degrees
    and none beyond outer_angle (light.rs:88-97, lights.wgsl:11-16)."""
    inner_angle: float = 10.0
    outer_angle: float = 18.0

    def packed(self) -> abi.sf_area_light:
        out = super().packed()
        out.kind = abi.SF_LIGHT_PROJECTOR
        out.direction[0] = self.inner_angle
        out.direction[1] = self.outer_angle
        return out


@dataclass
class TubeLight:
    """Light::Tube{start, end, radius, color, intensity}: a capsule emitter (light.rs:99-105,
    GpuLight::from_light uniforms.rs:717-729)."""
    start: tuple = (-0.5, 2.0, 0.0)
    end: tuple = (0.5, 2.0, 0.0)
    radius: float = 0.05
    color: tuple = (1.0, 1.0, 1.0)
    intensity: float = 10.0

    def packed(self) -> abi.sf_area_light:
        out = abi.sf_area_light()
        out.kind = abi.SF_LIGHT_TUBE
        out.center[:] = [float(x) for x in _v(self.start)]
        out.edge_u[:] = [float(x) for x in _v(self.end)]
        out.edge_v[0] = self.radius
        out.radiance[:] = [float(f32(c) * f32(self.intensity)) for c in _color(self.color)]
        return out


def kelvin_to_linear(kelvin: float):
    """Color::Kelvin (light.rs:28-58): Tanner Helland's black-body approximation,
    sRGB to linear, normalised so the brightest channel is 1 (binary32)."""
    t = f32(min(max(kelvin, 1000.0), 40000.0)) / f32(100.0)
    if t <= 66.0:
        r = f32(255.0)
        g = f32(99.4708) * f32(math.log(t)) - f32(161.11957)
    else:
        r = f32(329.69873) * f32((t - f32(60.0)) ** f32(-0.13320476))
        g = f32(288.12217) * f32((t - f32(60.0)) ** f32(-0.07551485))
    if t >= 66.0:
        b = f32(255.0)
    elif t <= 19.0:
        b = f32(0.0)
    else:
        b = f32(138.51773) * f32(math.log(t - f32(10.0))) - f32(305.0448)

    def srgb_to_linear(v):
        v = f32(v)
        return v / f32(12.92) if v <= 0.04045 else f32(((v + f32(0.055)) / f32(1.055)) ** f32(2.4))

    c = [srgb_to_linear(min(max(f32(x) / f32(255.0), 0.0), 1.0)) for x in (r, g, b)]
    m = max(c[0], c[1], c[2], f32(1e-6))
    return tuple(float(f32(x) / m) for x in c)


def _color(c):
    """A light colour: ("kelvin", K) / {"Kelvin": K} or a linear RGB triple."""
    if isinstance(c, (int, float)):
        return kelvin_to_linear(float(c))
    if isinstance(c, dict) and "Kelvin" in c:
        return kelvin_to_linear(float(c["Kelvin"]))
    if isinstance(c, tuple) and len(c) == 2 and c[0] == "kelvin":
        return kelvin_to_linear(float(c[1]))
    return tuple(float(x) for x in c)


@dataclass
class SunLight:
    """Light::Sun{direction (toward the sun), color, intensity (irradiance), angular_size (deg)}."""
    direction: tuple = (-0.4, 0.8, 0.3)
    color: tuple = (1.0, 1.0, 1.0)
    intensity: float = 6.0
    angular_size: float = 1.0

    def packed(self) -> abi.sf_area_light:
        out = abi.sf_area_light()
        out.kind = abi.SF_LIGHT_SUN
        out.direction[:] = [float(x) for x in _normalize_or(_v(self.direction), (0, 1, 0))]
        out.angular_size = self.angular_size
        out.radiance[:] = [float(f32(c) * f32(self.intensity)) for c in _color(self.color)]
        return out


@dataclass
class EnvironmentLight:
    """Light::Environment{zenith, horizon, ground, intensity}: a vertical gradient sky."""
    zenith: tuple = (0.2, 0.35, 0.7)
    horizon: tuple = (0.6, 0.65, 0.7)
    ground: tuple = (0.15, 0.12, 0.1)
    intensity: float = 1.0

    def packed(self) -> abi.sf_area_light:
        out = abi.sf_area_light()
        out.kind = abi.SF_LIGHT_ENVIRONMENT
        k = f32(self.intensity)
        out.zenith[:] = [float(f32(c) * k) for c in _color(self.zenith)]
        out.horizon[:] = [float(f32(c) * k) for c in _color(self.horizon)]
        out.ground[:] = [float(f32(c) * k) for c in _color(self.ground)]
        return out


def panorama_tables(rgb):
    """EnvironmentMap::from_rgb through the library, on the host only: (texels[h, w, 4]
    of rgb and cumulative distribution, uniform)."""
    import ctypes as C

    from ._lib import check, load

    rgb = np.ascontiguousarray(rgb, dtype=np.float32)
    h, w = rgb.shape[:2]
    lib = load()
    fp = C.POINTER(C.c_float)
    ow, oh, uni = C.c_uint32(), C.c_uint32(), C.c_int()
    check(lib.sf_environment_build(rgb.ctypes.data_as(fp), w, h, None, C.byref(ow), C.byref(oh), C.byref(uni)))
    out = np.zeros((oh.value, ow.value, 4), np.float32)
    check(lib.sf_environment_build(rgb.ctypes.data_as(fp), w, h, out.ctypes.data_as(fp), C.byref(ow), C.byref(oh),
                                   C.byref(uni)))
    return out, bool(uni.value)


class Panorama:
    """An equirectangular linear RGB panorama on the device (sf_environment_create):
    rgb[h, w, 3], row 0 at the zenith. Keep it alive while scenes render with it."""

    def __init__(self, ctx, rgb):
        import ctypes as C

        from ._lib import check

        self.ctx = ctx
        self.rgb = np.ascontiguousarray(rgb, dtype=np.float32)
        h, w = self.rgb.shape[:2]
        handle = C.c_void_p()
        check(ctx.lib.sf_environment_create(ctx.h, self.rgb.ctypes.data_as(C.POINTER(C.c_float)), w, h,
                                            C.byref(handle)))
        self.h = handle

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.sf_environment_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class HdriLight:
    """Light::Hdri{intensity, rotation (degrees about +y)} over a Panorama."""
    panorama: Panorama = None
    intensity: float = 1.0
    rotation: float = 0.0

    def packed(self) -> abi.sf_area_light:
        out = abi.sf_area_light()
        out.kind = abi.SF_LIGHT_HDRI
        out.environment = self.panorama.h.value if self.panorama is not None else None
        out.radiance[0] = self.intensity
        out.rotation = self.rotation
        return out


@dataclass
class Ramp:
    """Ramp (palette.rs:74-100): stops, optional positions, cyclic, frequency, phase, gamma."""
    stops: list = field(default_factory=lambda: [(0.0, 0.0, 0.0), (1.0, 1.0, 1.0)])
    positions: list = field(default_factory=list)
    cyclic: bool = False
    frequency: float = 1.0
    phase: float = 0.0
    gamma: float = 1.0
    smooth: bool = False


@dataclass
class OrbitColoring:
    """OrbitColoring (material.rs:18-56): weights of the four traps, the iteration
    fraction and n.y * 0.5 + 0.5, optional signed log remapping."""
    traps: tuple = (1.0, 0.0, 0.0, 0.0)
    iterations: float = 0.0
    normal: float = 0.0
    logarithmic: float = 0.0

    def pack(self, out: abi.sf_orbit_coloring):
        out.traps[:] = [float(x) for x in self.traps]
        out.iterations, out.normal, out.logarithmic = self.iterations, self.normal, self.logarithmic


@dataclass
class Coloring:
    """Coloring::Trap{slot, ramp} (material.rs:100-130); slot 4 = iterations, 5 = normal;
    with `orbit` set, Coloring::Orbit{channels, ramp} (slot 6)."""
    slot: int = 0
    ramp: Ramp = field(default_factory=Ramp)
    orbit: OrbitColoring | None = None


FINISH_PATTERNS = ["VeinedStone", "Patina", "BrushedMetal", "Basalt", "Ripples", "Rosettes", "CoastalRock", "Sand",
                   "Dust", "Concrete", "WeatheredConcrete", "WetConcrete"]


@dataclass
class FinishDetail:
    """FinishDetail (material.rs:200-224): a world-space pattern on a finish."""
    pattern: str = "VeinedStone"
    seed: int = 7
    scale: float = 2.0
    strength: float = 0.25
    bump: float = 0.004
    roughness_delta: float = 0.15
    tint: tuple = (0.3, 0.27, 0.2)

    def pack(self, out: abi.sf_finish_detail):
        out.pattern = FINISH_PATTERNS.index(self.pattern) + 1
        out.seed = self.seed
        out.scale, out.strength, out.bump, out.roughness_delta = self.scale, self.strength, self.bump, self.roughness_delta
        out.tint[:] = [float(x) for x in self.tint]


@dataclass
class Optics:
    """Optics (optics.rs:7-38): coverage, a rough dielectric interface and an interior medium."""
    opacity: float = 1.0
    transmission: float = 1.0
    ior: float = 1.5
    thin_walled: bool = False
    absorption_color: tuple = (1.0, 1.0, 1.0)
    absorption_distance: float = 1.0
    subsurface: float = 0.0
    subsurface_color: tuple = (0.9, 0.9, 0.9)
    subsurface_radius: float = 0.5

    def pack(self, out: abi.sf_optics):
        out.enabled = 1
        out.opacity, out.transmission, out.ior = self.opacity, self.transmission, self.ior
        out.thin_walled = int(self.thin_walled)
        out.absorption_color[:] = [float(x) for x in self.absorption_color]
        out.absorption_distance = self.absorption_distance
        out.subsurface = self.subsurface
        out.subsurface_color[:] = [float(x) for x in self.subsurface_color]
        out.subsurface_radius = self.subsurface_radius


@dataclass
class FractalTexture:
    """FractalTexture (texture.rs:62-136): a volumetric texture from a second graph.
    channel: ("trap", slot), ("iterations",), ("distance",) or ("orbit", OrbitColoring)."""
    graph: Graph = None
    channel: tuple = ("trap", 0)
    scale: float = 3.0
    offset: tuple = (0.37, 0.19, 0.53)
    rotation: tuple = (0.0, 0.0, 0.0)
    octaves: int = 2
    contrast: float = 2.0
    ramp: Ramp = field(default_factory=lambda: Ramp(stops=[(0.12, 0.22, 0.27), (0.86, 0.6, 0.22)]))
    strength: float = 1.0
    roughness: float = 0.35
    bump: float = 0.15
    parallax: float = 0.0
    parallax_steps: int = 8
    fan: tuple | None = None   # (period_x, period_z, rays)
    mask: tuple | None = None  # (trap slot, value, width)

    def pack(self, out: abi.sf_texture, graph_handle):
        kind = self.channel[0]
        out.graph = graph_handle
        out.channel = {"trap": None, "iterations": 4, "distance": 6, "orbit": 7}[kind] if kind != "trap" else int(self.channel[1])
        if kind == "orbit":
            self.channel[1].pack(out.orbit)
        out.scale = self.scale
        out.offset[:] = [float(x) for x in self.offset]
        out.rotation[:] = [float(x) for x in self.rotation]
        out.octaves, out.contrast = self.octaves, self.contrast
        _pack_ramp(self.ramp, out.ramp)
        out.strength, out.roughness, out.bump = self.strength, self.roughness, self.bump
        out.parallax, out.parallax_steps = self.parallax, self.parallax_steps
        if self.fan is not None:
            out.fan = 1
            out.fan_period[:] = [float(self.fan[0]), float(self.fan[1])]
            out.fan_rays = int(self.fan[2])
        if self.mask is not None:
            out.mask = 1
            out.mask_slot, out.mask_value, out.mask_width = int(self.mask[0]), float(self.mask[1]), float(self.mask[2])


def _pack_ramp(r: Ramp, out: abi.sf_coloring):
    """GpuRamp::from_ramp: stops with their positions (palette.rs:106-115)."""
    if len(r.stops) > abi.SF_MAX_RAMP_STOPS:
        raise ValueError("at most 16 ramp stops")
    n = len(r.stops)
    out.stop_count = n
    for i, c in enumerate(r.stops):
        # Ramp::position: given, else i / (n or n - 1)
        pos = r.positions[i] if r.positions else float(f32(i) / f32(n if r.cyclic else max(n - 1, 1)))
        out.stops[i][:] = [float(c[0]), float(c[1]), float(c[2]), float(pos)]
    out.cyclic = int(r.cyclic)
    out.smooth = int(r.smooth)
    out.positioned = int(bool(r.positions))
    out.frequency, out.phase, out.gamma = r.frequency, r.phase, r.gamma


@dataclass
class Finish:
    albedo: tuple = (0.7, 0.7, 0.7)
    roughness: float = 0.5
    metallic: float = 0.0
    specular: float = 0.04
    emission: tuple = (0.0, 0.0, 0.0)
    detail: FinishDetail | None = None
    optics: Optics | None = None

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
    coloring: Coloring | None = None
    texture: FractalTexture | None = None


@dataclass
class Fog:
    """Atmosphere's height fog (atmosphere.rs:7-28): extinction `density` at and below
    `height`, decaying as exp(-(y - height) * falloff) above it; Henyey-Greenstein
    `anisotropy`; scattering albedo `color` (0 = purely absorbing)."""
    density: float = 0.0
    color: tuple = (1.0, 1.0, 1.0)
    height: float = 0.0
    falloff: float = 1.0
    anisotropy: float = 0.0


@dataclass
class Scene:
    graph: Graph
    camera: Camera = field(default_factory=Camera)
    material: Material = field(default_factory=Material)
    lights: list = field(default_factory=list)
    seed: int = 0
    cavity_darkness: float = 0.0
    fog: Fog | None = None
    dune_wind: float = 0.0  # Dunes.wind_direction (degrees): the Sand detail's wind

    def desc(self, width: int, height: int, texture_graph=None) -> abi.sf_scene_desc:
        """The scene half of Uniforms::from_scene (uniforms.rs:748-830). texture_graph:
        the handle of the compiled texture graph when the material has a texture."""
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
        if len(self.lights) > abi.SF_MAX_SCENE_LIGHTS:
            # Scene::validate (scene/mod.rs:512)
            raise ValueError(f"a scene may have at most {abi.SF_MAX_SCENE_LIGHTS} lights, got {len(self.lights)}")
        if len(self.lights) > abi.SF_MAX_LIGHTS:
            # more than the inline array holds: the list replaces it (kept alive with d)
            table = (abi.sf_area_light * len(self.lights))(*[l.packed() for l in self.lights])
            d._light_table = table
            d.light_list = C.cast(table, C.POINTER(abi.sf_area_light))
            d.light_list_count = len(self.lights)
        else:
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
        if self.fog is not None and self.fog.density > 0.0:
            d.fog.density = self.fog.density
            d.fog.height = self.fog.height
            d.fog.falloff = self.fog.falloff
            d.fog.anisotropy = self.fog.anisotropy
            d.fog.color[:] = [float(c) for c in self.fog.color]
        d.seed = self.seed & 0xFFFFFFFFFFFFFFFF
        col = self.material.coloring
        d.coloring.slot = 0xFFFF
        if col is not None:
            _pack_ramp(col.ramp, d.coloring)
            d.coloring.slot = 6 if col.orbit is not None else col.slot
            if col.orbit is not None:
                col.orbit.pack(d.coloring_orbit)
        # ABI 1.3: finish details, optics, the texture
        d.dune_wind = self.dune_wind
        for i, f in enumerate(self.material.finishes):
            if f.detail is not None:
                f.detail.pack(d.details[i])
            if f.optics is not None:
                f.optics.pack(d.optics[i + 1])
        if self.material.optics is not None:
            self.material.optics.pack(d.optics[0])
        if self.material.texture is not None:
            if texture_graph is None:
                raise ValueError("a textured scene needs its compiled texture graph")
            self.material.texture.pack(d.texture, texture_graph)
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
    # 0: the reference's cone-relative hit test; > 0: fixed epsilon radius <= hit_epsilon
    hit_epsilon: float = 0.0

    def desc(self) -> abi.sf_render_config:
        c = abi.sf_render_config()
        c.integrator = {"megakernel": 0, "wavefront": 1}[self.integrator]
        c.width, c.height, c.samples_per_pixel = self.width, self.height, self.samples_per_pixel
        c.max_bounces, c.max_steps = self.max_bounces, self.max_steps
        c.pixel_tolerance = self.pixel_tolerance
        c.tile_size, c.samples_per_dispatch = self.tile_size, self.samples_per_dispatch
        c.hit_epsilon = self.hit_epsilon
        return c


# ---------------------------------------------------------------------------- scene files
def _rgb(c):
    """Color::Kelvin(K) / Color::Linear((r, g, b)) as RON values, or a bare triple."""
    from . import ron

    if isinstance(c, ron.Tuple) and c.name == "Kelvin":
        return kelvin_to_linear(float(c.items[0]))
    if isinstance(c, ron.Tuple) and c.name == "Linear":
        return tuple(ron.vec(c.items[0]))
    return tuple(ron.vec(c))


def _is_none(x):
    from . import ron

    return x is None or (isinstance(x, ron.Unit) and x.name == "None")


def _ramp_from_ron(r) -> Ramp:
    """Ramp (palette.rs:74-100) with its serde defaults."""
    from . import ron

    if _is_none(r) or r is None:
        return Ramp()
    interp = r.get("interpolation")
    return Ramp(stops=[tuple(ron.vec(x)) for x in r.get("stops", [])] or Ramp().stops,
                positions=[float(x) for x in r.get("positions", [])], cyclic=bool(r.get("cyclic", False)),
                frequency=float(r.get("frequency", 1.0)), phase=float(r.get("phase", 0.0)),
                gamma=float(r.get("gamma", 1.0)), smooth=isinstance(interp, ron.Unit) and interp.name == "Smooth")


def _orbit_from_ron(o) -> OrbitColoring:
    """OrbitColoring (material.rs:18-40), serde(default)."""
    from . import ron

    return OrbitColoring(traps=tuple(float(x) for x in ron.vec(o.get("traps", (1.0, 0.0, 0.0, 0.0)))),
                         iterations=float(o.get("iterations", 0.0)), normal=float(o.get("normal", 0.0)),
                         logarithmic=float(o.get("logarithmic", 0.0)))


def _coloring_from_ron(c):
    """Coloring::{None, Trap{slot, ramp}, Orbit{channels, ramp}} (material.rs:12-16)."""
    if _is_none(c):
        return None
    if isinstance(c, dict) and c.get("__name__") == "Trap":
        return Coloring(int(c["slot"]), _ramp_from_ron(c.get("ramp")))
    if isinstance(c, dict) and c.get("__name__") == "Orbit":
        return Coloring(6, _ramp_from_ron(c.get("ramp")), orbit=_orbit_from_ron(c.get("channels", {})))
    raise ValueError(f"colouring {c!r} is not on this path")


def _optics_from_ron(o):
    """Option<Optics> (optics.rs:7-38)."""
    from . import ron

    if _is_none(o):
        return None
    return Optics(opacity=float(o["opacity"]), transmission=float(o["transmission"]), ior=float(o["ior"]),
                  thin_walled=bool(o["thin_walled"]), absorption_color=tuple(ron.vec(o["absorption_color"])),
                  absorption_distance=float(o["absorption_distance"]), subsurface=float(o["subsurface"]),
                  subsurface_color=tuple(ron.vec(o["subsurface_color"])),
                  subsurface_radius=float(o["subsurface_radius"]))


def _detail_from_ron(d):
    """Option<FinishDetail> (material.rs:200-224)."""
    from . import ron

    if _is_none(d):
        return None
    pattern = d["pattern"].name if isinstance(d["pattern"], ron.Unit) else str(d["pattern"])
    return FinishDetail(pattern=pattern, seed=int(d["seed"]), scale=float(d["scale"]), strength=float(d["strength"]),
                        bump=float(d["bump"]), roughness_delta=float(d["roughness_delta"]),
                        tint=tuple(ron.vec(d["tint"])))


def _texture_from_ron(t):
    """Option<FractalTexture> (texture.rs:62-136) with its serde defaults."""
    from . import ron

    if _is_none(t):
        return None
    if not _is_none(t.get("planar")):
        raise ValueError("planar textures are not on this path")
    ch = t["channel"]
    if isinstance(ch, (ron.Unit, str)):
        channel = {"Distance": ("distance",), "Iterations": ("iterations",)}[getattr(ch, "name", ch)]
    elif ch.get("__name__") == "Trap":
        channel = ("trap", int(ch["slot"]))
    else:
        channel = ("orbit", _orbit_from_ron(ch.get("channels", {})))
    fan, mask = t.get("fan"), t.get("mask")
    return FractalTexture(
        graph=Graph.from_ron_value(t["graph"]), channel=channel, scale=float(t["scale"]),
        offset=tuple(ron.vec(t["offset"])), rotation=tuple(ron.vec(t["rotation"])), octaves=int(t["octaves"]),
        contrast=float(t["contrast"]), ramp=_ramp_from_ron(t.get("ramp")), strength=float(t["strength"]),
        roughness=float(t["roughness"]), bump=float(t["bump"]), parallax=float(t.get("parallax", 0.0)),
        parallax_steps=int(t.get("parallax_steps", 8)),
        fan=None if _is_none(fan) else (*[float(x) for x in ron.vec(fan["period"])], int(fan["rays"])),
        mask=None if _is_none(mask) else (int(mask["slot"]), float(mask["value"]), float(mask["width"])))


def _material_from_ron(m) -> "Material":
    """Material (material.rs:136-158): colouring, texture, surface variation, finishes
    (Finish, material.rs:160-176) and optics."""
    from . import ron

    sv = m.get("surface")
    surface = None if _is_none(sv) else SurfaceVariation(slot=int(sv["slot"]), roughness=tuple(ron.vec(sv["roughness"])),
                                                        metallic=tuple(ron.vec(sv["metallic"])))
    finishes = [Finish(albedo=tuple(ron.vec(f["albedo"])), roughness=float(f["roughness"]),
                       metallic=float(f["metallic"]), specular=float(f["specular"]),
                       emission=tuple(ron.vec(f.get("emission", (0.0, 0.0, 0.0)))),
                       detail=_detail_from_ron(f.get("detail")), optics=_optics_from_ron(f.get("optics")))
                for f in (m.get("finishes") or [])]
    return Material(albedo=tuple(ron.vec(m["albedo"])), roughness=float(m["roughness"]),
                    metallic=float(m["metallic"]), specular=float(m["specular"]),
                    optics=_optics_from_ron(m.get("optics")), finishes=finishes, surface=surface,
                    coloring=_coloring_from_ron(m.get("coloring")), texture=_texture_from_ron(m.get("texture")))


def scene_from_ron_value(v) -> Scene:
    """Scene (crates/syfrack-core/src/scene/mod.rs) from a parsed scenes/*.ron value: the
    graph fractal, Orbit/Free camera, Sun/Environment/Area/Projector/Tube lights, the
    material (colouring, surface variation, volumetric texture, finishes with their
    details and optics, optics), the height fog, cavity darkness and the seed. Creation
    scenes, planar textures and HDRI panoramas (files) are not read and raise
    ValueError."""
    from . import ron

    if "fractal" not in v:
        raise ValueError("creation scenes (a creation graph instead of a fractal) are not on this path")
    frac = v["fractal"]
    if not (isinstance(frac, ron.Tuple) and frac.name == "Graph"):
        raise ValueError("only graph fractals are on this path")
    graph = Graph.from_ron_value(frac.items[0])
    cam_v = v["camera"]
    mode = cam_v["mode"]
    if mode["__name__"] == "Orbit":
        cam = Camera.orbit(tuple(ron.vec(mode["point"])), float(mode["distance"]), float(mode["azimuth"]),
                           float(mode["elevation"]), float(mode.get("roll", 0.0)), float(cam_v["focal_mm"]))
    else:
        cam = Camera(tuple(ron.vec(mode["position"])), tuple(ron.vec(mode["target"])), float(mode.get("roll", 0.0)),
                     float(cam_v["focal_mm"]))
    cam.f_number = float(cam_v.get("f_number", 0.0))
    cam.focus_distance = float(cam_v.get("focus_distance", 3.0))
    lights = []
    for l in v.get("lights", []):
        kind = l["__name__"]
        if kind == "Sun":
            lights.append(SunLight(tuple(ron.vec(l["direction"])), _rgb(l["color"]), float(l["intensity"]),
                                   float(l["angular_size"])))
        elif kind == "Environment":
            if float(l.get("rotation", 0.0)) != 0.0:
                pass  # a vertical gradient does not change under rotation about y
            lights.append(EnvironmentLight(_rgb(l["zenith"]), _rgb(l["horizon"]), _rgb(l["ground"]),
                                           float(l["intensity"])))
        elif kind == "Area":
            lights.append(AreaLight(tuple(ron.vec(l["position"])), tuple(ron.vec(l["normal"])),
                                    tuple(ron.vec(l["size"])), _rgb(l["color"]), float(l["intensity"])))
        elif kind == "Projector":
            lights.append(ProjectorLight(tuple(ron.vec(l["position"])), tuple(ron.vec(l["normal"])),
                                         tuple(ron.vec(l["size"])), _rgb(l["color"]), float(l["intensity"]),
                                         float(l["inner_angle"]), float(l["outer_angle"])))
        elif kind == "Tube":
            lights.append(TubeLight(tuple(ron.vec(l["start"])), tuple(ron.vec(l["end"])), float(l["radius"]),
                                    _rgb(l["color"]), float(l["intensity"])))
        else:
            raise ValueError(f"{kind} lights are not on this path")
    mat = _material_from_ron(v["material"])
    atm = v.get("atmosphere", {})
    fog = None
    if float(atm.get("fog_density", 0.0)) > 0.0:
        fog = Fog(density=float(atm["fog_density"]), color=tuple(ron.vec(atm.get("fog_color", (1.0, 1.0, 1.0)))),
                  height=float(atm.get("fog_height", 0.0)), falloff=float(atm.get("fog_falloff", 1.0)),
                  anisotropy=float(atm.get("anisotropy", 0.0)))
    return Scene(graph=graph, camera=cam, material=mat, lights=lights, seed=int(v.get("seed", 0)),
                 cavity_darkness=float(atm.get("cavity_darkness", 0.0)), fog=fog)

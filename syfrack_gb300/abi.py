"""ctypes mirror of include/syfrack_gpu.h (the C ABI of libsyfrack_gpu.so)."""
from __future__ import annotations

import ctypes as C

SF_OK = 0
STATUS_NAMES = {
    0: "SF_OK", 1: "SF_ERR_INVALID", 2: "SF_ERR_GRAPH", 3: "SF_ERR_UNSUPPORTED",
    4: "SF_ERR_CUDA", 5: "SF_ERR_OOM", 6: "SF_ERR_TIMEOUT", 7: "SF_ERR_BUDGET",
    8: "SF_ERR_IO", 9: "SF_ERR_CHECKPOINT", 10: "SF_ERR_WAVEFRONT", 11: "SF_ERR_NO_DEVICE", 12: "SF_ERR_BUSY",
}

# enum sf_node_kind: the order of NodeKind (crates/syfrack-core/src/scene/graph/mod.rs:105-257)
NODE_KINDS = [
    "Input", "Output", "Translate", "Rotate", "Scale", "ScaleAxes", "Mirror", "BoxFold",
    "BoxFoldAxes", "SphereInversion", "SphereFold", "Abs", "MengerFold", "Kaleido", "Power",
    "AddOrigin", "AddSeed", "AddConstant", "Twist", "Bend", "Tile", "RepeatFinite", "Iterate",
    "Trap", "Sphere", "Torus", "Cylinder", "Box", "RoundBox", "Rock", "Plane", "NormFence",
    "BulbFence", "MaterialTag", "Bounded", "Instances", "Union", "Intersection", "Subtraction",
    "SmoothUnion", "SmoothIntersection",
]
KIND_ID = {k: i for i, k in enumerate(NODE_KINDS)}
MEASURES = ["Norm", "AxisX", "AxisY", "AxisZ", "PlaneY", "AngleXY", "AngleXZ", "AngleYZ", "LogNorm"]
TRAP_MODES = ["Minimum", "Maximum", "Last"]
FORMS = {0: "generic", 1: "bulb", 2: "box", 3: "menger"}

SF_MAX_LIGHTS = 8          # lights inline in sf_scene_desc
SF_MAX_SCENE_LIGHTS = 96   # MAX_LIGHTS (light.rs:7): the rest through light_list (ABI 1.6)
SF_MAX_FINISHES = 8
INTEGRATOR_MEGAKERNEL = 0
INTEGRATOR_WAVEFRONT = 1


class sf_node(C.Structure):
    _fields_ = [("id", C.c_uint32), ("kind", C.c_uint32), ("enabled", C.c_uint32),
                ("body_offset", C.c_uint32), ("body_len", C.c_uint32),
                ("u", C.c_uint32 * 3), ("f", C.c_float * 8)]


class sf_link(C.Structure):
    _fields_ = [("from_node", C.c_uint32), ("from_port", C.c_uint32),
                ("to_node", C.c_uint32), ("to_port", C.c_uint32)]


class sf_placement(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("angles", C.c_float * 3), ("scale", C.c_float * 3)]


class sf_graph_desc(C.Structure):
    _fields_ = [("nodes", C.POINTER(sf_node)), ("node_count", C.c_uint32),
                ("links", C.POINTER(sf_link)), ("link_count", C.c_uint32),
                ("body_ids", C.POINTER(C.c_uint32)), ("body_id_count", C.c_uint32),
                ("safety", C.c_float), ("bounding_radius_hint", C.c_float),
                ("placements", C.POINTER(sf_placement)), ("placement_count", C.c_uint32)]


class sf_de_sample(C.Structure):
    _fields_ = [("distance", C.c_float), ("traps", C.c_float * 4),
                ("iterations", C.c_uint32), ("material", C.c_uint32)]


class sf_graph_info(C.Structure):
    _fields_ = [("step_scale", C.c_float), ("lipschitz", C.c_float), ("trap_scales", C.c_float * 4),
                ("iteration_product", C.c_uint32), ("form", C.c_uint32), ("op_count", C.c_uint32),
                ("bounding_radius_hint", C.c_float),
                # ABI 1.4
                ("exact_union_leaves", C.c_uint32)]


class sf_camera(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("forward", C.c_float * 3), ("right", C.c_float * 3),
                ("up", C.c_float * 3), ("tan_half_fov", C.c_float), ("aspect", C.c_float),
                ("lens_radius", C.c_float), ("focus_distance", C.c_float)]


class sf_material(C.Structure):
    _fields_ = [("albedo", C.c_float * 3), ("roughness", C.c_float), ("metallic", C.c_float),
                ("specular", C.c_float), ("emission", C.c_float * 3)]


SF_LIGHT_AREA, SF_LIGHT_SUN, SF_LIGHT_ENVIRONMENT, SF_LIGHT_HDRI, SF_LIGHT_PROJECTOR, SF_LIGHT_TUBE = 0, 1, 2, 3, 4, 5
SF_MAX_RAMP_STOPS = 16


class sf_area_light(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("edge_u", C.c_float * 3), ("edge_v", C.c_float * 3),
                ("radiance", C.c_float * 3), ("kind", C.c_uint32), ("direction", C.c_float * 3),
                ("angular_size", C.c_float), ("zenith", C.c_float * 3), ("horizon", C.c_float * 3),
                ("ground", C.c_float * 3), ("environment", C.c_void_p), ("rotation", C.c_float)]


sf_light = sf_area_light


class sf_coloring(C.Structure):
    _fields_ = [("slot", C.c_uint32), ("stop_count", C.c_uint32), ("stops", (C.c_float * 4) * SF_MAX_RAMP_STOPS),
                ("cyclic", C.c_uint32), ("smooth", C.c_uint32), ("positioned", C.c_uint32),
                ("frequency", C.c_float), ("phase", C.c_float), ("gamma", C.c_float)]


class sf_fog(C.Structure):
    _fields_ = [("density", C.c_float), ("height", C.c_float), ("falloff", C.c_float),
                ("anisotropy", C.c_float), ("color", C.c_float * 3)]


class sf_finish_detail(C.Structure):
    _fields_ = [("pattern", C.c_uint32), ("seed", C.c_uint32), ("scale", C.c_float), ("strength", C.c_float),
                ("bump", C.c_float), ("roughness_delta", C.c_float), ("tint", C.c_float * 3)]


class sf_orbit_coloring(C.Structure):
    _fields_ = [("traps", C.c_float * 4), ("iterations", C.c_float), ("normal", C.c_float),
                ("logarithmic", C.c_float)]


class sf_optics(C.Structure):
    _fields_ = [("enabled", C.c_uint32), ("opacity", C.c_float), ("transmission", C.c_float), ("ior", C.c_float),
                ("thin_walled", C.c_uint32), ("absorption_color", C.c_float * 3),
                ("absorption_distance", C.c_float), ("subsurface", C.c_float),
                ("subsurface_color", C.c_float * 3), ("subsurface_radius", C.c_float)]


class sf_texture(C.Structure):
    _fields_ = [("graph", C.c_void_p), ("channel", C.c_uint32), ("orbit", sf_orbit_coloring),
                ("scale", C.c_float), ("offset", C.c_float * 3), ("rotation", C.c_float * 3),
                ("octaves", C.c_uint32), ("contrast", C.c_float), ("ramp", sf_coloring),
                ("strength", C.c_float), ("roughness", C.c_float), ("bump", C.c_float), ("parallax", C.c_float),
                ("parallax_steps", C.c_uint32), ("fan", C.c_uint32), ("fan_period", C.c_float * 2),
                ("fan_rays", C.c_uint32), ("mask", C.c_uint32), ("mask_slot", C.c_uint32),
                ("mask_value", C.c_float), ("mask_width", C.c_float)]


class sf_scene_desc(C.Structure):
    _fields_ = [("camera", sf_camera), ("material", sf_material),
                ("finishes", sf_material * SF_MAX_FINISHES), ("finish_count", C.c_uint32),
                ("lights", sf_area_light * SF_MAX_LIGHTS), ("light_count", C.c_uint32),
                ("variation_slot", C.c_uint32), ("variation_enabled", C.c_uint32),
                ("variation_roughness", C.c_float * 2), ("variation_metallic", C.c_float * 2),
                ("cavity_darkness", C.c_float), ("seed", C.c_uint64), ("coloring", sf_coloring),
                ("fog", sf_fog),
                # ABI 1.3
                ("details", sf_finish_detail * SF_MAX_FINISHES), ("dune_wind", C.c_float),
                ("coloring_orbit", sf_orbit_coloring), ("optics", sf_optics * (SF_MAX_FINISHES + 1)),
                ("texture", sf_texture),
                # ABI 1.6
                ("light_list", C.POINTER(sf_area_light)), ("light_list_count", C.c_uint32)]


class sf_render_config(C.Structure):
    _fields_ = [("integrator", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("samples_per_pixel", C.c_uint32), ("max_bounces", C.c_uint32),
                ("max_steps", C.c_uint32), ("pixel_tolerance", C.c_float),
                ("tile_size", C.c_uint32), ("samples_per_dispatch", C.c_uint32),
                ("hit_epsilon", C.c_float)]


class sf_tile(C.Structure):
    _fields_ = [("x", C.c_uint32), ("y", C.c_uint32), ("w", C.c_uint32), ("h", C.c_uint32),
                ("done", C.c_uint32)]

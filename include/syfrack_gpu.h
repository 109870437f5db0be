/*
 * syfrack_gpu.h -- C ABI of the GB300 (sm_103a) distance-estimator path.
 *
 * This header is the drop-in boundary for SyFrack's DE / sphere-trace /
 * escape-time hot path. Each entry point names the reference interface it
 * replaces (paths are relative to the SyFrack source tree). All functions
 * return sf_status (SF_OK == 0); handles are opaque; buffers passed as plain
 * pointers are caller-owned host memory unless the name says "device".
 * No C++ exception crosses this boundary. One thread drives one handle.
 *
 * Arithmetic is IEEE binary32 on the device, like the reference's glam Vec3
 * and WGSL f32 (crates/syfrack-core/src/scene/graph/eval.rs and the WGSL shaders).
 */
#ifndef SYFRACK_GPU_H
#define SYFRACK_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t sf_status;
enum {
    SF_OK = 0,
    SF_ERR_INVALID = 1,      /* bad argument (null pointer, size, range)            */
    SF_ERR_GRAPH = 2,        /* graph fails validation (cycle, ports, bounds)       */
    SF_ERR_UNSUPPORTED = 3,  /* valid graph/scene using a feature not built on GPU  */
    SF_ERR_CUDA = 4,         /* CUDA runtime error (message in sf_last_error)       */
    SF_ERR_OOM = 5,          /* device allocation failed                            */
    SF_ERR_TIMEOUT = 6,      /* bounded wait expired (renderer.rs:236 DISPATCH_TIMEOUT) */
    SF_ERR_BUDGET = 7,       /* HBM admission budget exceeded                       */
    SF_ERR_IO = 8,           /* checkpoint file could not be read or written        */
    SF_ERR_CHECKPOINT = 9,   /* checkpoint corrupt or from another producer         */
    SF_ERR_WAVEFRONT = 10,   /* wavefront invariant word non-zero (wavefront.rs:414-417) */
    SF_ERR_NO_DEVICE = 11,   /* no CUDA device / extension not usable               */
    SF_ERR_BUSY = 12,        /* request still queued or running                     */
};

/* Human-readable name of a status code. Never NULL. */
const char* sf_status_string(sf_status status);
/* Message of the last error on the calling thread ("" if none). */
const char* sf_last_error(void);
/* ABI version: (major << 16) | minor. */
uint32_t sf_abi_version(void);

/* ------------------------------------------------------------------ graph
 * The form graph of crates/syfrack-core/src/scene/graph/mod.rs:444-451
 * (Graph{nodes, links, safety, bounding_radius_hint}) passed flat.
 * Node kinds keep the order of NodeKind (graph/mod.rs:105-257).
 */
enum sf_node_kind {
    SF_NODE_INPUT = 0, SF_NODE_OUTPUT, SF_NODE_TRANSLATE, SF_NODE_ROTATE,
    SF_NODE_SCALE, SF_NODE_SCALE_AXES, SF_NODE_MIRROR, SF_NODE_BOX_FOLD,
    SF_NODE_BOX_FOLD_AXES, SF_NODE_SPHERE_INVERSION, SF_NODE_SPHERE_FOLD,
    SF_NODE_ABS, SF_NODE_MENGER_FOLD, SF_NODE_KALEIDO, SF_NODE_POWER,
    SF_NODE_ADD_ORIGIN, SF_NODE_ADD_SEED, SF_NODE_ADD_CONSTANT, SF_NODE_TWIST,
    SF_NODE_BEND, SF_NODE_TILE, SF_NODE_REPEAT_FINITE, SF_NODE_ITERATE,
    SF_NODE_TRAP, SF_NODE_SPHERE, SF_NODE_TORUS, SF_NODE_CYLINDER, SF_NODE_BOX,
    SF_NODE_ROUND_BOX, SF_NODE_ROCK, SF_NODE_PLANE, SF_NODE_NORM_FENCE,
    SF_NODE_BULB_FENCE, SF_NODE_MATERIAL_TAG, SF_NODE_BOUNDED,
    SF_NODE_INSTANCES, SF_NODE_UNION, SF_NODE_INTERSECTION,
    SF_NODE_SUBTRACTION, SF_NODE_SMOOTH_UNION, SF_NODE_SMOOTH_INTERSECTION,
    SF_NODE_KIND_COUNT
};
/* Trap measures and modes: graph/mod.rs:82-101 (Measure, TrapMode). */
enum sf_measure { SF_MEASURE_NORM = 0, SF_MEASURE_AXIS_X, SF_MEASURE_AXIS_Y,
    SF_MEASURE_AXIS_Z, SF_MEASURE_PLANE_Y, SF_MEASURE_ANGLE_XY,
    SF_MEASURE_ANGLE_XZ, SF_MEASURE_ANGLE_YZ, SF_MEASURE_LOG_NORM };
enum sf_trap_mode { SF_TRAP_MINIMUM = 0, SF_TRAP_MAXIMUM, SF_TRAP_LAST };

/*
 * One node. Parameters per kind (f = floats, u = unsigned):
 *   Translate f0..2 offset | Rotate f0..2 angles (deg) | Scale f0 factor
 *   ScaleAxes f0..2 | Mirror f0..2 normal, f3 offset | BoxFold f0 limit
 *   BoxFoldAxes f0..2 limit, u0..2 x/y/z | SphereInversion f0 radius f1 min_radius
 *   SphereFold f0 min_radius f1 fixed_radius | Abs u0..2 | MengerFold f0 scale f1..3 offset
 *   Kaleido u0 planes f0 phase (deg) | Power f0 power | AddSeed f0..2 multiplier
 *   AddConstant f0..2 multiplier f3..5 julia | Twist/Bend f0 rate | Tile f0..2 period
 *   RepeatFinite f0..2 period u0..2 count | Iterate u0 iterations f0 bailout,
 *     body = body_ids[body_offset .. body_offset+body_len]
 *   Trap u0 slot u1 measure u2 mode f0 scale | Sphere f0 radius | Torus f0 radius f1 tube
 *   Cylinder f0 radius f1 half_height | Box f0..2 half | RoundBox f0..2 half f3 radius
 *   Rock f0..2 half f3 erosion u0 seed | Plane f0..2 normal f3 offset | NormFence f0 inset
 *   MaterialTag u0 index | Bounded f0..2 half f3 margin | SmoothUnion/Intersection f0 k
 *   Instances f0..2 half f3 margin u0 first placement u1 placement count
 *     (placements[u0 .. u0+u1] of the descriptor; graph/mod.rs:241-246)
 */
typedef struct sf_node {
    uint32_t id;
    uint32_t kind;      /* enum sf_node_kind */
    uint32_t enabled;   /* 0 = disabled (Node.enabled) */
    uint32_t body_offset;
    uint32_t body_len;
    uint32_t u[3];
    float f[8];
} sf_node;

typedef struct sf_link {           /* Link{from:(node,port), to:(node,port)} */
    uint32_t from_node, from_port, to_node, to_port;
} sf_link;

/* Placement{position, angles (degrees, glam intrinsic XYZ), scale} (graph/mod.rs:26-30):
 * one independently transformed copy of an Instances node's template. */
typedef struct sf_placement {
    float position[3];
    float angles[3];
    float scale[3];
} sf_placement;

typedef struct sf_graph_desc {
    const sf_node* nodes;
    uint32_t node_count;
    const sf_link* links;
    uint32_t link_count;
    const uint32_t* body_ids;      /* concatenated Iterate bodies */
    uint32_t body_id_count;
    float safety;
    float bounding_radius_hint;
    const sf_placement* placements;/* concatenated Instances placements (may be NULL) */
    uint32_t placement_count;
} sf_graph_desc;

/* DeSample (crates/syfrack-core/src/scene/fractal.rs:18-27). */
typedef struct sf_de_sample {
    float distance;
    float traps[4];      /* normalised min(trap/scale, 1); 1 when unwritten */
    uint32_t iterations; /* clamped to the iteration product */
    uint32_t material;
} sf_de_sample;

/* Constants derived on the host, as Uniforms::from_fractal (uniforms.rs:183-189). */
typedef struct sf_graph_info {
    float step_scale;            /* safety / lipschitz(hint): eval.rs:879-881 */
    float lipschitz;             /* eval.rs:828-849 */
    float trap_scales[4];        /* eval.rs:853-877 */
    uint32_t iteration_product;  /* validate.rs:112-141 */
    uint32_t form;               /* SF_FORM_*: specialised device code path */
    uint32_t op_count;           /* length of the lowered device program */
    float bounding_radius_hint;
    /* ABI 1.4: the leaves of the exact union branch-and-bound (graph_wgsl.rs:1112-1154)
     * when the Output's input is a union over 2 to 32 leaves and the graph has a
     * skippable Bounded or Instances node, else 0. sf_de_probe and the preview search
     * unions of three or more leaves; every kernel's sample is the whole program's. */
    uint32_t exact_union_leaves;
} sf_graph_info;
enum { SF_FORM_GENERIC = 0, SF_FORM_BULB = 1, SF_FORM_BOX = 2, SF_FORM_MENGER = 3 };

typedef struct sf_context sf_context;
typedef struct sf_graph sf_graph;
typedef struct sf_environment sf_environment;  /* an HDRI panorama on the device */

/* Device context: owns the CUDA stream, the module and the HBM admission
 * budget (0 = 90% of free memory). Replaces GpuContext::new (gpu.rs:15-36)
 * and Renderer::new (renderer.rs:328). */
sf_status sf_context_create(int device, uint64_t hbm_budget_bytes, sf_context** out);
sf_status sf_context_destroy(sf_context* ctx);
/* The cudaStream_t every call of this context is ordered on. */
sf_status sf_context_stream(sf_context* ctx, void** stream_out);
/* Bytes currently admitted against the budget, and the budget. */
sf_status sf_context_memory(sf_context* ctx, uint64_t* used, uint64_t* budget);

/* Validates and lowers a graph. Replaces graph_wgsl::compile (graph_wgsl.rs:949-952)
 * + ParamLayout::pack; the lowered program lives in device memory. */
/* Graph::validate (scene/graph/validate.rs:146-330) and the derived constants, on the
 * host only (no context, no device): the checks sf_graph_compile makes before lowering. */
sf_status sf_graph_validate(const sf_graph_desc* desc, sf_graph_info* out);
sf_status sf_graph_compile(sf_context* ctx, const sf_graph_desc* desc, sf_graph** out);

/* EnvironmentMap::from_rgb (crates/syfrack-render/src/environment.rs:271-366): an
 * equirectangular linear RGB panorama (width*height*3 floats, row 0 at the zenith,
 * finite, at most 8192x4096) reduced in solid angle to at most 2048x1024 texels, each
 * with the cumulative luminance x solid-angle distribution of its importance sampling
 * (the bilinear halo included). sf_environment_build runs on the host only: it writes
 * out_width*out_height texels (rgb, cdf) when `texels` is not NULL; pass NULL first to
 * learn the size. sf_environment_create keeps the texels on the device. */
sf_status sf_environment_build(const float* rgb, uint32_t width, uint32_t height, float* texels,
                               uint32_t* out_width, uint32_t* out_height, int* uniform);
sf_status sf_environment_create(sf_context* ctx, const float* rgb, uint32_t width, uint32_t height,
                                sf_environment** out);
sf_status sf_environment_destroy(sf_environment* env);
sf_status sf_graph_info_get(const sf_graph* graph, sf_graph_info* out);
/* Value edits without re-lowering: same topology, new floats (topology_key semantics,
 * graph/mod.rs:397-425). Fails with SF_ERR_GRAPH if the topology changed. */
sf_status sf_graph_update(sf_graph* graph, const sf_graph_desc* desc);
sf_status sf_graph_destroy(sf_graph* graph);

/* Batched DE evaluation at n points (xyz interleaved, host memory) -> n samples.
 * Replaces Renderer::probe_distances (renderer.rs:645-648) / de_probe.wgsl:9-17. */
sf_status sf_de_probe(sf_graph* graph, const float* xyz, size_t n, sf_de_sample* out);
/* Same on device buffers, asynchronous on the context stream: SoA x,y,z in;
 * distance[n], traps[4n] (slot-major: traps[k*n+i]), iterations[n], material[n] out. */
sf_status sf_de_probe_device(sf_graph* graph, const float* x, const float* y, const float* z,
                             size_t n, float* distance, float* traps, uint32_t* iterations,
                             uint32_t* material);

/* ------------------------------------------------------------------ scene */
/* CameraBasis (crates/syfrack-core/src/scene/camera.rs:44-56), as packed in
 * Uniforms.camera (uniforms.rs:754-766). */
typedef struct sf_camera {
    float origin[3], forward[3], right[3], up[3];
    float tan_half_fov, aspect, lens_radius, focus_distance;
} sf_camera;
/* Material / Finish (material.rs:136-170). */
typedef struct sf_material {
    float albedo[3];
    float roughness, metallic, specular;
    float emission[3];
} sf_material;
/* One light of Scene.lights (light.rs:63-120), in scene order (next-event sampling
 * visits them in that order). kind selects the fields:
 *   Area (GpuLight, uniforms.rs:671-713): centre, full width edge (edge_u), full
 *     height edge (edge_v), radiance = color * intensity;
 *   Sun: direction toward the sun, angular_size = full angular diameter in degrees,
 *     radiance = irradiance (color * intensity);
 *   Environment: zenith, horizon and ground radiance (colors * intensity);
 *   Hdri: an equirectangular panorama (below), intensity in radiance[0], rotation;
 *   Projector (ABI 1.5; Light::Projector, uniforms.rs:671-716): an Area light (centre,
 *     edges, radiance) whose emission about its normal is full within direction[0]
 *     degrees (the inner angle), none beyond direction[1] degrees (the outer angle,
 *     0 < outer < 90, inner <= outer) and blended between (lights.wgsl:11-16);
 *   Tube (ABI 1.5; Light::Tube, uniforms.rs:717-729): a capsule from center (the
 *     start) to edge_u (the end point), radius edge_v[0], radiance = color * intensity. */
enum {
    SF_LIGHT_AREA = 0, SF_LIGHT_SUN = 1, SF_LIGHT_ENVIRONMENT = 2, SF_LIGHT_HDRI = 3,
    SF_LIGHT_PROJECTOR = 4, SF_LIGHT_TUBE = 5
};
typedef struct sf_area_light {
    float center[3], edge_u[3], edge_v[3], radiance[3];
    uint32_t kind;
    float direction[3];
    float angular_size;
    float zenith[3], horizon[3], ground[3];
    /* Hdri: the panorama (sf_environment_create), radiance[0] = intensity, rotation in
     * degrees about +y. The panorama must outlive the sessions that render with it. */
    sf_environment* environment;
    float rotation;
} sf_area_light;
typedef sf_area_light sf_light;
#define SF_MAX_LIGHTS 8          /* lights held inline in sf_scene_desc */
#define SF_MAX_SCENE_LIGHTS 96   /* Scene::lights bound, MAX_LIGHTS (light.rs:7); ABI 1.6 */
#define SF_MAX_FINISHES 8
#define SF_MAX_RAMP_STOPS 16
/* Material.coloring (material.rs:100-130) as GpuColoring (uniforms.rs:193-215): the
 * ramp (palette.rs:74-100) multiplies the albedo by its value at the sample's trap
 * slot (0..3), iteration fraction (4), n.y * 0.5 + 0.5 (5) or the orbit mix of
 * sf_scene_desc.coloring_orbit (6, ABI 1.3); 0xffff = none. */
typedef struct sf_coloring {
    uint32_t slot;
    uint32_t stop_count;              /* 0: white */
    float stops[SF_MAX_RAMP_STOPS][4];/* rgb, position (evenly spaced unless positioned) */
    uint32_t cyclic, smooth, positioned;
    float frequency, phase, gamma;
} sf_coloring;
/* Height fog, Atmosphere (atmosphere.rs:7-28) as GpuAtmosphere.a/b (uniforms.rs:217-227):
 * extinction `density` at and below `height`, decaying as exp(-(y - height) * falloff)
 * above it; Henyey-Greenstein `anisotropy` (-0.99..0.99); scattering albedo `color`.
 * density 0 = no fog. A fog scene issues one shadow segment per area light for its
 * line integral besides the surface's: at most 8 shadow segments per bounce. */
typedef struct sf_fog {
    float density, height, falloff, anisotropy;
    float color[3];
} sf_fog;
/* FinishDetail (material.rs:200-212) as GpuFinish.detail_* (uniforms.rs:797-815): a
 * world-space pattern (finish_detail.wgsl) that tints the albedo, shifts roughness and
 * bends the shading normal. pattern: 0 = none, else FinishPattern's order from 1
 * (VeinedStone, Patina, BrushedMetal, Basalt, Ripples, Rosettes, CoastalRock, Sand,
 * Dust, Concrete, WeatheredConcrete) to 12 (WetConcrete). Concrete kinds (10-12) add
 * the Oren-Nayar rough diffuse lobe. */
typedef struct sf_finish_detail {
    uint32_t pattern, seed;
    float scale, strength, bump, roughness_delta;
    float tint[3];
} sf_finish_detail;
/* OrbitColoring (material.rs:18-56): a signed mix of the four traps, the iteration
 * fraction and n.y * 0.5 + 0.5, optionally log-remapped (logarithmic > 0). */
typedef struct sf_orbit_coloring {
    float traps[4];
    float iterations, normal, logarithmic;
} sf_orbit_coloring;
/* Optics (optics.rs:7-21) as GpuOptics (uniforms.rs:95-122): stochastic coverage
 * (opacity), a rough dielectric interface (transmission probability, ior, thin-walled
 * sheet) and a homogeneous interior medium (Beer-Lambert absorption reaching
 * absorption_color after absorption_distance; subsurface scattering of the given
 * albedo with mean free path subsurface_radius / subsurface). enabled 0 = opaque. */
typedef struct sf_optics {
    uint32_t enabled;
    float opacity, transmission, ior;
    uint32_t thin_walled;
    float absorption_color[3], absorption_distance;
    float subsurface, subsurface_color[3], subsurface_radius;
} sf_optics;
/* FractalTexture (texture.rs:62-100) as GpuTexture (uniforms.rs:316-380): a volumetric
 * texture evaluated by a second compiled graph (texture.wgsl, pattern.wgsl:2-49) on
 * surfaces without a MaterialTag. channel: 0-3 trap, 4 iteration fraction, 6 signed
 * distance, 7 orbit mix (orbit). The ramp colours the value (its slot is unused). The
 * graph must outlive the sessions that render with it. */
typedef struct sf_texture {
    sf_graph* graph;
    uint32_t channel;
    sf_orbit_coloring orbit;
    float scale, offset[3], rotation[3];  /* rotation: Euler XYZ in degrees */
    uint32_t octaves;                     /* 1..4 */
    float contrast;
    sf_coloring ramp;
    float strength, roughness, bump;      /* albedo, roughness and relief effects */
    float parallax;                       /* depth in texture units, 0 = none */
    uint32_t parallax_steps;              /* 4..32 */
    uint32_t fan;                         /* FanMapping: staggered fans on world XZ */
    float fan_period[2];
    uint32_t fan_rays;
    uint32_t mask;                        /* TextureMask: only where trap `mask_slot` is near mask_value */
    uint32_t mask_slot;
    float mask_value, mask_width;
} sf_texture;
typedef struct sf_scene_desc {
    sf_camera camera;
    sf_material material;                 /* index 0: the global surface */
    sf_material finishes[SF_MAX_FINISHES];/* MaterialTag 1..8 */
    uint32_t finish_count;
    sf_area_light lights[SF_MAX_LIGHTS];
    uint32_t light_count;
    /* SurfaceVariation (uniforms.rs:485-495): trap slot drives roughness/metallic. */
    uint32_t variation_slot, variation_enabled;
    float variation_roughness[2], variation_metallic[2];
    float cavity_darkness;                /* atmosphere.b.w, 0 = off */
    uint64_t seed;                        /* Scene.seed; the device uses lo ^ hi */
    sf_coloring coloring;                 /* slot 0xffff (or no stops): no colouring */
    sf_fog fog;
    /* ABI 1.3: the rest of make_surface (pathtrace.wgsl:271-386) and the optics of
     * radiance (:833-1105). Zeroed fields keep the 1.2 behaviour. */
    sf_finish_detail details[SF_MAX_FINISHES]; /* FinishDetail of finish i (MaterialTag i+1) */
    float dune_wind;                      /* Dunes.wind_direction in degrees (Sand detail) */
    sf_orbit_coloring coloring_orbit;     /* channels of coloring.slot 6 (Coloring::Orbit) */
    sf_optics optics[SF_MAX_FINISHES + 1];/* 0: Material.optics; i: finish i's optics */
    sf_texture texture;                   /* Material.texture; graph NULL = none */
    /* ABI 1.6: a scene of up to SF_MAX_SCENE_LIGHTS lights (Scene::validate,
     * scene/mod.rs:512). A non-NULL light_list holds light_list_count lights and
     * replaces lights/light_count; sessions copy it at creation. Sessions take up to
     * 96 lights; batches, the server, previews and exports take SF_MAX_LIGHTS. The
     * wavefront integrator stores at most 8 shadow segments per bounce (one per sky
     * light plus the surface's, and one per emitter in fog); the megakernel traces
     * them as they are issued and has no such bound. */
    const sf_area_light* light_list;
    uint32_t light_list_count;
} sf_scene_desc;

/* RenderConfig (renderer.rs:17-43), validated as RenderConfig::validate (:81-138).
 * hit_epsilon (ABI 1.2) has no field in the reference: 0 keeps the reference's
 * cone-relative hit test radius / t < pixel_cone * pixel_tolerance
 * (pathtrace.wgsl:117-122) for every segment; a value > 0 replaces it with the
 * fixed-epsilon test radius <= hit_epsilon (candidates accepted at the step budget
 * within 4 * hit_epsilon), the rule of a benchmark stated as "epsilon 1e-4". The
 * normal-tap step and bounce offsets keep their pixel-cone formulas either way. */
enum { SF_INTEGRATOR_MEGAKERNEL = 0, SF_INTEGRATOR_WAVEFRONT = 1 };
typedef struct sf_render_config {
    uint32_t integrator;
    uint32_t width, height, samples_per_pixel, max_bounces, max_steps;
    float pixel_tolerance;
    uint32_t tile_size, samples_per_dispatch;
    float hit_epsilon;
} sf_render_config;

/* Tile{x,y,w,h,done} (crates/syfrack-render/src/tiles.rs:4-11). */
typedef struct sf_tile { uint32_t x, y, w, h, done; } sf_tile;


/* ------------------------------------------------------------------ primary rays
 * Primary-ray sphere trace through pixel centres (control.wgsl:266-291 ray set-up,
 * pathtrace.wgsl:78-145 march). rule 0: the reference's cone-relative hit test
 * radius/t < pixel_cone*tolerance; rule 1: fixed epsilon radius <= eps. normal_mode
 * 0: 6-tap central difference, 1: 4-tap tetrahedral (common.wgsl:376-387), both with
 * h = max(t*pixel_cone*0.5, 1e-4)*tolerance. Outputs (host, width*height each):
 * t (-1 on a miss), steps, normal (3 planes: x[], y[], z[]). */
typedef struct sf_primary_desc {
    sf_camera camera;
    uint32_t width, height, max_steps;
    int32_t rule;          /* 0 cone-relative, 1 absolute epsilon */
    int32_t normal_mode;   /* 0 central (6 taps), 1 tetrahedral (4 taps) */
    float eps, t_far, pixel_tolerance;
} sf_primary_desc;
sf_status sf_primary_trace(sf_graph* graph, const sf_primary_desc* desc, float* t_out, uint32_t* steps_out,
                           float* normal_out);

/* ------------------------------------------------------------------ statistics & timing */
typedef struct sf_stats {
    uint64_t de_evals;         /* distance-estimator evaluations */
    uint64_t de_iterations;    /* Iterate loop iterations executed inside them */
    uint64_t segments;         /* march_segment runs: camera, continuation and shadow */
    uint64_t shadow_segments;
    uint64_t steps;            /* primary kernel: march steps; deep zoom: rebases */
    uint64_t launches;         /* kernels launched by this handle */
    double kernel_ms;          /* device time of the timed kernels (profiling on) */
    double trace_ms;           /* of which the trace (march) kernels */
    uint64_t trace_launches;
    uint64_t warp_de_calls;    /* warp-level DE invocations of the trace kernel */
    uint64_t iteration_slots;  /* per invocation: warp max iterations x active lanes */
    uint64_t warp_cycles;      /* trace kernel, profiling level 2: SM cycles of its warps */
    uint64_t tail_cycles;      /* of which after the warp first found the launch's work exhausted */
} sf_stats;
/* Per-kernel CUDA-event timing on the context stream (off by default): 0 off, 1 on,
 * 2 on and the trace kernel also counts warp_de_calls and iteration_slots (a
 * diagnostic instantiation that pays a warp reduction per DE call; with 0 or 1 those
 * two counters stay unchanged). */
sf_status sf_context_set_profiling(sf_context* ctx, int enable);
sf_status sf_context_stats(sf_context* ctx, sf_stats* out);
sf_status sf_context_reset_stats(sf_context* ctx);
/* Measured FP32 FMA throughput of the device (TFLOP/s, FMA = 2 flops): the
 * roofline denominator of the FP32-bound DE kernels. No counterpart in the
 * reference (a diagnostic like its adapter probe, shaders/probe.wgsl). */
sf_status sf_device_fp32_peak(sf_context* ctx, double* tflops);
/* Blocks until the context stream is idle or timeout_ms passes (SF_ERR_TIMEOUT). */
sf_status sf_context_sync(sf_context* ctx, uint32_t timeout_ms);

/* ------------------------------------------------------------------ render sessions
 * RenderSession (crates/syfrack-render/src/session.rs:113-162): progressive
 * accumulation over a TileGrid (tiles.rs:14-90) with samples_per_dispatch samples
 * per dispatch. Film planes follow RenderOutput (renderer.rs:151-164): accum
 * holds sample sums (accum += (L,1) per sample in ascending sample order,
 * pathtrace.wgsl:1243-1245); depth/aux come from sample 0. */
typedef struct sf_session sf_session;
typedef struct sf_progress {
    uint32_t tiles, dispatches, samples_min, samples_max, target;
    uint64_t pixel_samples_done, pixel_samples_total;
    uint32_t status_word;   /* wavefront invariant bits 1/2/4 (wavefront.wgsl:183,:220,:236); 8 = a bounce
                               issued more shadow segments than the arena holds */
} sf_progress;
/* The film planes of wf_commit (wavefront.wgsl:232-260). The volume layer split
 * (pathtrace.wgsl:1197-1199, 1243-1266): a sample's volume part is all its radiance
 * when its camera segment scattered in the fog, else that segment's in-scattered
 * emitter light; volume sums it, moments holds the Welford sums of
 * max(0, delta * (v - new_mean)) in ascending sample order, surface sums radiance -
 * volume; each plane's w is the sample count. Fog scenes keep these planes on the
 * device (48 more bytes per pixel and 16 per path); without fog the volume part is
 * zero: volume and moments read (0, 0, 0, samples) and surface equals accum. Any
 * pointer may be NULL. */
typedef struct sf_film_planes {
    float* accum;   /* 4*width*height: rgb sums and sample count */
    float* depth;   /* width*height */
    float* aux;     /* 4*width*height: normal xyz, steps (-1 on a miss) */
    float* volume;  /* 4*width*height: volume sums and sample count */
    float* moments; /* 4*width*height: volume Welford moments and sample count */
    float* surface; /* 4*width*height: surface sums and sample count */
    float* color;   /* 4*width*height: accum rgb / max(count, 1), alpha 1 (RenderOutput.color) */
} sf_film_planes;

/* Session::new (session.rs:165). The integrator field selects the per-pixel
 * megakernel (pathtrace.wgsl main) or the wavefront stages (wavefront.rs:310-419). */
sf_status sf_session_create(sf_context* ctx, sf_graph* graph, const sf_scene_desc* scene,
                            const sf_render_config* cfg, sf_session** out);
/* Wavefront::dispatch / Renderer::dispatch: `samples` samples of one tile,
 * asynchronous on the context stream (no host wait). */
sf_status sf_session_dispatch(sf_session* s, sf_tile tile, uint32_t samples);
/* RenderSession::step (session.rs:694-877): dispatches least-advanced tiles
 * (TileGrid::next_pending) until budget_ms of wall time is spent or the image
 * reached samples_per_pixel; *done = 1 when complete. Waits for the device. */
sf_status sf_session_step(sf_session* s, uint32_t budget_ms, int* done);
/* Bounded wait for the session's work; returns the invariant word. */
sf_status sf_session_sync(sf_session* s, uint32_t timeout_ms, uint32_t* status_word);
sf_status sf_session_progress(sf_session* s, sf_progress* out);
sf_status sf_session_tiles(sf_session* s, sf_tile* tiles, uint32_t capacity, uint32_t* count);
/* Copies the film planes to host buffers (RenderSession::readback, session.rs:879). */
sf_status sf_session_readback(sf_session* s, sf_film_planes* out);
sf_status sf_session_stats(sf_session* s, sf_stats* out);
/* Checkpoint (session.rs:1194-1346): state + film planes + FNV-1a hash + producer
 * identity, written to a sibling directory and swapped in. Resume refuses a
 * corrupt state or another producer with SF_ERR_CHECKPOINT. */
sf_status sf_session_save(sf_session* s, const char* dir);
sf_status sf_session_resume(sf_context* ctx, sf_graph* graph, const char* dir, sf_session** out);
sf_status sf_session_destroy(sf_session* s);

/* ------------------------------------------------------------------ preview
 * ControlSession (crates/syfrack-render/src/control/mod.rs:172-530): an interactive
 * preview of primary rays through pixel centres on the exact field, marched in
 * resumable quanta of `quantum` DE evaluations per pixel (0 = 128) with no step
 * budget, shaded with the control engine's fixed light (control.wgsl:54-99). No
 * graph is ever compiled: a graph edit (sf_graph_update) or sf_preview_set uploads
 * data; sf_preview_set restarts the image. The machine runs on its own
 * highest-priority stream. */
typedef struct sf_preview sf_preview;
sf_status sf_preview_create(sf_context* ctx, sf_graph* graph, const sf_scene_desc* scene, uint32_t width,
                            uint32_t height, uint32_t quantum, sf_preview** out);
/* set_scene: another graph and/or scene (NULL keeps the current one); restarts. */
sf_status sf_preview_set(sf_preview* p, sf_graph* graph, const sf_scene_desc* scene);
/* tick: polls the previous quantum and submits at most one; never waits for the
 * device. *complete = 1 once every pixel has ended. A non-finite distance fails
 * the preview with SF_ERR_GRAPH. */
sf_status sf_preview_tick(sf_preview* p, int* complete);
/* wait_complete: ticks until complete or timeout_ms (SF_ERR_TIMEOUT); diagnostic. */
sf_status sf_preview_wait(sf_preview* p, uint32_t timeout_ms);
sf_status sf_preview_progress(sf_preview* p, uint32_t* completed_pixels, uint32_t* dispatches);
/* accum = preview colour (1 in w), depth (-1 on a miss), aux = normal and march steps. */
sf_status sf_preview_readback(sf_preview* p, sf_film_planes* out);
/* pick(u, v) in [0, 1]^2: the pixel's depth (<= 0: nothing there) and aux. */
sf_status sf_preview_pick(sf_preview* p, float u, float v, float* depth, float* aux);
sf_status sf_preview_destroy(sf_preview* p);

/* ------------------------------------------------------------------ tiled export
 * ExportSession in ExportMode::Tiled (export.rs:95-300, TiledExport :830-900): the image
 * lives in host memory; the device holds one tile-sized film and path arena. Each tile
 * renders all its samples (camera and RNG in image coordinates, samples in ascending
 * order, so the image equals a resident session's), then its planes are copied back
 * while the next tile renders and are committed whole: a checkpoint never holds part
 * of a tile. Checkpoints write state.bin and export.bin (the image) with FNV-1a
 * checksums; resume refuses a changed image ("checksum") or another producer. */
typedef struct sf_export sf_export;
sf_status sf_export_create(sf_context* ctx, sf_graph* graph, const sf_scene_desc* scene,
                           const sf_render_config* cfg, sf_export** out);
/* ExportSession::step: renders tiles until budget_ms passes (0 = one tile); *done = 1
 * once every tile is committed. */
sf_status sf_export_step(sf_export* e, uint32_t budget_ms, int* done);
sf_status sf_export_progress(sf_export* e, sf_progress* out);
/* The host image (committed tiles; others hold the cleared planes). */
sf_status sf_export_readback(sf_export* e, sf_film_planes* out);
sf_status sf_export_save(sf_export* e, const char* dir);
sf_status sf_export_resume(sf_context* ctx, sf_graph* graph, const char* dir, sf_export** out);
/* Device bytes the export holds (TiledExport::device_buffer_bytes). */
sf_status sf_export_device_bytes(sf_export* e, uint64_t* out);
sf_status sf_export_destroy(sf_export* e);
/* Autotuning knobs of the wavefront trace kernel (256 threads per block): resident
 * blocks per SM (2..4, selecting the register budget; default 3), the march step
 * quantum after which an open segment is saved and re-queued (0 = unbounded, the
 * default), and the regeneration threshold: how many lanes of a warp must be idle
 * before they take new segments together (1..32, 1 = at once; default 4). */
sf_status sf_session_set_launch(sf_session* s, uint32_t min_blocks_per_sm, uint32_t quantum, uint32_t regen);

/* ------------------------------------------------------------------ batches
 * Many jobs -- different graphs, scenes, image sizes and sample counts -- rendered
 * by one wavefront: one set of persistent trace launches per round covers every
 * job's paths (the reference renders jobs one after another, each through its own
 * Renderer/RenderSession, renderer.rs:668-693). A pass renders
 * cfg.samples_per_dispatch samples of every job; the pass is captured once in a
 * CUDA graph and replayed. Each job's image is its whole film (tile = image). */
typedef struct sf_batch sf_batch;
typedef struct sf_batch_job {
    sf_graph* graph;
    sf_scene_desc scene;
    sf_render_config cfg;
} sf_batch_job;
sf_status sf_batch_create(sf_context* ctx, const sf_batch_job* jobs, uint32_t n_jobs, sf_batch** out);
/* Trace-kernel shape for the batch: resident blocks per SM (2..4), step quantum and
 * regeneration threshold (as sf_session_set_launch). */
sf_status sf_batch_set_launch(sf_batch* b, uint32_t min_blocks_per_sm, uint32_t quantum, uint32_t regen);
/* Autotuner: times one pass per candidate shape (2..4 blocks per SM x quanta 0,
 * 64, 128, 256, then regeneration thresholds 1, 4, 8, 16 lanes at the best of those),
 * keeps the fastest, clears the films and rewinds the sample indices. */
sf_status sf_batch_autotune(sf_batch* b, uint32_t* min_blocks_per_sm, uint32_t* quantum, uint32_t* regen,
                            float* best_ms);
/* Queues `passes` passes (graph replays when use_graph != 0); asynchronous. */
sf_status sf_batch_run(sf_batch* b, uint32_t passes, int use_graph);
sf_status sf_batch_sync(sf_batch* b, uint32_t timeout_ms, uint32_t* status_word);
sf_status sf_batch_readback(sf_batch* b, uint32_t job, sf_film_planes* out);
sf_status sf_batch_destroy(sf_batch* b);

/* ------------------------------------------------------------------ escape time
 * PlanarFractal (crates/syfrack-core/src/scene/planar.rs:20-39); family:
 * 0 Julia, 1 Mandelbrot, 2 BurningShip, 3 Newton, 4 Nova, 5 Phoenix. Angles in
 * degrees. Iterations are not capped at the reference's 512 (planar.rs:205-210). */
typedef struct sf_planar_desc {
    uint32_t family, power, iterations;
    float julia[2], center[2];
    float zoom, angle, inversion, twist, relaxation, memory, bailout, trap_radius, stripes;
} sf_planar_desc;
/* Flat canvas mapping of the 2D branch (pathtrace.wgsl:1226-1239, uniforms.rs:760-764). */
typedef struct sf_canvas {
    float center[2];
    float zoom, rotation_deg;
    uint32_t width, height;
    uint64_t seed;
} sf_canvas;
/* PlanarFractal::sample at n points (xy interleaved, host): distance[n],
 * traps[4n] (slot-major), iterations[n]. Orbit arithmetic is unfused binary32,
 * so iteration counts equal the reference's f32 evaluation exactly. */
sf_status sf_planar_probe(sf_context* ctx, const sf_planar_desc* f, const float* xy, size_t n, float* distance,
                          float* traps, uint32_t* iterations);
/* One sample per pixel of a tile of the canvas; sample = 0xffffffff for pixel
 * centres, else the jitter of rng_init(px, sample, seed). Host outputs sized tile w*h. */
sf_status sf_escape2d(sf_context* ctx, const sf_planar_desc* f, const sf_canvas* canvas, sf_tile tile,
                      uint32_t sample, float* distance, float* traps, uint32_t* iterations);

/* Deep zoom (no counterpart in the reference, which caps zoom at 1e4): Mandelbrot
 * z <- z^2 + c around the double-double centre hi + lo, pixel pitch = width_units /
 * image width. The reference orbit is that of c_ref = hi; each pixel's FP32 offset
 * from it is lo + its position times the pitch, so lo keeps the centre's digits
 * below an FP64 ulp of hi. FP32 perturbation deltas with rebasing.
 * Outputs per pixel: iteration count (first n with |z_n| > bailout, else max_iter)
 * and smooth value n + 1 - log2(ln|z_n|). reference_f64 != 0 also runs the
 * full-FP64 direct iteration at c = hi + (lo + offset) into iters_f64/smooth_f64
 * (may be NULL otherwise).
 * orbit_mode (ABI 1.2) says where the reference orbit Z_n of c_ref comes from:
 * SF_ORBIT_DEVICE (0), FP64 on the GPU (one thread); SF_ORBIT_HOST (1), FP64 on a
 * host core, uploaded (the same unfused operations: the same orbit to the last
 * bit); SF_ORBIT_GIVEN (2), the caller's orbit: orbit_len entries of four floats
 * (Re hi, Im hi, Re lo, Im lo) with Z_n = hi + lo, from Z_0 = 0 through the last
 * entry the perturbation may use (its escape or max_iter), 1 <= orbit_len <=
 * max_iter + 1 -- a diagnostic that lets an orbit of higher precision stand in. */
enum { SF_ORBIT_DEVICE = 0, SF_ORBIT_HOST = 1, SF_ORBIT_GIVEN = 2 };
typedef struct sf_deep_zoom_desc {
    double center_hi[2], center_lo[2];
    double width_units;
    uint32_t width, height, max_iter;
    float bailout;
    uint32_t orbit_mode;
    uint32_t orbit_len;
    const float* orbit;
} sf_deep_zoom_desc;
sf_status sf_deep_zoom(sf_context* ctx, const sf_deep_zoom_desc* d, uint32_t* iterations, float* smooth,
                       int reference_f64, uint32_t* iters_f64, float* smooth_f64, uint64_t* rebases);
/* Deep zoom that allocates nothing; it has no counterpart in the reference. For
 * callers that cannot let a library call cudaMalloc (hosts that own all device
 * memory through their own pool; threads that cannot take cudaMalloc's implicit
 * device-wide synchronisation). Outputs are the caller's DEVICE buffers of
 * width*height entries; the work is queued on `stream` (a cudaStream_t, NULL for
 * the legacy default stream) on the current device and the call returns without
 * waiting. The reference orbit lives in a file-scope device array held by every
 * GPU that loads the library until exit (1 MB): max_iter above 65536 is rejected
 * with SF_ERR_INVALID. The first call on a device looks that array up, so make it
 * before any stream capture. All calls share the array: calls that overlap on the
 * GPU (two streams, two threads) race; order them on one stream. The array's address
 * is looked up once per device and kept for the life of the process: after
 * cudaDeviceReset (or anything else that re-creates the device's primary context)
 * the kept address is stale, so do not call this entry point again in that process.
 * Frames hold at most 2^31 pixels (SF_ERR_INVALID beyond), as for sf_deep_zoom. The
 * orbit is always computed on the device here (orbit_mode must be SF_ORBIT_DEVICE). */
sf_status sf_deep_zoom_noalloc(const sf_deep_zoom_desc* d, uint32_t* iterations, float* smooth, void* stream);

/* ------------------------------------------------------------------ serving
 * Continuous batching of the interactive requests of SyFrack's renderer: previews
 * (RenderSession::new + the first dispatch, session.rs:165, wavefront.rs:310),
 * progressive refinements that add samples to a preview's film (RenderSession::step,
 * session.rs:694) and 2D escape-time tiles (PlanarFractal::sample over a canvas,
 * planar.rs:77). The reference serves one session per thread with one dispatch in
 * flight; here one scheduler thread per server forms batches from the queue whenever
 * one of its slots (a wavefront arena with its own streams) is free and the HBM
 * budget admits the batch's films and tile outputs. Films stay in device memory from
 * a preview to its last refinement. A request's result does not depend on what it was
 * batched with: 3D paths run the same kernel for a graph form in any batch and each
 * pixel sums its samples in ascending order; 2D pixels are independent. */
enum sf_request_kind { SF_REQ_PREVIEW = 0, SF_REQ_REFINE = 1, SF_REQ_TILE_2D = 2 };
enum sf_request_state { SF_REQ_QUEUED = 0, SF_REQ_RUNNING = 1, SF_REQ_DONE = 2, SF_REQ_FAILED = 3 };
/* What a 2D tile returns: everything sf_escape2d returns (distance, the four trap
 * planes, iterations), or only iterations and the smooth time (trap 0), for which
 * the ring, stripe and angle traps are not computed. */
enum sf_tile_outputs { SF_TILE_ALL = 0, SF_TILE_COUNTS = 1 };
typedef struct sf_server sf_server;
typedef struct sf_server_config {
    uint64_t hbm_budget;        /* device bytes for films and tile outputs together   */
    uint64_t host_result_bytes; /* pinned host pool holding finished results          */
    uint32_t slots;             /* batches in flight at once, 1..8                    */
    uint32_t path_capacity;     /* paths per 3D batch (a request needs w*h*samples)   */
    uint32_t max_jobs;          /* requests per batch, 1..1024                        */
    uint32_t max_tile_pixels;   /* 2D pixels per batch                                */
    uint32_t min_blocks, quantum, regen; /* trace launch shape (sf_batch_set_launch)  */
    uint32_t pad;
} sf_server_config;
typedef struct sf_request {
    uint32_t kind;              /* sf_request_kind                                    */
    uint32_t samples;           /* REFINE: samples added to the parent's film         */
    uint64_t parent;            /* REFINE: ticket of the preview that owns the film   */
    sf_graph* graph;            /* PREVIEW                                            */
    sf_scene_desc scene;        /* PREVIEW                                            */
    sf_render_config cfg;       /* PREVIEW: size, samples_per_pixel of the first pass,
                                   bounces and steps; later refinements keep them     */
    sf_planar_desc planar;      /* TILE_2D                                            */
    sf_canvas canvas;           /* TILE_2D: the whole canvas, sampled at pixel centres */
    uint32_t tile_outputs;      /* TILE_2D: sf_tile_outputs                           */
    uint32_t pad;
} sf_request;
typedef struct sf_result {
    uint32_t state;             /* sf_request_state                                   */
    sf_status status;           /* SF_OK unless FAILED                                */
    uint32_t kind, width, height;
    uint32_t samples;           /* 3D: samples in the film after this request         */
    uint32_t batch_requests;    /* requests in the batch that carried it              */
    uint32_t pad;
    uint64_t work;              /* 3D: paths traced; 2D: pixels                       */
    double submit_ms, start_ms, done_ms; /* server clock (ms since sf_server_create)  */
    const float* accum;         /* 3D: width*height float4 sample sums (film order)   */
    const uint32_t* iterations; /* 2D: width*height iteration counts                  */
    const float* smooth;        /* 2D: width*height trap 0 (smooth time / iterations) */
    const float* distance;      /* 2D, SF_TILE_ALL: width*height r/(1+r)              */
    const float* traps;         /* 2D, SF_TILE_ALL: 4 planes of width*height (slot-major) */
} sf_result;
typedef struct sf_server_stats {
    uint64_t submitted, completed, failed, batches, batched_requests;
    uint64_t admission_waits;   /* batches cut short by the HBM budget                */
    uint64_t hbm_used, hbm_peak, hbm_reserved, host_used;
    uint64_t launches;
    double now_ms;
} sf_server_stats;
/* Starts the scheduler thread. Defaults for zero fields: 4 slots, 4M paths, 256 jobs,
 * 32M tile pixels, 1 GiB of host results, launch shape 3 blocks/SM, quantum 128 and
 * regeneration threshold 4. */
sf_status sf_server_create(sf_context* ctx, const sf_server_config* cfg, sf_server** out);
/* Queues a request; returns at once with its ticket (tickets start at 1). */
sf_status sf_serve_submit(sf_server* s, const sf_request* req, uint64_t* ticket);
/* Non-blocking state of a request; result pointers stay valid until sf_serve_release. */
sf_status sf_serve_poll(sf_server* s, uint64_t ticket, sf_result* out);
/* Waits up to timeout_ms (0 = no limit) for DONE or FAILED; SF_ERR_TIMEOUT otherwise. */
sf_status sf_serve_wait(sf_server* s, uint64_t ticket, uint32_t timeout_ms, sf_result* out);
/* Drops a finished request's result; a preview's film is freed once no queued
 * refinement needs it. SF_ERR_BUSY while the request is queued or running. */
sf_status sf_serve_release(sf_server* s, uint64_t ticket);
sf_status sf_server_stats_get(sf_server* s, sf_server_stats* out);
/* Stops the scheduler after the batches in flight; queued requests fail. */
sf_status sf_server_destroy(sf_server* s);

#ifdef __cplusplus
}
#endif
#endif /* SYFRACK_GPU_H */

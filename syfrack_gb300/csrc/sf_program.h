// Lowered form graph and per-launch parameter blocks shared by the host
// library (sf_host.cpp) and the sm_103a kernels (sf_kernels.cu). Plain data only.
//
// The reference compiles a Graph into a WGSL `de_sample` function and packs its
// scalars into a uniform array (graph_wgsl.rs:949-1179, ParamLayout :30-184).
// Here a graph is lowered once on the host into a `DeProgram`:
//   * `form` names a specialised device routine when the graph is one of the
//     iterated forms (Mandelbulb, Mandelbox, Menger body orders of graphs/*.ron),
//     whose constants are read from `fp`;
//   * otherwise `ops` is a postfix program run by the generic interpreter: every
//     distance leaf re-evaluates its point chain from the input point (leaves
//     that share a prefix recompute it; the result is identical), fences push a
//     distance state, combinations pop two.
#pragma once
#include <stdint.h>

#define SF_MAX_OPS 255
#define SF_MAX_LOOP_DEPTH 4
#define SF_MAX_DIST_STACK 6
#define SF_MAX_INST_DEPTH 3  // nested Instances levels (MAX_DEPTH, graph/mod.rs:41)
#define SF_MAX_UNION_LEAVES 32  // leaves of the exact union branch-and-bound

// Opcodes of the generic interpreter. Point and fence operations use the node
// kind (enum sf_node_kind) as their code; control codes start at 100.
enum {
    SF_OP_BEGIN = 100,      // point state := input point
    SF_OP_ITER_BEGIN = 101, // a = iterations, b = index of the matching ITER_END, f0 = bailout, f1 = bailout_t
    SF_OP_ITER_END = 102,   // a = index of the matching ITER_BEGIN
    SF_OP_FENCE_OFF = 103,  // disabled fence: push +inf with the point's iter/traps
    SF_OP_EMPTY = 104,      // unconnected distance input: push the empty state
    SF_OP_TAG = 105,        // a = material index
    SF_OP_BOUND = 106,      // top.d = max(top.d, box(point)); f0..2 = half
    SF_OP_COMBINE = 107,    // a = node kind of the combination, f0 = k
    SF_OP_END = 108,
    // A Bounded node the device may skip (graph_wgsl.rs:800-814): the op follows the
    // port-0 point chain and computes bound = box(point, f0..2); in fast mode, when
    // bound > f3 (margin), it pushes {bound, no traps, 0 iterations, material 0,
    // flags 1} and jumps past the detail branch to b; otherwise it pushes the bound
    // and the detail branch follows, closed by BOUND_END.
    SF_OP_BOUND_FAST = 109,
    SF_OP_BOUND_END = 110,  // detail.d = max(bound, detail.d); the detail's payload and flags stay
    // Instances (graph_wgsl.rs:744-790): a = placement count, b = index of INST_END,
    // c = offset of the node's block in inst_data (12 floats of inverse affine rows per
    // placement, then 8 floats per hierarchy node: centre, half, escape, placement or -1),
    // f0..2 = half, f3 = margin, f4 = 1 when the copies may be skipped (fast). The ops
    // between INST_BEGIN and INST_END evaluate the template at a copy's local point;
    // they may hold further Instances, nested up to SF_MAX_INST_DEPTH levels.
    SF_OP_INST_BEGIN = 111,
    SF_OP_INST_END = 112    // a = index of the matching INST_BEGIN
};

struct DeOp {
    uint32_t code;
    uint32_t a, b, c;
    float f[8];
};

// Constants of the specialised forms.
struct FormParams {
    uint32_t iterations;
    uint32_t trap_slot, trap_measure, trap_mode;  // the body's Trap node
    uint32_t trap_squared;  // Norm trap in Minimum/Last mode: kept as |p|^2, one sqrt at the end
    float bailout;
    float bailout_t;     // largest float x with sqrtf(x) <= bailout: |p| > bailout <=> dot(p,p) > bailout_t
    float power;         // Bulb
    uint32_t power_int;  // Bulb: 0 = trigonometric path, else the integer exponent 1..16
    float limit;         // Box: fold limit
    float min_radius2, fixed_radius2, fold_k_min;  // Box: mr^2, fr^2, fr^2/mr^2
    uint32_t fold_clamped;  // Box: fr >= mr, so the fold factor is min(fr^2/mr^2, max(fr^2/r^2, 1))
    float scale;         // Box: Scale factor; Menger: fold scale
    float abs_scale;     // Box: |scale|
    float offset[3];     // Menger: fold offset
    float fence[3];      // NormFence inset / Box half
    uint32_t material;   // MaterialTag index applied to the root (0 = none)
};

struct DeProgram {
    uint32_t form;  // SF_FORM_*
    uint32_t n_ops;
    uint32_t iteration_product;
    uint32_t max_stack;
    uint32_t fast_bounds;  // number of BOUND_FAST ops: samples may carry the conservative flag
    uint32_t inst_floats;  // length of inst_data
    uint64_t inst_data;    // device address of the Instances blocks (const float*), 0 when none
    float trap_scales[4];
    FormParams fp;
    DeOp ops[SF_MAX_OPS];
    // The exact union branch-and-bound (graph_wgsl.rs:1112-1154): when the graph has a
    // skippable Bounded or Instances node and the Output's input is a tree of enabled
    // Unions over 2..SF_MAX_UNION_LEAVES distinct leaves, leaf i (in depth-first order,
    // first occurrence) is the self-contained op range [leaf_begin[i], leaf_end[i]),
    // which pushes one distance state. 0 = exact samples run the whole program. Kept
    // after the ops, whose offset in shared memory stays that of the plain program.
    uint32_t union_leaves;
    uint8_t leaf_begin[SF_MAX_UNION_LEAVES], leaf_end[SF_MAX_UNION_LEAVES];
};
static_assert(SF_MAX_OPS <= 255, "leaf ranges are stored as bytes");

// One area light in device form (GpuLight of uniforms.rs:671-713 with the
// derived quantities the shading code needs every bounce).
// kind SF_LIGHT_AREA: a = centre, b/c = full edges, color = radiance, n/area/inv_*;
// SF_LIGHT_SUN: a = unit direction toward the sun, color = irradiance, cos_max;
// SF_LIGHT_ENVIRONMENT: a/b/c = zenith/horizon/ground radiance, energy = their largest
// luminance, peak = their largest component.
// SF_LIGHT_HDRI: a.x/a.y = cos/sin of the rotation, a.z = 1 for uniform sampling,
// color.x = intensity, texels = the panorama's (rgb, cdf) rows of tw x th texels.
// SF_LIGHT_AREA with projector = 1: a projector (GpuLight kind.y, uniforms.rs:671-716),
// whose emission follows beam = (cos inner, cos outer, tan outer angle);
// SF_LIGHT_TUBE (uniforms.rs:717-729): a capsule, a = start, b = end, radius, length.
struct DevLight {
    float a[3], b[3], c[3], color[3];
    float n[3];          // safe_normalize(cross(b, c))
    float area;          // emitter_area: |cross(b, c)|, a tube's 2 pi r (length + 2 r)
    float inv_bb, inv_cc;// 1 / dot(b,b), 1 / dot(c,c)
    float lum;           // luminance(color)
    uint32_t kind;
    float cos_max, energy, peak;
    uint32_t tw, th;
    uint64_t texels;     // device address of float4 texels (HDRI)
    uint32_t projector;
    float beam[3];
    float radius, length;
};
#define SF_MAX_RAMP 16
// Lights held in DevScene itself (staged into shared memory with it); a scene's further
// lights, up to 96, follow its DevScene in device memory at SF_LIGHT_TABLE_OFFSET.
#define SF_SHARED_LIGHTS 8

struct DevMaterial {
    float albedo[3], roughness, metallic, specular, emission[3];
};
// A ramp (GpuRamp, palette_sample of common.wgsl:331-362): stops (rgb, position).
struct DevRamp {
    uint32_t n, cyclic, smooth, positioned;
    float map[3];  // frequency, phase, gamma
    float stops[SF_MAX_RAMP][4];
};
// GpuFinish.detail_* (uniforms.rs:797-815): kind (FinishPattern 1..12, 0 = none), seed,
// mapping = scale, strength, bump, roughness delta; tint.
struct DevDetail {
    uint32_t kind, seed;
    float mapping[4];
    float tint[3];
};
// GpuOptics (uniforms.rs:95-122): surface = opacity, transmission, ior, thin sheet;
// absorption = sigma_a rgb, distance (> 0: optics enabled); subsurface = albedo rgb,
// collision rate.
struct DevOptics {
    float surface[4], absorption[4], subsurface[4];
};
// GpuTexture (uniforms.rs:316-380) with the texture graph's lowered program.
struct DevTexture {
    uint32_t channel, octaves, budget;  // kind.x, kind.y, kind.z (iteration budget)
    uint32_t enabled;
    float mapping[4];   // offset xyz, scale
    float rotation[4];  // Euler radians xyz, contrast
    float effects[4];   // colour, roughness, bump strength, enabled
    float weights[4], extra[4];  // orbit channel mix
    float parallax[2];  // depth, layer budget
    float fan[4];       // period xz, rays, enabled
    float mask[4];      // trap slot, value, width, enabled
    uint64_t prog;      // device address of the texture graph's DeProgram
    DevRamp ramp;
};

// Scene constants of one render (the Uniforms subset of common.wgsl:163-191
// that the DE path reads).
struct DevScene {
    float origin[3], forward[3], right[3], up[3];
    float tan_half, aspect, lens_radius, focus_distance;
    uint32_t width, height;
    uint32_t max_bounces, max_steps;
    uint32_t seed;
    uint32_t light_count, finish_count;
    uint32_t variation_slot, variation_enabled;
    float var_rough[2], var_metal[2];
    float cavity;
    float pixel_tolerance, step_scale, extent;  // extent = max(200, far)
    float pixel_cone;                           // tan_half * 2 / width
    float hit_eps;                              // > 0: fixed-epsilon hit test; 0: cone-relative
    uint32_t iteration_product;
    // Material.coloring: slot (0..3 trap, 4 iterations, 5 normal, 6 orbit mix, else none)
    // and ramp; col_weights / col_extra = the orbit mix (GpuColoring.weights, .extra)
    uint32_t col_slot;
    float col_weights[4], col_extra[3];
    DevRamp col;
    uint32_t shadow_slots;            // shadow requests a bounce can make (shadow_slots_of)
    float fog[4];                     // density, height, falloff, anisotropy (atmosphere.a)
    float fog_color[3];               // scattering albedo (atmosphere.b.xyz)
    DevMaterial material;
    DevMaterial finishes[8];
    DevLight lights[SF_SHARED_LIGHTS];
    // make_surface's detail and texture and radiance's optics. rich: SF_RICH_* bits of
    // what the scene uses (0 keeps every path of the plain surface).
    uint32_t rich;
    float dune_wind;  // radians
    DevDetail details[8];
    DevOptics optics[9];
    DevTexture tex;
};
// Byte offset from a DevScene in device memory to its lights past SF_SHARED_LIGHTS.
#define SF_LIGHT_TABLE_OFFSET ((sizeof(DevScene) + 255) & ~size_t(255))
enum { SF_RICH_DETAIL = 1, SF_RICH_TEXTURE = 2, SF_RICH_OPTICS = 4, SF_RICH_ROUGH_DIFFUSE = 8 };

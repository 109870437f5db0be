// TEST INFRASTRUCTURE -- NOT THE PRODUCT.
//
// CPU restatement of SyFrack's distance-estimator path, used only to check
// results in tests/ and __graft_entry__.smoke(), and as bench.py's CPU baseline.
// Templated on the real type R:
//   R = float  : the reference's own binary32 arithmetic, operation order kept
//                (built with -ffp-contract=off, libm float functions, like Rust's
//                f32 methods on Linux);
//   R = double : the FP64 oracle.
// Each function cites the reference file:line it restates (paths relative to
// the SyFrack source tree). Parity is pinned by the reference's golden DE
// vectors (crates/syfrack-core/tests/fixtures/parity/*.ron) and by the known
// answers of its unit tests (eval.rs, planar.rs, fractal.rs).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <set>
#include <string>
#include <vector>

#include "../include/syfrack_gpu.h"

namespace orc {

// ---------------------------------------------------------------- math shims
inline float r_sqrt(float x) { return sqrtf(x); }
inline double r_sqrt(double x) { return std::sqrt(x); }
inline float r_sin(float x) { return sinf(x); }
inline double r_sin(double x) { return std::sin(x); }
inline float r_cos(float x) { return cosf(x); }
inline double r_cos(double x) { return std::cos(x); }
inline float r_atan2(float y, float x) { return atan2f(y, x); }
inline double r_atan2(double y, double x) { return std::atan2(y, x); }
inline float r_log(float x) { return logf(x); }
inline double r_log(double x) { return std::log(x); }
inline float r_log1p(float x) { return log1pf(x); }
inline double r_log1p(double x) { return std::log1p(x); }
inline float r_exp(float x) { return expf(x); }
inline double r_exp(double x) { return std::exp(x); }
inline float r_tan(float x) { return tanf(x); }
inline double r_tan(double x) { return std::tan(x); }
inline float r_pow(float x, float y) { return powf(x, y); }
inline double r_pow(double x, double y) { return std::pow(x, y); }
inline float r_acos(float x) { return acosf(x); }
inline double r_acos(double x) { return std::acos(x); }
inline float r_floor(float x) { return floorf(x); }
inline double r_floor(double x) { return std::floor(x); }
inline float r_fmod(float x, float y) { return fmodf(x, y); }
inline double r_fmod(double x, double y) { return std::fmod(x, y); }
template <class R> inline R r_abs(R x) { return x < R(0) ? -x : (x == R(0) ? R(0) : x); }
// Rust f32::min/max ignore a NaN operand.
template <class R> inline R r_min(R a, R b) { if (a != a) return b; if (b != b) return a; return a < b ? a : b; }
template <class R> inline R r_max(R a, R b) { if (a != a) return b; if (b != b) return a; return a > b ? a : b; }
template <class R> inline R r_clamp(R x, R lo, R hi) { return r_min(r_max(x, lo), hi); }
template <class R> inline bool r_finite(R x) { return std::isfinite(x); }
// Rust rem_euclid for floats.
template <class R> inline R r_rem_euclid(R x, R m) { R r = r_fmod(x, m); return r < R(0) ? r + r_abs(m) : r; }
template <class R> inline R to_radians(R deg) { return deg * (R(3.14159265358979323846) / R(180)); }

template <class R> struct V2 {
    R x, y;
    V2() : x(0), y(0) {}
    V2(R a, R b) : x(a), y(b) {}
    V2 operator+(V2 o) const { return {x + o.x, y + o.y}; }
    V2 operator-(V2 o) const { return {x - o.x, y - o.y}; }
    V2 operator*(R s) const { return {x * s, y * s}; }
    V2 operator/(R s) const { return {x / s, y / s}; }
    R dot(V2 o) const { return x * o.x + y * o.y; }
    R length() const { return r_sqrt(dot(*this)); }
    R length_squared() const { return dot(*this); }
};
template <class R> struct V3 {
    R x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(R a, R b, R c) : x(a), y(b), z(c) {}
    static V3 splat(R s) { return {s, s, s}; }
    V3 operator+(V3 o) const { return {x + o.x, y + o.y, z + o.z}; }
    V3 operator-(V3 o) const { return {x - o.x, y - o.y, z - o.z}; }
    V3 operator*(V3 o) const { return {x * o.x, y * o.y, z * o.z}; }
    V3 operator/(V3 o) const { return {x / o.x, y / o.y, z / o.z}; }
    V3 operator*(R s) const { return {x * s, y * s, z * s}; }
    V3 operator/(R s) const { return {x / s, y / s, z / s}; }
    V3 operator-() const { return {-x, -y, -z}; }
    R dot(V3 o) const { return x * o.x + y * o.y + z * o.z; }
    R length() const { return r_sqrt(dot(*this)); }
    R length_squared() const { return dot(*this); }
    V3 abs() const { return {r_abs(x), r_abs(y), r_abs(z)}; }
    R max_element() const { return r_max(r_max(x, y), z); }
    R min_element() const { return r_min(r_min(x, y), z); }
    V3 cross(V3 o) const { return {y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x}; }
    R& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class R> inline V3<R> vmin(V3<R> a, V3<R> b) { return {r_min(a.x, b.x), r_min(a.y, b.y), r_min(a.z, b.z)}; }
template <class R> inline V3<R> vmax(V3<R> a, V3<R> b) { return {r_max(a.x, b.x), r_max(a.y, b.y), r_max(a.z, b.z)}; }
template <class R> inline V3<R> vclamp(V3<R> v, V3<R> lo, V3<R> hi) { return vmin(vmax(v, lo), hi); }
// WGSL normalize(v) = v / length(v).
template <class R> inline V3<R> normalize(V3<R> v) { return v / v.length(); }
// glam try_normalize().unwrap_or(Y) as common.wgsl:241-246 (safe_normalize).
template <class R> inline V3<R> safe_normalize(V3<R> v) {
    R l = v.length();
    R rcp = R(1) / l;
    if (!(l > R(0)) || !(rcp > R(0)) || !(rcp <= std::numeric_limits<R>::max())) return {0, 1, 0};
    return v * rcp;
}
template <class R> inline V3<R> mixv(V3<R> a, V3<R> b, R t) { return a * (R(1) - t) + b * t; }
template <class R> inline R mixs(R a, R b, R t) { return a * (R(1) - t) + b * t; }

// ---------------------------------------------------------------- graph
// Graph preparation: node lookup (graph/mod.rs:483-497), active_nodes,
// body_owners, topo_order (validate.rs:10-85), iteration_product
// (validate.rs:112-141), trap_scales / lipschitz / step_scale (eval.rs:828-881).
struct Graph {
    std::vector<sf_node> nodes;
    std::vector<sf_link> links;
    std::vector<uint32_t> body;
    float safety = 1.f, hint = 1.f;
    // prepared
    bool ok = false;
    std::string error;
    std::vector<uint32_t> order;     // topo order of active non-body nodes
    std::vector<uint32_t> plan;      // needed subset for the output, topo order
    uint32_t output = 0;
    float trap_scales[4] = {1, 1, 1, 1};
    uint32_t iteration_product = 1;
    float lipschitz = 1.f, step_scale = 1.f;
    std::set<uint32_t> fast_bounds;  // Bounded / Instances nodes the GPU may skip (graph_wgsl.rs:1019-1031)
    std::vector<sf_placement> placements;
    // Instances: the fence hierarchy per node (bvh.rs), and the evaluation plan of
    // every target (the output and each enabled Instances node's template).
    struct InstBounds { float center[3], half[3]; size_t escape; int64_t placement; };
    std::map<uint32_t, std::vector<InstBounds>> instances;
    std::map<uint32_t, std::vector<uint32_t>> plans;
    // The exact union search (graph_wgsl.rs:1112-1154): the leaves below the Output's
    // enabled Unions, depth-first, first input first, a leaf reached twice kept once
    // (union_leaves, :18-26); an unconnected port is a leaf of its own (UINT32_MAX:
    // the empty state). Each leaf has a plan.
    std::vector<uint32_t> union_leaves;

    const sf_node* node(uint32_t id) const {
        for (auto& n : nodes) if (n.id == id) return &n;
        return nullptr;
    }
    bool input_of(uint32_t to, uint32_t port, uint32_t* from) const {
        for (auto& l : links) if (l.to_node == to && l.to_port == port) { *from = l.from_node; return true; }
        return false;
    }
    std::vector<uint32_t> body_of(const sf_node& n) const {
        std::vector<uint32_t> b;
        if (n.kind != SF_NODE_ITERATE) return b;
        for (uint32_t i = 0; i < n.body_len; ++i) b.push_back(body[n.body_offset + i]);
        return b;
    }
};

inline bool is_point_to_point(uint32_t k) {
    switch (k) {
    case SF_NODE_TRANSLATE: case SF_NODE_ROTATE: case SF_NODE_SCALE: case SF_NODE_SCALE_AXES:
    case SF_NODE_MIRROR: case SF_NODE_BOX_FOLD: case SF_NODE_BOX_FOLD_AXES:
    case SF_NODE_SPHERE_INVERSION: case SF_NODE_SPHERE_FOLD: case SF_NODE_ABS:
    case SF_NODE_MENGER_FOLD: case SF_NODE_KALEIDO: case SF_NODE_POWER: case SF_NODE_ADD_ORIGIN:
    case SF_NODE_ADD_SEED: case SF_NODE_ADD_CONSTANT: case SF_NODE_TWIST: case SF_NODE_BEND:
    case SF_NODE_TILE: case SF_NODE_REPEAT_FINITE: case SF_NODE_ITERATE: case SF_NODE_TRAP:
        return true;
    default: return false;
    }
}
inline bool is_fence(uint32_t k) {
    return k == SF_NODE_SPHERE || k == SF_NODE_TORUS || k == SF_NODE_CYLINDER || k == SF_NODE_BOX ||
           k == SF_NODE_ROUND_BOX || k == SF_NODE_ROCK || k == SF_NODE_PLANE ||
           k == SF_NODE_NORM_FENCE || k == SF_NODE_BULB_FENCE;
}
inline bool is_combine(uint32_t k) {
    return k == SF_NODE_UNION || k == SF_NODE_INTERSECTION || k == SF_NODE_SUBTRACTION ||
           k == SF_NODE_SMOOTH_UNION || k == SF_NODE_SMOOTH_INTERSECTION;
}
// NodeKind::inputs (graph/mod.rs:366-386): number of input ports.
inline uint32_t input_count(uint32_t k) {
    if (k == SF_NODE_INPUT) return 0;
    if (k == SF_NODE_BOUNDED || is_combine(k)) return 2;
    return 1;
}

bool prepare(Graph& g);
// bvh::build (bvh.rs:26-102): the fence hierarchy of one Instances node.
std::vector<Graph::InstBounds> bvh_build(const sf_placement* pl, uint32_t count, const float* half);

// ---------------------------------------------------------------- DE
template <class R> struct PointState { V3<R> p; R dr; uint32_t iter; R traps[4]; };
template <class R> struct DistState { R d; uint32_t material; uint32_t iter; R traps[4]; uint32_t flags = 0; };
template <class R> struct Sample { R distance; R traps[4]; uint32_t iterations; uint32_t material; uint32_t flags = 0; };

// fast = false: Graph::evaluate (eval.rs), identical to the GPU's de_sample_exact.
// fast = true: the GPU's de_sample (graph_wgsl.rs:800-814): a skippable Bounded
// branch outside its margin gives its bound, flagged (flags = 1).
template <class R> Sample<R> evaluate(const Graph& g, V3<R> p, bool fast = false);
// The reference's exact sample with the union search (graph_wgsl.rs:1112-1154): every
// leaf probed for its bound, then the leaves whose bound can beat the best evaluated
// exactly, lowest bound first; when the search does not apply (fewer than two leaves,
// more than 128, or no skippable node) the plain exact sample.
// exact_leaves (optional): adds the number of leaves evaluated exactly after the probes.
template <class R> Sample<R> evaluate_union_search(const Graph& g, V3<R> p, uint32_t* exact_leaves = nullptr);

// ---------------------------------------------------------------- transport
template <class R> struct Camera { V3<R> origin, forward, right, up; R tan_half, aspect, lens_radius, focus_distance; };
// kind 0 Area: a centre, b/c full edges, color radiance; 1 Sun: a unit direction,
// color irradiance, cos_max; 2 Environment: a/b/c zenith/horizon/ground radiance.
// A panorama's tables (environment.rs:271-366): w x h texels of (r, g, b, cdf).
struct Panorama { uint32_t w = 0, h = 0; bool uniform = false; std::vector<float> texels; };
bool panorama_tables(const float* rgb, uint32_t width, uint32_t height, Panorama& out);
// Panoramas by the key the scene descriptor's environment field carries.
void panorama_register(uint64_t key, const Panorama& p);
const Panorama* panorama_find(uint64_t key);
template <class R> struct Light {
    V3<R> a, b, c, color;
    uint32_t kind = 0;
    R cos_max = 1, energy = 0, peak = 0;
    const Panorama* pano = nullptr;  // HDRI: a = (cos, sin of the rotation, uniform), color.x = intensity
    // a projector is an area light with its beam (cos inner, cos outer, tan outer);
    // a tube (SF_LIGHT_TUBE): a = start, b = end, radius and length
    bool projector = false;
    R beam[3] = {0, 0, 0};
    R radius = 0, length = 0;
};
template <class R> struct Coloring {
    uint32_t slot = 0xffff, n = 0;
    bool cyclic = false, smooth = false, positioned = false;
    R frequency = 1, phase = 0, gamma = 1;
    V3<R> stops[SF_MAX_RAMP_STOPS];
    R pos[SF_MAX_RAMP_STOPS];
};
template <class R> struct Mat { V3<R> albedo; R roughness, metallic, specular; V3<R> emission; };
// FinishDetail (GpuFinish.detail_*, uniforms.rs:797-815): kind 0 = none.
template <class R> struct Detail { uint32_t kind = 0, seed = 0; R scale = 1, strength = 0, bump = 0, rough_delta = 0; V3<R> tint; };
// GpuOptics (uniforms.rs:103-122): enabled when absorption.w > 0.
template <class R> struct Optics { R surface[4] = {0, 0, 0, 0}, absorption[4] = {0, 0, 0, 0}, subsurface[4] = {0, 0, 0, 0}; };
// GpuTexture (uniforms.rs:340-379) with the texture's own graph.
template <class R> struct Texture {
    const Graph* graph = nullptr;
    uint32_t channel = 0, octaves = 1, budget = 1;
    R mapping[4] = {0, 0, 0, 1}, rotation[4] = {0, 0, 0, 1}, effects[4] = {0, 0, 0, 0};
    R weights[4] = {0, 0, 0, 0}, extra[3] = {0, 0, 0};
    R parallax[2] = {0, 8}, fan[4] = {0, 0, 0, 0}, mask[4] = {0, 0, 0, 0};
    Coloring<R> ramp;
};
template <class R> struct Scene {
    Camera<R> cam;
    Mat<R> material;
    Mat<R> finishes[SF_MAX_FINISHES];
    uint32_t finish_count = 0;
    Light<R> lights[SF_MAX_SCENE_LIGHTS];  // Scene::lights, at most MAX_LIGHTS (light.rs:7)
    uint32_t light_count = 0;
    Coloring<R> coloring;
    R col_weights[4] = {0, 0, 0, 0}, col_extra[3] = {0, 0, 0};  // the orbit mix of coloring slot 6
    Detail<R> details[SF_MAX_FINISHES];
    R dune_wind = 0;  // radians
    Optics<R> optics[SF_MAX_FINISHES + 1];
    bool has_optics = false;
    Texture<R> tex;
    uint32_t variation_slot = 0, variation_enabled = 0;
    R var_rough[2] = {0, 0}, var_metal[2] = {0, 0};
    R cavity = 0;
    R fog[4] = {0, 0, 0, 0};  // density, height, falloff, anisotropy (atmosphere.a)
    V3<R> fog_color;          // atmosphere.b.xyz
    uint32_t seed = 0;
    // fractal uniforms (uniforms.rs:183-189, :781-782)
    R pixel_tolerance = 1, far = 200, step_scale = 1;
    R hit_eps = 0;  // > 0: fixed-epsilon hit test radius <= hit_eps; 0: cone-relative
    uint32_t iteration_product = 1;
    uint32_t width = 1, height = 1, max_bounces = 4, max_steps = 256;
};
template <class R> Scene<R> make_scene(const Graph& g, const sf_scene_desc& d, const sf_render_config& c);
// pattern_value (pattern.wgsl:2-49) of the scene's texture at p.
template <class R> R texture_value_at(const Scene<R>& sc, V3<R> p);

// L: the sample's radiance; V: its volume part (pathtrace.wgsl:1197-1198: all of L when
// the camera segment scattered in fog, else that segment's in-scattered emitter light);
// both zero when L is not finite (main's `ok`, :1243-1250).
struct PixelResult { double L[3]; double V[3]; double depth; double aux[4]; uint32_t segments; uint64_t de_evals; };
template <class R> PixelResult radiance(const Graph& g, const Scene<R>& sc, uint32_t px, uint32_t py, uint32_t sample);

template <class R> struct Hit { bool hit; R t; uint32_t steps; Sample<R> sample; bool exhausted; uint32_t light_index; };
template <class R> Hit<R> march_segment(const Graph& g, V3<R> ro, V3<R> rd, R step_scale, R hit_cone,
                                        R t_end, uint32_t max_steps, bool absolute_rule, R eps,
                                        uint64_t* de_evals);
template <class R> V3<R> normal_tetra(const Graph& g, V3<R> p, R h);
template <class R> V3<R> normal_central(const Graph& g, V3<R> p, R h);

// PCG chain (pathtrace.wgsl:20-37).
inline uint32_t pcg(uint32_t v) {
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
inline uint32_t rng_init(uint32_t px, uint32_t py, uint32_t sample, uint32_t seed) {
    uint32_t h = pcg(seed);
    h = pcg(h ^ px);
    h = pcg(h ^ py);
    h = pcg(h ^ sample);
    return h;
}
template <class R> inline R rnd(uint32_t* state) {
    *state = pcg(*state);
    return R(float(*state >> 8u) * (1.0f / 16777216.0f));
}

// ---------------------------------------------------------------- planar
struct PlanarParams {
    uint32_t family, power, iterations;
    double julia[2], center[2];
    double zoom, angle, inversion, twist, relaxation, memory, bailout, trap_radius, stripes;
};
template <class R> Sample<R> planar_sample(const PlanarParams& f, V2<R> input);

}  // namespace orc

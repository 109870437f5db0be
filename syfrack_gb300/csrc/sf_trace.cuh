// Sphere tracing and path transport on sm_103a.
//
// Device twins of pathtrace.wgsl (PCG :20-37, march_segment :78-145, BRDF
// :195-463, direct_light :471-558, camera_ray :781-800, radiance :802-1201)
// and lights.wgsl (:150-356), with ocean, portals, guiding, nature phenomena and
// spectral dispersion off (each is an identity when off). The bounce body
// is one function (bounce_body) used by both the per-pixel megakernel and the
// wavefront shade stage, so both integrators perform identical arithmetic.
#pragma once
#include "sf_de.cuh"
#include "sf_surface.cuh"

#define SF_NO_LIGHT 0xffffffffu
// What a shading kernel is built with (a template argument of make_surface, bounce_body
// and the kernels that inline them): finish details, optics and the transported
// footprint; the volumetric texture's interpreter.
enum { SF_FEAT_RICH = 1, SF_FEAT_TEX = 2 };

// ------------------------------------------------------------------ RNG
__device__ __forceinline__ uint32_t pcg(uint32_t v) {
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
__device__ __forceinline__ uint32_t rng_init(uint32_t px, uint32_t py, uint32_t sample, uint32_t seed) {
    uint32_t h = pcg(seed);
    h = pcg(h ^ px);
    h = pcg(h ^ py);
    h = pcg(h ^ sample);
    return h;
}
__device__ __forceinline__ float rnd(uint32_t& state) {
    state = pcg(state);
    return float(state >> 8u) * (1.0f / 16777216.0f);
}

// ------------------------------------------------------------------ camera
__device__ __forceinline__ void camera_ray(const DevScene& S, uint32_t px, uint32_t py, uint32_t& rng, float3& o,
                                           float3& d) {
    float jx = rnd(rng);
    float jy = rnd(rng);
    float ndcx = ((float(px) + jx) / float(S.width)) * 2.0f - 1.0f;
    float ndcy = ((float(py) + jy) / float(S.height)) * 2.0f - 1.0f;
    float3 dir = normalize3(ld3(S.forward) + ld3(S.right) * (ndcx * S.tan_half) +
                            ld3(S.up) * (-ndcy * S.tan_half / S.aspect));
    float3 origin = ld3(S.origin);
    if (S.lens_radius > 0.0f) {
        float3 focus = origin + dir * (S.focus_distance / fmaxf(dot3(dir, ld3(S.forward)), 1e-4f));
        float r = S.lens_radius * sqrtf(rnd(rng));
        float phi = 2.0f * SF_PI * rnd(rng);
        origin = origin + ld3(S.right) * (r * cosf(phi)) + ld3(S.up) * (r * sinf(phi));
        dir = normalize3(focus - origin);
    }
    o = origin;
    d = dir;
}

// ------------------------------------------------------------------ march state machine
// march_segment (pathtrace.wgsl:78-145) split into resumable steps so that a
// persistent kernel can interleave lanes: march_query() gives the point to
// evaluate, march_update() consumes its DE. absolute = fixed-epsilon hit test.
enum { MARCH_CONTINUE = 0, MARCH_HIT = 1, MARCH_MISS = 2, MARCH_EXHAUSTED = 3 };
// The best candidate's sample is not kept: a candidate accepted at the step
// budget is re-evaluated at cand_t (same point, same code, same sample).
struct March {
    float3 ro, rd;
    float t, omega, prev_radius, step_len, t_end;
    float cand_t, cand_err;
    uint32_t i;  // steps taken
};
__device__ __forceinline__ void march_begin(March& m, float3 ro, float3 rd, float t_end) {
    m.ro = ro; m.rd = rd; m.t = 0.0f; m.omega = 1.2f; m.prev_radius = 0.0f; m.step_len = 0.0f;
    m.t_end = t_end; m.cand_t = 0.0f; m.cand_err = 1e30f; m.i = 0;
}
// Before a step: decide whether the march continues; returns MARCH_CONTINUE when a
// DE evaluation at m.ro + m.rd * m.t is needed. MARCH_HIT here means the step
// budget ended on an accepted candidate (at m.cand_t).
__device__ __forceinline__ int march_check(const March& m, uint32_t max_steps, float accept) {
    if (m.i >= max_steps) return m.cand_err < accept * 4.0f ? MARCH_HIT : MARCH_EXHAUSTED;
    if (m.t >= m.t_end) return MARCH_MISS;
    return MARCH_CONTINUE;
}
// After the DE distance d at the current t: MARCH_HIT (hit at m.t), MARCH_MISS
// (proven clear) or MARCH_CONTINUE (t advanced). A flagged sample (a skipped
// Bounded branch's bound) steps the march but is never a hit or a candidate.
__device__ __forceinline__ int march_update(March& m, float d, uint32_t flags, float safety, float accept,
                                            bool absolute) {
    m.i += 1;
    float radius = fabsf(d) * safety;
    bool sor_fail = m.omega > 1.0f && (radius + m.prev_radius) < m.step_len * 1.0001f;
    if (sor_fail) { m.step_len = m.step_len - m.omega * m.step_len; m.omega = 1.0f; }
    else m.step_len = radius * m.omega;
    m.prev_radius = radius;
    float err = absolute ? radius : radius * rcp_approx(fmaxf(m.t, 1e-6f));
    const bool exact = flags == 0u;
    if (!sor_fail && exact && err < m.cand_err) { m.cand_t = m.t; m.cand_err = err; }
    if (!sor_fail && exact && (absolute ? err <= accept : err < accept)) return MARCH_HIT;
    if (!sor_fail && m.t + m.step_len >= m.t_end) {
        if (radius >= m.t_end - m.t) return MARCH_MISS;
        m.omega = 1.0f;
        m.step_len = radius;
    }
    m.t += m.step_len;
    return MARCH_CONTINUE;
}

// The scene's hit rule: a fixed epsilon when the render asks for one, else the
// reference's cone-relative test at the pixel tolerance.
__device__ __forceinline__ bool hit_absolute(const DevScene& S) { return S.hit_eps > 0.0f; }
__device__ __forceinline__ float hit_accept(const DevScene& S) {
    return S.hit_eps > 0.0f ? S.hit_eps : S.pixel_cone * S.pixel_tolerance;
}

// ------------------------------------------------------------------ shading arithmetic
// The shading code below (not the march and not the DE) uses WGSL's accuracy class
// for division (2.5 ulp) and sqrt: PTX div.approx / sqrt.approx and the reciprocal
// square root, a few ulp each, instead of the correctly rounded slow paths.
__device__ __forceinline__ float wdiv(float a, float b) {
    float q;
    asm("div.approx.ftz.f32 %0, %1, %2;" : "=f"(q) : "f"(a), "f"(b));
    return q;
}
__device__ __forceinline__ float wsqrt(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float3 wnormalize(float3 v) { return v * rsqrtf(dot3(v, v)); }
// glam try_normalize().unwrap_or(Y) (common.wgsl:241-246) with the reciprocal square root.
__device__ __forceinline__ float3 wsafe_normalize(float3 v) {
    const float l2 = dot3(v, v);
    const float r = rsqrtf(l2);
    if (!(l2 > 0.0f) || !(r <= 3.4028235e38f)) return mk3(0.f, 1.f, 0.f);
    return v * r;
}

// ------------------------------------------------------------------ lights (lights.wgsl)
// A scene's lights past SF_SHARED_LIGHTS, staged from its light table (after the scene
// in device memory, SF_LIGHT_TABLE_OFFSET) into dynamic
// shared memory by the kernels that read lights (stage_more_lights); the launch gives
// (light_count - SF_SHARED_LIGHTS) * sizeof(DevLight) bytes, none for up to 8 lights.
extern __shared__ __align__(16) DevLight sf_more_lights[];
__device__ __forceinline__ void stage_more_lights(const DevScene* scene_g) {
    const uint32_t n = scene_g->light_count;
    if (n <= SF_SHARED_LIGHTS) return;
    uint32_t avail;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(avail));
    const uint32_t words = min((n - SF_SHARED_LIGHTS) * uint32_t(sizeof(DevLight) / 4), avail / 4u);
    const uint32_t* s = reinterpret_cast<const uint32_t*>(reinterpret_cast<const char*>(scene_g) + SF_LIGHT_TABLE_OFFSET);
    uint32_t* d = reinterpret_cast<uint32_t*>(sf_more_lights);
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) d[i] = __ldg(s + i);
}
// Light i of the scene: the first SF_SHARED_LIGHTS staged with the scene, the rest
// staged by stage_more_lights; both in shared memory.
__device__ __forceinline__ const DevLight& light_of(const DevScene& S, uint32_t i) {
    if (i < SF_SHARED_LIGHTS) return S.lights[i];
    return sf_more_lights[i - SF_SHARED_LIGHTS];
}
__device__ __forceinline__ float area_intersection(float3 ro, float3 rd, const DevLight& l) {
    float3 n = ld3(l.n);
    float den = dot3(n, rd);
    if (fabsf(den) < 1e-7f) return 1e30f;
    float t = dot3(ld3(l.a) - ro, n) / den;
    if (t <= 1e-6f) return 1e30f;
    float3 q = ro + rd * t - ld3(l.a);
    float x = dot3(q, ld3(l.b)) * l.inv_bb;
    float y = dot3(q, ld3(l.c)) * l.inv_cc;
    if (fabsf(x) > 0.5f || fabsf(y) > 0.5f) return 1e30f;
    return t;
}
// Emitters (lights.wgsl:5-168): rectangles, projectors (a rectangle with a beam) and
// tubes (capsules) are hit by rays and sampled for next events. Their arithmetic is
// rounded operation by operation (e_add .. e_mul, explicit fmaf), so the kernels that
// inline it round it alike and the two integrators stay equal bit for bit.
__device__ __forceinline__ float3 e_add(float3 a, float3 b) {
    return mk3(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z));
}
__device__ __forceinline__ float3 e_sub(float3 a, float3 b) {
    return mk3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}
__device__ __forceinline__ float3 e_mul(float3 a, float s) {
    return mk3(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s));
}
__device__ __forceinline__ bool is_emitter(const DevLight& l) {
    return l.kind == SF_LIGHT_AREA || l.kind == SF_LIGHT_TUBE;
}
// beam_profile (lights.wgsl:11-16): the projector's smootherstep from its outer cone
// to its inner one; 1 for the other emitters.
__device__ __forceinline__ float beam_profile(const DevLight& l, float3 direction) {
    if (!l.projector) return 1.0f;
    const float cosine = dot3(ld3(l.n), direction);
    const float t = fminf(
        fmaxf(wdiv(__fsub_rn(cosine, l.beam[1]), fmaxf(__fsub_rn(l.beam[0], l.beam[1]), 1e-7f)), 0.0f), 1.0f);
    return __fmul_rn(__fmul_rn(__fmul_rn(t, t), t), fmaf(t, fmaf(6.0f, t, -15.0f), 10.0f));
}
__device__ __forceinline__ float3 emitter_radiance(const DevLight& l, float3 direction) {
    return e_mul(ld3(l.color), beam_profile(l, direction));
}
// cone_segment (lights.wgsl:23-68): the part of [0, end] of a ray inside the positive
// cone of apex, axis and cosine; empty as (1, 0).
static __device__ float2 cone_segment(float3 ro, float3 rd, float end, float3 apex, float3 axis, float cosine) {
    float2 interval = make_float2(0.0f, end);
    const float3 delta = e_sub(ro, apex);
    const float axial = dot3(delta, axis), slope = dot3(rd, axis);
    if (fabsf(slope) < 1e-8f) {
        if (axial < 0.0f) return make_float2(1.0f, 0.0f);
    } else {
        const float crossing = wdiv(-axial, slope);
        if (slope > 0.0f) interval.x = fmaxf(interval.x, crossing);
        else interval.y = fminf(interval.y, crossing);
    }
    if (interval.y <= interval.x) return make_float2(1.0f, 0.0f);
    const float c2 = __fmul_rn(cosine, cosine);
    const float s2 = __fmul_rn(__fsub_rn(1.0f, cosine), __fadd_rn(1.0f, cosine));
    const float3 radial = e_sub(delta, e_mul(axis, axial));
    const float3 radial_slope = e_sub(rd, e_mul(axis, slope));
    const float a = __fsub_rn(__fmul_rn(__fmul_rn(s2, slope), slope), __fmul_rn(c2, dot3(radial_slope, radial_slope)));
    const float b = __fmul_rn(2.0f, __fsub_rn(__fmul_rn(__fmul_rn(s2, axial), slope),
                                              __fmul_rn(c2, dot3(radial, radial_slope))));
    const float c = __fsub_rn(__fmul_rn(__fmul_rn(s2, axial), axial), __fmul_rn(c2, dot3(radial, radial)));
    if (fabsf(a) < 1e-12f) {
        if (fabsf(b) < 1e-12f) {
            if (c < 0.0f) return make_float2(1.0f, 0.0f);
        } else if (b > 0.0f) {
            interval.x = fmaxf(interval.x, wdiv(-c, b));
        } else {
            interval.y = fminf(interval.y, wdiv(-c, b));
        }
        return interval;
    }
    const float discriminant = __fsub_rn(__fmul_rn(b, b), __fmul_rn(__fmul_rn(4.0f, a), c));
    if (discriminant <= 0.0f) {
        const float middle = __fmul_rn(__fadd_rn(interval.x, interval.y), 0.5f);
        if (__fadd_rn(__fmul_rn(__fadd_rn(__fmul_rn(a, middle), b), middle), c) < 0.0f) return make_float2(1.0f, 0.0f);
        return interval;
    }
    const float root = wsqrt(discriminant);
    const float q = __fmul_rn(-0.5f, __fadd_rn(b, b >= 0.0f ? root : -root));
    const float r0 = wdiv(q, a), r1 = wdiv(c, q);
    const float low = fminf(r0, r1), high = fmaxf(r0, r1);
    if (a < 0.0f) return make_float2(fmaxf(interval.x, low), fminf(interval.y, high));
    if (fminf(interval.y, low) > interval.x) return make_float2(interval.x, fminf(interval.y, low));
    return make_float2(fmaxf(interval.x, high), interval.y);
}
// projector_bound_apex (lights.wgsl:72-75): the apex of a cone bounding the whole
// rectangle's beam, moved back by its half diagonal over tan(outer).
__device__ __forceinline__ float3 projector_bound_apex(const DevLight& l) {
    const float3 d = e_add(ld3(l.b), ld3(l.c));
    const float radius = __fmul_rn(0.5f, wsqrt(dot3(d, d)));
    return e_sub(ld3(l.a), e_mul(ld3(l.n), wdiv(radius, l.beam[2])));
}
// emitter_normal (lights.wgsl:87-94): a tube's normal is radial from its axis.
__device__ __forceinline__ float3 emitter_normal(const DevLight& l, float3 point) {
    if (l.kind != SF_LIGHT_TUBE) return ld3(l.n);
    const float3 axis = e_sub(ld3(l.b), ld3(l.a));
    const float3 pa = e_sub(point, ld3(l.a));
    const float t = fminf(fmaxf(wdiv(dot3(pa, axis), dot3(axis, axis)), 0.0f), 1.0f);
    return wsafe_normalize(e_sub(pa, e_mul(axis, t)));
}
// tube_intersection (lights.wgsl:97-129): the closest hit of the cylinder and its two
// spherical caps.
static __device__ float tube_intersection(float3 ro, float3 rd, const DevLight& l) {
    const float3 A = ld3(l.a), B = ld3(l.b);
    const float r = l.radius, len = l.length;
    const float r2 = __fmul_rn(r, r);
    const float3 axis = e_mul(e_sub(B, A), wdiv(1.0f, len));
    const float3 oa = e_sub(ro, A);
    const float axial_ray = dot3(axis, rd), axial_origin = dot3(axis, oa);
    const float3 side = cross3(axis, rd);
    const float a = dot3(side, side);
    float nearest = 1e30f;
    if (a > 1e-10f) {
        const float perpendicular = wdiv(dot3(oa, side), wsqrt(a));
        const float h = __fsub_rn(r2, __fmul_rn(perpendicular, perpendicular));
        if (h < 0.0f) return nearest;
        const float middle = wdiv(-__fsub_rn(dot3(rd, oa), __fmul_rn(axial_origin, axial_ray)), a);
        const float root = wsqrt(wdiv(fmaxf(0.0f, h), a));
        for (int i = 0; i < 2; ++i) {
            const float t = __fadd_rn(middle, i == 1 ? root : -root);
            const float y = __fadd_rn(axial_origin, __fmul_rn(t, axial_ray));
            if (t > 1e-6f && y >= 0.0f && y <= len) nearest = fminf(nearest, t);
        }
    } else {
        const float3 radial = e_sub(oa, e_mul(axis, axial_origin));
        if (dot3(radial, radial) > r2) return nearest;
    }
    for (int cap = 0; cap < 2; ++cap) {
        const float3 oc = e_sub(ro, cap == 1 ? B : A);
        const float projection = dot3(oc, rd);
        const float3 closest = e_sub(oc, e_mul(rd, projection));
        const float h = __fsub_rn(r2, dot3(closest, closest));
        if (h < 0.0f) continue;
        const float sh = wsqrt(h);
        for (int i = 0; i < 2; ++i) {
            const float t = __fadd_rn(-projection, i == 1 ? sh : -sh);
            const float y = dot3(e_sub(e_add(ro, e_mul(rd, t)), A), axis);
            const bool on_cap = cap == 1 ? y >= len : y <= 0.0f;
            if (t > 1e-6f && on_cap) nearest = fminf(nearest, t);
        }
    }
    return nearest;
}
__device__ __forceinline__ float emitter_intersection(float3 ro, float3 rd, const DevLight& l) {
    return l.kind == SF_LIGHT_TUBE ? tube_intersection(ro, rd, l) : area_intersection(ro, rd, l);
}
// sample_emitter_point (lights.wgsl:143-160): a rectangle's point from (u, v); a
// tube's from (choice, polar, phi): its cylinder by area, else one of its caps.
struct EmitterPoint {
    float3 position, normal;
};
__device__ __forceinline__ void tangent_frame(float3 n, float3& t, float3& bt);
static __device__ EmitterPoint sample_emitter_point(const DevLight& l, float u, float v, float w) {
    EmitterPoint e;
    if (l.kind != SF_LIGHT_TUBE) {
        e.position = e_add(e_add(ld3(l.a), e_mul(ld3(l.b), __fsub_rn(u, 0.5f))), e_mul(ld3(l.c), __fsub_rn(v, 0.5f)));
        e.normal = ld3(l.n);
        return e;
    }
    const float3 A = ld3(l.a), B = ld3(l.b);
    const float3 axis = e_mul(e_sub(B, A), wdiv(1.0f, l.length));
    float3 t, bt;
    tangent_frame(axis, t, bt);
    float sp, cp;
    sincosf(__fmul_rn(2.0f * SF_PI, w), &sp, &cp);
    const float3 radial = e_add(e_mul(t, cp), e_mul(bt, sp));
    const float cylinder_fraction = wdiv(l.length, __fadd_rn(l.length, __fmul_rn(2.0f, l.radius)));
    if (u < cylinder_fraction) {
        const float g = __fsub_rn(1.0f, v);  // mix(a, b, polar)
        e.position = e_add(e_add(e_mul(A, g), e_mul(B, v)), e_mul(radial, l.radius));
        e.normal = radial;
        return e;
    }
    const bool top = wdiv(__fsub_rn(u, cylinder_fraction), __fsub_rn(1.0f, cylinder_fraction)) >= 0.5f;
    const float3 n = e_add(e_mul(radial, wsqrt(fmaxf(0.0f, __fsub_rn(1.0f, __fmul_rn(v, v))))),
                           e_mul(axis, top ? v : -v));
    e.position = e_add(top ? B : A, e_mul(n, l.radius));
    e.normal = n;
    return e;
}
// area_weight (lights.wgsl:285-302): the selection weight of an emitter at p.
__device__ __forceinline__ float area_weight(float3 p, float3 n, const DevLight& l) {
    const bool tube = l.kind == SF_LIGHT_TUBE;
    const float3 center = tube ? (ld3(l.a) + ld3(l.b)) * 0.5f : ld3(l.a);
    float3 to_light = center - p;
    float dist2 = fmaxf(dot3(to_light, to_light), 1e-6f);
    float3 dir = to_light * rsqrtf(dist2);
    float facing = tube ? 0.25f : fmaxf(dot3(ld3(l.n), -dir), 0.0f);
    if (l.projector) {
        const float3 delta = p - projector_bound_apex(l);
        const float axial = dot3(delta, ld3(l.n));
        if (axial < 0.0f || axial * axial < l.beam[1] * l.beam[1] * dot3(delta, delta)) return 0.0f;
        facing *= fmaxf(0.025f, beam_profile(l, -dir));
    }
    return wdiv(l.lum * l.area * facing * fmaxf(dot3(n, dir), 0.15f), dist2);
}
__device__ __forceinline__ float area_total_weight(const DevScene& S, float3 p, float3 n) {
    float total = 0.0f;
    for (uint32_t i = 0; i < S.light_count; ++i)
        if (is_emitter(light_of(S, i))) total += area_weight(p, n, light_of(S, i));
    return total;
}
__device__ __forceinline__ float mis_power(float a, float b) {
    float scale = fmaxf(a, b);
    if (scale <= 0.0f) return 0.0f;
    float pa = wdiv(a, scale), pb = wdiv(b, scale);
    return wdiv(pa * pa, fmaf(pa, pa, pb * pb));
}
// Emitter hit by a continuation ray (area_emission, lights.wgsl:330-356).
static __device__ float3 area_emission(const DevScene& S, float3 ro, float3 rd, float distance, float prev_pdf, bool use_mis,
                                float3 prev_normal, float prev_total) {
    float3 L = mk3(0.f, 0.f, 0.f);
    for (uint32_t i = 0; i < S.light_count; ++i) {
        const DevLight& l = light_of(S, i);
        if (!is_emitter(l)) continue;
        float cos_l = dot3(emitter_normal(l, e_add(ro, e_mul(rd, distance))), -rd);
        if (cos_l <= 0.0f) continue;
        float t = emitter_intersection(ro, rd, l);
        if (fabsf(t - distance) > fmaxf(1e-6f, distance * 1e-6f)) continue;
        float w = 1.0f;
        if (use_mis) {
            float pl = wdiv(distance * distance, fmaxf(l.area * cos_l, 1e-20f));
            float selection = 0.0f;
            if (prev_total > 0.0f) selection = wdiv(area_weight(ro, prev_normal, l), prev_total);
            pl = pl * selection;
            w = mis_power(prev_pdf, pl);
        }
        L = L + emitter_radiance(l, -rd) * w;
    }
    return L;
}
// Nearest emitter along a ray, before the geometry march (trace_geometry_lights).
__device__ __forceinline__ float nearest_emitter(const DevScene& S, float3 ro, float3 rd, float t_end, uint32_t& li) {
    float nearest = t_end;
    li = SF_NO_LIGHT;
    for (uint32_t i = 0; i < S.light_count; ++i) {
        if (!is_emitter(light_of(S, i))) continue;
        float t = emitter_intersection(ro, rd, light_of(S, i));
        if (t < nearest) { nearest = t; li = i; }
    }
    return nearest;
}

// ------------------------------------------------------------------ BRDF
struct Surface {
    float3 n, diffuse, f0, emission;
    float alpha;
    float diffuse_sigma;  // > 0: Oren-Nayar rough diffuse (concrete finish details)
};
__device__ __forceinline__ float luminance(float3 c) { return fmaf(c.z, 0.0722f, fmaf(c.x, 0.2126f, c.y * 0.7152f)); }
__device__ __forceinline__ void tangent_frame(float3 n, float3& t, float3& bt) {
    float s = n.z >= 0.0f ? 1.0f : -1.0f;
    float a = wdiv(-1.0f, s + n.z);
    float b = n.x * n.y * a;
    t = mk3(1.0f + s * n.x * n.x * a, s * b, -s * n.x);
    bt = mk3(b, s + n.y * n.y * a, -n.y);
}
// t*v.x + bt*v.y + n*v.z and x*(1-f) + y*f with fixed fusion (the first product of
// each sum fused last), so every kernel that inlines them rounds the same way.
__device__ __forceinline__ float3 frame_mul(float3 t, float3 bt, float3 n, float3 v) {
    return mk3(fmaf(n.x, v.z, fmaf(t.x, v.x, bt.x * v.y)), fmaf(n.y, v.z, fmaf(t.y, v.x, bt.y * v.y)),
               fmaf(n.z, v.z, fmaf(t.z, v.x, bt.z * v.y)));
}
// L + c rounded as an add (never fused with the product that made c): the wavefront
// adds a shadow segment's radiance from memory a round later, the megakernel inline.
__device__ __forceinline__ float3 add_rn(float3 a, float3 b) {
    return mk3(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z));
}
__device__ __forceinline__ float3 lerp3(float3 x, float3 y, float f) {
    const float g = 1.0f - f;
    return mk3(fmaf(x.x, g, y.x * f), fmaf(x.y, g, y.y * f), fmaf(x.z, g, y.z * f));
}
__device__ __forceinline__ float3 cosine_sample(float3 n, float r1, float r2) {
    float phi = 2.0f * SF_PI * r1;
    float r = wsqrt(r2);
    float3 t, bt;
    tangent_frame(n, t, bt);
    float sp, cp;
    sincosf(phi, &sp, &cp);
    return frame_mul(t, bt, n, mk3(r * cp, r * sp, wsqrt(fmaxf(0.0f, 1.0f - r2))));
}
__device__ __forceinline__ float ggx_d(float nh, float a2) {
    float d = nh * nh * (a2 - 1.0f) + 1.0f;
    return wdiv(a2, SF_PI * d * d);
}
__device__ __forceinline__ float smith_g1(float nv, float a2) {
    return wdiv(2.0f * nv, nv + wsqrt(a2 + (1.0f - a2) * nv * nv));
}
__device__ __forceinline__ float3 fresnel(float3 f0, float vh) {
    float m = 1.0f - vh;
    float m2 = m * m;
    float p5 = m2 * m2 * m;  // pow(1 - vh, 5)
    return f0 + (mk3(1.f, 1.f, 1.f) - f0) * p5;
}
static __device__ float3 sample_ggx_h(float3 n, float3 v, float alpha, float r1, float r2) {
    float3 t, bt;
    tangent_frame(n, t, bt);
    float3 lv = mk3(dot3(t, v), dot3(bt, v), dot3(n, v));
    float3 vh = wsafe_normalize(mk3(alpha * lv.x, alpha * lv.y, fmaxf(lv.z, 1e-5f)));
    float lensq = fmaf(vh.x, vh.x, vh.y * vh.y);
    float3 t1 = mk3(1.f, 0.f, 0.f);
    if (lensq > 0.0f) t1 = mk3(-vh.y, vh.x, 0.0f) * rsqrtf(lensq);
    float3 t2 = cross3(vh, t1);
    float r = wsqrt(r1);
    float phi = 2.0f * SF_PI * r2;
    float sp, cp;
    sincosf(phi, &sp, &cp);
    float x = r * cp;
    float blend = 0.5f * (1.0f + vh.z);
    float y0 = wsqrt(fmaxf(0.0f, 1.0f - x * x));
    float y = fmaf(y0, 1.0f - blend, (r * sp) * blend);
    float3 nh = frame_mul(t1, t2, vh, mk3(x, y, wsqrt(fmaxf(0.0f, fmaf(-y, y, fmaf(-x, x, 1.0f))))));
    return frame_mul(t, bt, n, wsafe_normalize(mk3(alpha * nh.x, alpha * nh.y, fmaxf(nh.z, 0.0f))));
}
static __device__ float3 brdf_eval(const Surface& s, float3 v, float3 l) {
    float nl = dot3(s.n, l), nv = dot3(s.n, v);
    if (nl <= 0.0f || nv <= 0.0f) return mk3(0.f, 0.f, 0.f);
    float3 h = wnormalize(v + l);
    float nh = fmaxf(dot3(s.n, h), 0.0f);
    float vh = fmaxf(dot3(v, h), 0.0f);
    float a2 = s.alpha * s.alpha;
    float3 f = fresnel(s.f0, vh);
    float3 spec = f * wdiv(ggx_d(nh, a2) * smith_g1(nv, a2) * smith_g1(nl, a2), fmaxf(4.0f * nv * nl, 1e-4f));
    if (s.diffuse_sigma > 0.0f) {
        // Oren-Nayar reflectance (pathtrace.wgsl:408-419); the lobe stays cosine-sampled
        const float sigma2 = s.diffuse_sigma * s.diffuse_sigma;
        const float a = 1.0f - wdiv(sigma2, 2.0f * (sigma2 + 0.33f));
        const float b = wdiv(0.45f * sigma2, sigma2 + 0.09f);
        const float sin_l = wsqrt(fmaxf(0.0f, 1.0f - nl * nl));
        const float sin_v = wsqrt(fmaxf(0.0f, 1.0f - nv * nv));
        const float cos_phi = fmaxf(0.0f, wdiv(dot3(l - s.n * nl, v - s.n * nv), fmaxf(sin_l * sin_v, 1e-8f)));
        const float factor = a + wdiv(b * cos_phi * sin_l * sin_v, fmaxf(fmaxf(nl, nv), 1e-5f));
        return s.diffuse * (mk3(1.f, 1.f, 1.f) - f) * (factor * (1.0f / SF_PI)) + spec;
    }
    return s.diffuse * (mk3(1.f, 1.f, 1.f) - f) * (1.0f / SF_PI) + spec;
}
__device__ __forceinline__ float spec_probability(const Surface& s, float nv) {
    float3 f = fresnel(s.f0, nv);
    return fminf(fmaxf(wdiv(luminance(f), fmaxf(luminance(f) + luminance(s.diffuse), 1e-4f)), 0.05f), 0.95f);
}
static __device__ float bsdf_pdf(const Surface& s, float3 v, float3 l, float p_spec) {
    float nl = dot3(s.n, l);
    if (nl <= 0.0f) return 0.0f;
    float3 hh = wnormalize(v + l);
    float nh = fmaxf(dot3(s.n, hh), 0.0f);
    float a2 = s.alpha * s.alpha;
    float nv = fmaxf(dot3(s.n, v), 1e-4f);
    float pdf_spec = wdiv(ggx_d(nh, a2) * smith_g1(nv, a2), 4.0f * nv);
    return fmaf(p_spec, pdf_spec, (1.0f - p_spec) * nl * (1.0f / SF_PI));
}
// make_surface (pathtrace.wgsl:271-386): the colouring ramp or orbit mix, the finish
// of a MaterialTag, surface variation, the finish's world-space detail and, on
// untagged surfaces, the volumetric texture. FEAT selects what the calling kernel is
// built with: SF_FEAT_RICH (finish details, optics, the footprint), SF_FEAT_TEX (the
// texture's interpreter); 0 is the plain surface. p is the hit point, n the
// shading-side normal, v toward the eye and footprint the path's texture width.
template <int FEAT = 0>
static __device__ Surface make_surface(const DevScene& S, float3 p, float3 n, float3 v, const DeSampleF& smp,
                                       float footprint) {
    const DevMaterial* m = &S.material;
    const bool assigned = smp.material > 0 && smp.material <= S.finish_count;
    if (assigned) m = &S.finishes[smp.material - 1];
    float3 albedo = ld3(m->albedo);
    if (!assigned && S.col.n) {  // the colouring ramp (pathtrace.wgsl:275-288)
        const uint32_t slot = S.col_slot;
        const float iter_frac = float(smp.iter) / fmaxf(float(S.iteration_product), 1.0f);
        if (slot == 6) albedo = albedo * ramp_sample(S.col, orbit_mix(S.col_weights, S.col_extra, smp.traps, iter_frac,
                                                                      n.y * 0.5f + 0.5f));
        else if (slot < 4) albedo = albedo * ramp_sample(S.col, smp.traps[slot]);
        else if (slot == 5) albedo = albedo * ramp_sample(S.col, n.y * 0.5f + 0.5f);
        else if (slot == 4) albedo = albedo * ramp_sample(S.col, iter_frac);
    }
    float rough = m->roughness, metallic = m->metallic, spec = m->specular;
    float3 emission = assigned ? ld3(m->emission) : mk3(0.f, 0.f, 0.f);
    if (!assigned && S.variation_enabled) {
        uint32_t slot = S.variation_slot;
        float value = slot < 4 ? smp.traps[slot]
                               : (slot == 5 ? n.y * 0.5f + 0.5f : float(smp.iter) / fmaxf(float(S.iteration_product), 1.0f));
        float t = fminf(fmaxf(value, 0.0f), 1.0f);
        rough = S.var_rough[0] + (S.var_rough[1] - S.var_rough[0]) * t;
        metallic = S.var_metal[0] + (S.var_metal[1] - S.var_metal[0]) * t;
    }
    float3 shading_n = n;
    float diffuse_sigma = 0.0f;
    if ((FEAT & SF_FEAT_RICH) && assigned && (S.rich & SF_RICH_DETAIL) && S.details[smp.material - 1].kind != 0u) {
        const DevDetail& f = S.details[smp.material - 1];
        float4 detail = finish_eval(f, p, footprint, S.dune_wind);
        if (f.kind == 9u) detail = scale4(detail, sstep(0.10f, 0.80f, n.y));  // powder settles on tops
        if (f.kind == 12u) detail.w *= sstep(0.45f, 0.95f, n.y);
        const float value = detail.w;
        const float amount = f.mapping[1] * value;
        albedo = mk3(mixf(albedo.x, f.tint[0], amount), mixf(albedo.y, f.tint[1], amount),
                     mixf(albedo.z, f.tint[2], amount));
        if (f.kind == 9u) {
            rough += fmaxf(f.mapping[3], 0.0f) * amount;
            metallic *= 1.0f - amount;
            spec = mixf(spec, 0.025f, amount);
        } else if (f.kind == 12u) {
            rough = mixf(rough, fminf(fmaxf(rough + f.mapping[3], 0.025f), 1.0f), amount);
            spec = mixf(spec, 0.0204f, amount);
            metallic *= 1.0f - amount;
        } else {
            rough += f.mapping[3] * (2.0f * value - 1.0f);
        }
        if (f.kind == 2u) metallic *= 1.0f - 0.75f * amount;
        if (fabsf(f.mapping[2]) > 0.0f) shading_n = finish_normal(f.mapping[2], n, xyz(detail));
        if (f.kind >= 10u) diffuse_sigma = 1.0f;  // times the final roughness below
    }
    if constexpr ((FEAT & SF_FEAT_TEX) != 0) {
        const DevTexture& T = S.tex;
        const float amount = texture_mask(T, smp.traps);
        if (!assigned && T.effects[3] > 0.0f && amount > 0.0f) {
            const float3 tex_p = texture_parallax(T, p, n, v, footprint);
            const float value = texture_filtered_value(T, tex_p, footprint);
            const float3 c = ramp_sample(T.ramp, value);
            const float k = T.effects[0] * amount;
            albedo = albedo * mk3(mixf(1.0f, c.x, k), mixf(1.0f, c.y, k), mixf(1.0f, c.z, k));
            rough = mixf(rough, value, T.effects[1] * amount);
            if (T.effects[2] > 0.0f) {
                const float3 tn = texture_normal(T, tex_p, n, footprint);
                shading_n = safe_normalize3(mk3(mixf(n.x, tn.x, amount), mixf(n.y, tn.y, amount), mixf(n.z, tn.z, amount)));
            }
        }
    }
    rough = fminf(fmaxf(rough, 0.02f), 1.0f);
    Surface s;
    s.n = shading_n;
    s.diffuse = albedo * (1.0f - metallic);
    s.f0 = mk3(spec, spec, spec) * (1.0f - metallic) + albedo * metallic;
    s.alpha = rough * rough;
    s.emission = emission;
    s.diffuse_sigma = (FEAT & SF_FEAT_RICH) ? diffuse_sigma * rough * 0.45f : 0.0f;
    return s;
}

// ------------------------------------------------------------------ path state
struct PathState {
    float3 o, d, tp, L, prev_normal;
    float3 pv;  // primary_volume (pathtrace.wgsl:821): the camera segment's in-scattered emitter light
    float prev_pdf, prev_area_total;
    uint32_t rng, bounce;
    bool prev_from_bsdf;
    bool prev_from_volume;  // the segment left a fog scattering point (its emitters were estimated there)
    bool volume_path;       // the camera segment scattered in the fog (pathtrace.wgsl:822)
    // rich surfaces (DevScene.rich != 0): the transported texture footprint
    // (pathtrace.wgsl:811-814) and the optics state (:830-840): inside a solid
    // dielectric medium of finish slot medium_slot, coverage null events taken.
    float tex_width, tex_spread;
    bool solid_medium;
    uint32_t medium_slot, null_surfaces;
};
// The sample's volume part for the film's volume planes (pathtrace.wgsl:1198).
__device__ __forceinline__ float3 path_volume(const PathState& ps) { return ps.volume_path ? ps.L : ps.pv; }
// Result of a continuation trace (Hit of pathtrace.wgsl:60-74 plus the normal).
struct HitInfo {
    bool hit, exhausted;
    float t;
    uint32_t steps, light_index;
    DeSampleF sample;
    float3 n;  // geometric normal at a surface hit (tetrahedral, common.wgsl:376-387)
};
// Next-event request: a visibility segment and the radiance it carries if clear.
struct ShadowReq {
    float3 o, dir;
    float t_end;
    float3 contrib;
    bool volume = false;  // the camera segment's in-scattered light: also counted in PathState.pv
};
#define SF_MAX_SHADOWS 8  // shadow requests of one bounce: at most one per light
enum { PATH_CONTINUE = 1, PATH_DONE = 0 };

__device__ __forceinline__ void path_begin(const DevScene& S, PathState& ps, uint32_t px, uint32_t py, uint32_t sample) {
    ps.rng = rng_init(px, py, sample, S.seed);
    camera_ray(S, px, py, ps.rng, ps.o, ps.d);
    ps.tp = mk3(1.f, 1.f, 1.f);
    ps.L = mk3(0.f, 0.f, 0.f);
    ps.prev_normal = mk3(0.f, 0.f, 0.f);
    ps.prev_pdf = 0.0f;
    ps.prev_area_total = 0.0f;
    ps.prev_from_bsdf = false;
    ps.prev_from_volume = false;
    ps.pv = mk3(0.f, 0.f, 0.f);
    ps.volume_path = false;
    ps.bounce = 0;
    ps.tex_width = 0.0f;
    ps.tex_spread = S.pixel_cone * 0.5f;
    ps.solid_medium = false;
    ps.medium_slot = 0;
    ps.null_surfaces = 0;
}

// ------------------------------------------------------------------ optics (optics.wgsl)
// material_optics (optics.wgsl:1-3): finish slots beyond the finish count read slot 0.
__device__ __forceinline__ const DevOptics& material_optics(const DevScene& S, uint32_t index) {
    return S.optics[index <= S.finish_count ? index : 0u];
}
__device__ __forceinline__ bool optics_enabled(const DevOptics& o) { return o.absorption[3] > 0.0f; }
// The medium a path starts in (pathtrace.wgsl:833-840): inside a transmissive solid
// (not a thin sheet) with optics when the exact sample at the ray origin is negative.
__device__ __forceinline__ void optics_initial_medium(const DevScene& S, PathState& ps, float d, uint32_t material) {
    const DevOptics& o = material_optics(S, material);
    ps.solid_medium = d < 0.0f && optics_enabled(o) && o.surface[1] > 0.0f && o.surface[3] == 0.0f;
    ps.medium_slot = material;
}
// ocean_fresnel (ocean.wgsl:151-159): unpolarised dielectric reflectance.
__device__ __forceinline__ float dielectric_fresnel(float cosine, float eta) {
    const float ci = fminf(fmaxf(fabsf(cosine), 0.0f), 1.0f);
    const float st2 = eta * eta * (1.0f - ci * ci);
    if (st2 >= 1.0f) return 1.0f;
    const float ct = wsqrt(fmaxf(0.0f, 1.0f - st2));
    const float rs = wdiv(eta * ci - ct, fmaxf(eta * ci + ct, 1e-6f));
    const float rp = wdiv(ci - eta * ct, fmaxf(ci + eta * ct, 1e-6f));
    return 0.5f * (rs * rs + rp * rp);
}
// WGSL refract(e1, e2, eta): zero on total internal reflection.
__device__ __forceinline__ float3 refract3(float3 i, float3 n, float eta) {
    const float ni = dot3(n, i);
    const float k = 1.0f - eta * eta * (1.0f - ni * ni);
    if (k < 0.0f) return mk3(0.f, 0.f, 0.f);
    return i * eta - n * (eta * ni + wsqrt(k));
}
__device__ __forceinline__ float3 reflect3(float3 i, float3 n) { return i - n * (2.0f * dot3(n, i)); }
__device__ __forceinline__ float3 exp3(float3 a) { return mk3(expf(a.x), expf(a.y), expf(a.z)); }

// point_stream of radiance (pathtrace.wgsl:823): the pixel's rotation of the
// radical-inverse points.
__device__ __forceinline__ uint32_t point_stream_of(const DevScene& S, uint32_t px, uint32_t py) {
    return pcg(pcg(px ^ S.seed) ^ pcg(py ^ 0x27d4eb2du));
}

// ------------------------------------------------------------------ sky lights
// environment_value / _probability / _emission (pathtrace.wgsl:164-190).
__device__ __forceinline__ float3 environment_value(const DevLight& l, float3 dir) {
    if (dir.y >= 0.0f) return lerp3(ld3(l.b), ld3(l.a), wsqrt(dir.y));
    return lerp3(ld3(l.b), ld3(l.c), wsqrt(-dir.y));
}
__device__ __forceinline__ float environment_probability(const DevLight& l, float area_total) {
    if (l.energy <= 0.0f) return 0.0f;
    const float e = 4.0f * SF_PI * l.energy;
    return fminf(fmaxf(wdiv(e, e + area_total), 0.05f), 1.0f);
}
static __device__ float3 environment_emission(const DevScene& S, float3 dir, float pdf, bool use_mis, float3 n,
                                              bool from_volume, float area_total) {
    float3 L = mk3(0.f, 0.f, 0.f);
    for (uint32_t i = 0; i < S.light_count; ++i) {
        const DevLight& l = light_of(S, i);
        if (l.kind != SF_LIGHT_ENVIRONMENT) continue;
        float w = 1.0f;
        if (use_mis) {
            const float density = from_volume ? 1.0f / (4.0f * SF_PI) : fmaxf(dot3(n, dir), 0.0f) * (1.0f / SF_PI);
            w = mis_power(pdf, environment_probability(l, area_total) * density);
        }
        L = L + environment_value(l, dir) * w;
    }
    return L;
}
// sun_pdf, sun_radiance (pathtrace.wgsl:432-468): a disk of cos_max around a.
__device__ __forceinline__ float sun_pdf(float cos_max) { return wdiv(1.0f, 2.0f * SF_PI * fmaxf(1.0f - cos_max, 1e-7f)); }
static __device__ float3 sun_radiance(const DevScene& S, float3 dir, float pdf_bsdf, bool use_mis) {
    float3 L = mk3(0.f, 0.f, 0.f);
    for (uint32_t i = 0; i < S.light_count; ++i) {
        const DevLight& l = light_of(S, i);
        if (l.kind != SF_LIGHT_SUN || dot3(dir, ld3(l.a)) < l.cos_max) continue;
        const float pl = sun_pdf(l.cos_max);
        const float w = use_mis ? mis_power(pdf_bsdf, pl) : 1.0f;
        L = L + ld3(l.color) * (pl * w);
    }
    return L;
}
// HDRI panoramas (environment.wgsl:7-107): equirectangular texels (rgb, cdf), bilinear
// lookups, and a CDF proposal mixed with 1/16 uniform sampling.
#define SF_HDRI_UNIFORM_MIX 0.0625f
__device__ __forceinline__ float3 hdri_local(const DevLight& l, float3 d) {
    return mk3(fmaf(l.a[0], d.x, l.a[1] * d.z), d.y, fmaf(-l.a[1], d.x, l.a[0] * d.z));
}
__device__ __forceinline__ float3 hdri_world(const DevLight& l, float3 d) {
    return mk3(fmaf(l.a[0], d.x, -(l.a[1] * d.z)), d.y, fmaf(l.a[1], d.x, l.a[0] * d.z));
}
__device__ __forceinline__ float2 hdri_uv(const DevLight& l, float3 dir) {
    const float3 q = hdri_local(l, dir);
    const float u = atan2f(q.z, q.x) / (2.0f * SF_PI) + 1.0f;
    return make_float2(u - floorf(u), acosf(fminf(fmaxf(q.y, -1.0f), 1.0f)) / SF_PI);
}
__device__ __forceinline__ float hdri_cell_area(const DevLight& l, uint32_t row) {
    const float step = SF_PI / float(l.th);
    return (2.0f * SF_PI / float(l.tw)) * 2.0f * sinf((float(row) + 0.5f) * step) * sinf(step * 0.5f);
}
__device__ __forceinline__ float4 hdri_fetch(const DevLight& l, uint32_t index) {
    return __ldg(reinterpret_cast<const float4*>(l.texels) + index);
}
__device__ __forceinline__ float3 hdri_texel(const DevLight& l, int x, int y) {
    const int w = int(l.tw);
    const uint32_t col = uint32_t(((x % w) + w) % w);
    const uint32_t row = uint32_t(min(max(y, 0), int(l.th) - 1));
    const float4 t = hdri_fetch(l, row * l.tw + col);
    return mk3(t.x, t.y, t.z);
}
static __device__ float3 hdri_lookup(const DevLight& l, float3 dir) {
    const float2 uv = hdri_uv(l, dir);
    const float px = uv.x * float(l.tw) - 0.5f, py = uv.y * float(l.th) - 0.5f;
    const float bx = floorf(px), by = floorf(py);
    const float fx = px - bx, fy = py - by;
    const int x = int(bx), y = int(by);
    const float3 top = lerp3(hdri_texel(l, x, y), hdri_texel(l, x + 1, y), fx);
    const float3 bottom = lerp3(hdri_texel(l, x, y + 1), hdri_texel(l, x + 1, y + 1), fx);
    return lerp3(top, bottom, fy) * l.color[0];
}
static __device__ float hdri_pdf(const DevLight& l, float3 dir) {
    if (l.a[2] > 0.0f) return 1.0f / (4.0f * SF_PI);
    const float2 uv = hdri_uv(l, dir);
    const uint32_t col = min(uint32_t(uv.x * float(l.tw)), l.tw - 1);
    const uint32_t row = min(uint32_t(uv.y * float(l.th)), l.th - 1);
    const uint32_t index = row * l.tw + col;
    const float before = index > 0 ? hdri_fetch(l, index - 1).w : 0.0f;
    const float mass = fmaxf(hdri_fetch(l, index).w - before, 0.0f);
    return fmaf(1.0f - SF_HDRI_UNIFORM_MIX, wdiv(mass, hdri_cell_area(l, row)), SF_HDRI_UNIFORM_MIX / (4.0f * SF_PI));
}
static __device__ float3 hdri_sample(const DevLight& l, float r0, float r1, float r2) {
    float phi = 2.0f * SF_PI * r1;
    float cos_theta = 1.0f - 2.0f * r2;
    float sin_squared = fmaxf(0.0f, fmaf(-cos_theta, cos_theta, 1.0f));
    if (l.a[2] <= 0.0f && r0 >= SF_HDRI_UNIFORM_MIX) {
        const float cdf_sample = wdiv(r0 - SF_HDRI_UNIFORM_MIX, 1.0f - SF_HDRI_UNIFORM_MIX);
        uint32_t lo = 0, hi = l.tw * l.th;
        while (lo < hi) {  // the first texel whose cumulative share exceeds the sample
            const uint32_t mid = lo + (hi - lo) / 2u;
            if (hdri_fetch(l, mid).w <= cdf_sample) lo = mid + 1u;
            else hi = mid;
        }
        const uint32_t index = min(lo, l.tw * l.th - 1u);
        const uint32_t col = index % l.tw, row = index / l.tw;
        phi = 2.0f * SF_PI * (float(col) + r1) / float(l.tw);
        const float top = SF_PI * float(row) / float(l.th);
        const float bottom = SF_PI * float(row + 1u) / float(l.th);
        const float band = 2.0f * sinf((top + bottom) * 0.5f) * sinf((bottom - top) * 0.5f);
        const float cap = fmaf(r2, band, 2.0f * sinf(top * 0.5f) * sinf(top * 0.5f));
        const float lower_cap = fmaf(1.0f - r2, band, 2.0f * cosf(bottom * 0.5f) * cosf(bottom * 0.5f));
        if (row < l.th / 2u) {
            cos_theta = 1.0f - cap;
            sin_squared = cap * (2.0f - cap);
        } else {
            cos_theta = lower_cap - 1.0f;
            sin_squared = lower_cap * (2.0f - lower_cap);
        }
    }
    const float sin_theta = wsqrt(fmaxf(0.0f, sin_squared));
    float sp, cp;
    sincosf(phi, &sp, &cp);
    return hdri_world(l, mk3(sin_theta * cp, cos_theta, sin_theta * sp));
}
static __device__ float3 hdri_emission(const DevScene& S, float3 dir, float previous_pdf, bool use_mis) {
    float3 L = mk3(0.f, 0.f, 0.f);
    for (uint32_t i = 0; i < S.light_count; ++i) {
        const DevLight& l = light_of(S, i);
        if (l.kind != SF_LIGHT_HDRI) continue;
        const float w = use_mis ? mis_power(previous_pdf, hdri_pdf(l, dir)) : 1.0f;
        L = L + hdri_lookup(l, dir) * w;
    }
    return L;
}

// cone_sample (pathtrace.wgsl:210-215).
__device__ __forceinline__ float3 cone_sample(float3 dir, float cos_max, float r1, float r2) {
    const float cos_t = 1.0f - r1 * (1.0f - cos_max);
    const float sin_t = wsqrt(fmaxf(0.0f, 1.0f - cos_t * cos_t));
    float sp, cp;
    sincosf(2.0f * SF_PI * r2, &sp, &cp);
    float3 t, bt;
    tangent_frame(dir, t, bt);
    return frame_mul(t, bt, dir, mk3(sin_t * cp, sin_t * sp, cos_t));
}

// ------------------------------------------------------------------ height fog
// fog_sigma .. fog_free_flight (pathtrace.wgsl:562-615): the capped exponential
// height fog, its optical depth integrated exactly on each side of the fog height,
// and collision distances drawn by inverting that integral. S.fog = density, height,
// falloff, anisotropy.
__device__ __forceinline__ float fog_sigma(const DevScene& S, float3 p) {
    return S.fog[0] * expf(fminf(0.0f, -(p.y - S.fog[1]) * S.fog[2]));
}
static __device__ float fog_segment_tau(const DevScene& S, float3 ro, float3 rd, float begin, float end) {
    const float distance = fmaxf(end - begin, 0.0f);
    if (distance == 0.0f) return 0.0f;
    const float sigma = fog_sigma(S, ro + rd * begin);
    const float mid_height = ro.y + rd.y * ((begin + end) * 0.5f);
    if (mid_height <= S.fog[1] || S.fog[2] == 0.0f) return S.fog[0] * distance;
    const float k = rd.y * S.fog[2];
    const float x = k * distance;
    if (fabsf(x) < 0.001f) return sigma * distance * (1.0f - x * 0.5f + x * x / 6.0f);
    return fmaxf(0.0f, wdiv(sigma - fog_sigma(S, ro + rd * end), k));
}
__device__ __forceinline__ float fog_split(const DevScene& S, float3 ro, float3 rd, float distance) {
    if (fabsf(rd.y) < 1e-8f) return distance;
    return fminf(fmaxf(wdiv(S.fog[1] - ro.y, rd.y), 0.0f), distance);
}
static __device__ float fog_optical_depth(const DevScene& S, float3 ro, float3 rd, float distance) {
    const float split = fog_split(S, ro, rd, distance);
    return fog_segment_tau(S, ro, rd, 0.0f, split) + fog_segment_tau(S, ro, rd, split, distance);
}
__device__ __forceinline__ float fog_transmittance(const DevScene& S, float3 ro, float3 rd, float distance) {
    return expf(-fog_optical_depth(S, ro, rd, distance));
}
static __device__ float fog_invert_segment(const DevScene& S, float3 ro, float3 rd, float begin, float end, float tau) {
    const float sigma = fog_sigma(S, ro + rd * begin);
    const float k = rd.y * S.fog[2];
    if (ro.y + rd.y * ((begin + end) * 0.5f) <= S.fog[1] || fabsf(k * (end - begin)) < 0.0001f)
        return fminf(end, begin + wdiv(tau, fmaxf(sigma, 1e-30f)));
    if (sigma > 1e-20f)
        return fminf(fmaxf(begin - wdiv(logf(fmaxf(1e-7f, 1.0f - wdiv(tau * k, sigma))), k), begin), end);
    const float remaining = fmaxf(0.0f, fog_segment_tau(S, ro, rd, begin, end) - tau);
    const float end_sigma = fog_sigma(S, ro + rd * end);
    return fminf(fmaxf(end + wdiv(logf(fmaxf(1e-7f, 1.0f + wdiv(remaining * k, fmaxf(end_sigma, 1e-30f)))), -k), begin),
                 end);
}
static __device__ float fog_free_flight(const DevScene& S, float3 ro, float3 rd, float t_end, uint32_t& rng) {
    if (S.fog[0] <= 0.0f) return t_end;
    const float tau = -logf(fmaxf(1.0f - rnd(rng), 1e-7f));
    const float split = fog_split(S, ro, rd, t_end);
    const float first = fog_segment_tau(S, ro, rd, 0.0f, split);
    const float total = first + fog_segment_tau(S, ro, rd, split, t_end);
    if (tau >= total) return t_end;
    if (tau < first) return fog_invert_segment(S, ro, rd, 0.0f, split, tau);
    return fog_invert_segment(S, ro, rd, split, t_end, tau - first);
}
// hg_phase, hg_sample (pathtrace.wgsl:717-731).
__device__ __forceinline__ float hg_phase(float cos_theta, float g) {
    const float d = 1.0f + g * g - 2.0f * g * cos_theta;
    return wdiv(1.0f - g * g, 4.0f * SF_PI * d * wsqrt(d));
}
__device__ __forceinline__ float3 hg_sample(float3 dir, float g, float r1, float r2) {
    float cos_t = 1.0f - 2.0f * r1;
    if (fabsf(g) > 1e-3f) {
        const float sq = wdiv(1.0f - g * g, 1.0f - g + 2.0f * g * r1);
        cos_t = wdiv(1.0f + g * g - sq * sq, 2.0f * g);
    }
    const float sin_t = wsqrt(fmaxf(0.0f, 1.0f - cos_t * cos_t));
    float sp, cp;
    sincosf(2.0f * SF_PI * r2, &sp, &cp);
    float3 t, bt;
    tangent_frame(dir, t, bt);
    return frame_mul(t, bt, dir, mk3(sin_t * cp, sin_t * sp, cos_t));
}
// volume_coordinate (pathtrace.wgsl:43-58): the radical inverse of the sample index
// in the dimension's prime base, rotated per pixel and emitter.
__device__ __forceinline__ float volume_coordinate(uint32_t sample_index, uint32_t dimension, uint32_t stream) {
    const uint32_t base = dimension == 0 ? 2u : dimension == 1 ? 3u : dimension == 2 ? 5u
                        : dimension == 3 ? 7u : dimension == 4 ? 11u : 13u;
    uint32_t index = sample_index + 1u;
    float inverse = 1.0f / float(base);
    float value = 0.0f;
    while (index != 0u) {
        value = __fadd_rn(value, __fmul_rn(float(index % base), inverse));
        index /= base;
        inverse = inverse / float(base);
    }
    const float shift = float(pcg(stream ^ (dimension * 0x9e3779b9u)) >> 8u) / 16777216.0f;
    const float v = value + shift;
    return v - floorf(v);
}
// fog_segment_weight (pathtrace.wgsl:621-633): max-channel power over the distance
// from the segment's closest point to the emitter's centre (a tube's midpoint), on the
// part of the segment inside a projector's bounding cone.
static __device__ float fog_segment_weight(float3 ro, float3 rd, float end, const DevLight& l) {
    const float3 center = l.kind == SF_LIGHT_TUBE ? (ld3(l.a) + ld3(l.b)) * 0.5f : ld3(l.a);
    float2 interval = make_float2(0.0f, end);
    if (l.projector) {
        interval = cone_segment(ro, rd, end, projector_bound_apex(l), ld3(l.n), l.beam[1]);
        if (interval.y <= interval.x) return 0.0f;
    }
    const float along = fminf(fmaxf(dot3(center - ro, rd), interval.x), interval.y);
    const float3 delta = center - (ro + rd * along);
    return wdiv(fmaxf(fmaxf(l.color[0], l.color[1]), l.color[2]) * l.area, dot3(delta, delta) + l.area);
}
// volume_light_probability (lights.wgsl:319-323): independent per-emitter roulette.
__device__ __forceinline__ float volume_light_probability(float weight, float total) {
    if (total <= 0.0f) return 0.0f;
    return fminf(1.0f, wdiv(3.0f * weight, total));
}
// fog_segment_direct (pathtrace.wgsl:635-715): in-scattered emitter light along the
// segment [0, end] of the current ray as a line integral. Each area light passes an
// independent roulette; the point on the segment mixes equiangular sampling about a
// sampled emitter point with the truncated optical-depth distribution (one-sample
// MIS, balance weights). Primary segments use the rotated radical-inverse points.
// Each sample is one shadow segment, handed to `emit` with radiance `tp` × (its
// estimate) × colour.
template <class Emit>
static __device__ void fog_segment_direct(const DevScene& S, float3 tp, float3 ro, float3 rd, float end, uint32_t& rng,
                                          uint32_t point_index, uint32_t point_stream, bool primary, Emit&& emit) {
    const float3 color = ld3(S.fog_color);
    if (end <= 0.0f || fmaxf(fmaxf(color.x, color.y), color.z) <= 0.0f) return;
    const float tau_end = fog_optical_depth(S, ro, rd, end);
    if (tau_end <= 0.0f) return;
    float total = 0.0f;
    for (uint32_t i = 0; i < S.light_count; ++i)
        if (is_emitter(light_of(S, i))) total += fog_segment_weight(ro, rd, end, light_of(S, i));
    const float g = S.fog[3];
    for (uint32_t i = 0; i < S.light_count; ++i) {
        const DevLight& l = light_of(S, i);
        if (!is_emitter(l)) continue;
        const float probability = volume_light_probability(fog_segment_weight(ro, rd, end, l), total);
        const uint32_t stream = pcg(point_stream ^ (i * 0x85ebca6bu));
        float selection = rnd(rng);
        if (primary) selection = volume_coordinate(point_index, 5u, stream);
        if (probability <= 0.0f || selection >= probability) continue;
        // sample_emitter draws two numbers for a rectangle, three for a tube
        float u1 = rnd(rng);
        float u2 = rnd(rng);
        float u3 = l.kind == SF_LIGHT_TUBE ? rnd(rng) : 0.0f;
        if (primary) {
            u1 = volume_coordinate(point_index, 0u, stream);
            u2 = volume_coordinate(point_index, 1u, stream);
            u3 = volume_coordinate(point_index, 2u, stream);
        }
        const EmitterPoint emitter = sample_emitter_point(l, u1, u2, u3);
        const float3 q = emitter.position;
        float2 interval = make_float2(0.0f, end);
        if (l.projector) {
            interval = cone_segment(ro, rd, end, q, ld3(l.n), l.beam[1]);
            if (interval.y <= interval.x) continue;
        }
        const float tau_begin = fog_optical_depth(S, ro, rd, interval.x);
        const float tau_finish = fog_optical_depth(S, ro, rd, interval.y);
        const float tau_span = fmaxf(0.0f, tau_finish - tau_begin);
        if (tau_span <= 0.0f) continue;
        float conditional_mass = 1.0f - expf(-tau_span);
        if (tau_span < 0.001f) conditional_mass = tau_span * (1.0f - tau_span * 0.5f + tau_span * tau_span / 6.0f);
        const float interval_mass = expf(-tau_begin) * conditional_mass;
        if (interval_mass < 1e-30f) continue;
        const float3 delta = q - ro;
        const float projection = dot3(delta, rd);
        const float3 perp_v = delta - rd * projection;
        const float perpendicular = wsqrt(dot3(perp_v, perp_v));
        const float theta_a = atan2f(interval.x - projection, fmaxf(perpendicular, 1e-6f));
        const float theta_b = atan2f(interval.y - projection, fmaxf(perpendicular, 1e-6f));
        const float span = theta_b - theta_a;
        const bool regular = perpendicular > 1e-4f && span > 1e-5f;
        float xi = rnd(rng);
        float technique = rnd(rng);
        if (primary) {
            xi = volume_coordinate(point_index, 3u, stream);
            technique = volume_coordinate(point_index, 4u, stream);
        }
        float t = mixf(interval.x, interval.y, xi);
        if (technique < 0.5f) {
            if (regular)
                t = fminf(fmaxf(projection + perpendicular * tanf(mixf(theta_a, theta_b, xi)), interval.x), interval.y);
        } else {
            const float tau = tau_begin - logf(fmaxf(1.0f - xi * conditional_mass, 1e-7f));
            const float split = fog_split(S, ro, rd, interval.y);
            const float first = fog_segment_tau(S, ro, rd, 0.0f, split);
            t = tau < first ? fog_invert_segment(S, ro, rd, 0.0f, split, tau)
                            : fog_invert_segment(S, ro, rd, split, interval.y, tau - first);
        }
        const float3 p = ro + rd * t;
        const float transmittance = expf(-fog_optical_depth(S, ro, rd, t));
        const float sigma = fog_sigma(S, p);
        float angular_pdf = wdiv(1.0f, interval.y - interval.x);
        if (regular) {
            const float dt = t - projection;
            angular_pdf = wdiv(perpendicular, span * (perpendicular * perpendicular + dt * dt));
        }
        const float distance_pdf = 0.5f * (angular_pdf + wdiv(sigma * transmittance, interval_mass));
        const float3 to_light = q - p;
        const float distance2 = dot3(to_light, to_light);
        if (distance2 < 1e-8f) continue;
        const float distance = wsqrt(distance2);
        const float3 wi = to_light * wdiv(1.0f, distance);
        const float cosine = dot3(emitter.normal, -wi);
        if (cosine <= 0.0f) continue;
        const float tr = transmittance * expf(-fog_optical_depth(S, p, wi, distance));
        const float light_pdf = wdiv(distance2, fmaxf(l.area * cosine, 1e-20f));
        const float scale = wdiv(sigma * tr * hg_phase(dot3(rd, wi), g), probability * distance_pdf * light_pdf);
        ShadowReq sh;
        sh.o = p;
        sh.dir = wi;
        sh.t_end = fmaxf(0.0f, distance - fmaxf(1e-5f, distance * 1e-6f));
        sh.contrib = tp * ((emitter_radiance(l, -wi) * scale) * color);
        sh.volume = primary;  // pathtrace.wgsl:985: bounce 0's direct volume
        emit(sh);
    }
}
// fog_direct_light (pathtrace.wgsl:733-772): next events at a scattering point for
// the sky lights (environment: uniform sphere with its roulette; panoramas; suns),
// phase function in place of the BRDF; `tpc` = throughput × fog colour.
template <class Emit>
static __device__ void fog_direct_light(const DevScene& S, float3 tpc, float3 p, float3 rd, float area_total, bool last,
                                        uint32_t& rng, Emit&& emit) {
    const float g = S.fog[3];
    for (uint32_t i = 0; i < S.light_count; ++i) {
        const DevLight& l = light_of(S, i);
        float3 dir, value;
        float pl;
        if (l.kind == SF_LIGHT_ENVIRONMENT) {
            if (l.peak <= 0.0f) continue;
            const float probability = environment_probability(l, area_total);
            if (rnd(rng) >= probability) continue;
            const float z = 1.0f - 2.0f * rnd(rng);
            const float phi = 2.0f * SF_PI * rnd(rng);
            const float radius = wsqrt(fmaxf(0.0f, 1.0f - z * z));
            float sp, cp;
            sincosf(phi, &sp, &cp);
            dir = mk3(radius * cp, z, radius * sp);
            pl = probability * (1.0f / (4.0f * SF_PI));
            value = environment_value(l, dir);
        } else if (l.kind == SF_LIGHT_HDRI) {
            if (l.color[0] <= 0.0f) continue;
            const float r0 = rnd(rng);
            const float r1 = rnd(rng);
            const float r2 = rnd(rng);
            dir = hdri_sample(l, r0, r1, r2);
            pl = hdri_pdf(l, dir);
            value = hdri_lookup(l, dir);
        } else if (l.kind == SF_LIGHT_SUN) {
            const float r1 = rnd(rng);
            const float r2 = rnd(rng);
            dir = cone_sample(ld3(l.a), l.cos_max, r1, r2);
            pl = sun_pdf(l.cos_max);
            value = ld3(l.color);
        } else {
            continue;
        }
        const float tr = fog_transmittance(S, p, dir, S.extent);
        const float ph = hg_phase(dot3(rd, dir), g);
        const float w = last ? 1.0f : mis_power(pl, ph);
        ShadowReq sh;
        sh.o = p;
        sh.dir = dir;
        sh.t_end = S.extent;
        // the sun's colour is its irradiance: no division by the disk's pdf
        sh.contrib = tpc * (l.kind == SF_LIGHT_SUN ? value * ph * tr * w : value * ph * tr * wdiv(w, pl));
        emit(sh);
    }
}

// One bounce of `radiance` (pathtrace.wgsl:841-1196) after its trace: hit
// classification, sky and emitter emission with MIS, surface, next-event sampling
// (direct_light, pathtrace.wgsl:471-558: every environment and sun, and the one
// selected area light, in scene order; each visibility test is handed to `emit`,
// which adds its radiance if the segment is clear) and BSDF continuation with
// Russian roulette. Writes first-hit depth/aux at bounce 0. In fog (pathtrace.wgsl:
// 980-1011) the segment first adds its in-scattered emitter light, then a collision
// drawn along it may scatter the path (next events for the sky lights, phase-sampled
// continuation) before the hit is reached. `point_index` is the sample index and
// `point_stream` the pixel's rotation (point_stream_of) of the primary segment's points.
// optical_bounce (optics.wgsl:30-64) without dispersion or thin-film coating: the
// dielectric's VNDF reflection or transmission (a thin sheet passes straight through
// with its absorption tint), drawn as its own mixture component.
struct OpticalBounce {
    float3 direction, weight;
    bool transmitted, valid;
};
static __device__ OpticalBounce optical_bounce(const DevOptics& o, float3 n, float3 rd, float alpha, bool entering,
                                               uint32_t& rng) {
    OpticalBounce b;
    const float index = o.surface[2];
    const bool thin = o.surface[3] > 0.0f;
    const float3 tint = exp3(mk3(-o.absorption[0] * o.absorption[3], -o.absorption[1] * o.absorption[3],
                                 -o.absorption[2] * o.absorption[3]));
    if (index <= 1.0001f) {
        b.direction = rd;
        b.weight = thin ? tint : mk3(1.f, 1.f, 1.f);
        b.transmitted = true;
        b.valid = true;
        return b;
    }
    const float eta = (entering || thin) ? wdiv(1.0f, index) : index;
    const float r1 = rnd(rng);
    const float r2 = rnd(rng);
    const float3 h = sample_ggx_h(n, -rd, alpha, r1, r2);
    float f = dielectric_fresnel(fmaxf(0.0f, dot3(-rd, h)), eta);
    if (thin) f = wdiv(2.0f * f, 1.0f + f);
    float3 color = mk3(f, f, f);
    float probability = f;
    const float3 transmitted = refract3(rd, h, eta);
    if (!thin && dot3(transmitted, transmitted) < 0.5f) {  // total internal reflection
        color = mk3(1.f, 1.f, 1.f);
        probability = 1.0f;
    }
    const float a2 = alpha * alpha;
    if (rnd(rng) < probability) {
        b.direction = reflect3(rd, h);
        const float cosine = dot3(n, b.direction);
        b.weight = color * wdiv(smith_g1(fmaxf(cosine, 1e-6f), a2), fmaxf(probability, 1e-20f));
        b.transmitted = false;
        b.valid = cosine > 0.0f;
        return b;
    }
    b.direction = thin ? rd : transmitted;
    const float cosine = -dot3(n, b.direction);
    const float3 w = thin ? tint : mk3(1.f, 1.f, 1.f) * (smith_g1(fmaxf(cosine, 1e-6f), a2) * eta * eta);
    b.weight = w * (mk3(1.f, 1.f, 1.f) - color) * wdiv(1.0f, fmaxf(1.0f - probability, 1e-20f));
    b.transmitted = true;
    b.valid = cosine > 0.0f && dot3(b.direction, b.direction) > 0.5f;
    return b;
}

// One bounce of `radiance` (pathtrace.wgsl:841-1196) after its trace: the interior
// medium of a dielectric (absorption, subsurface scattering), hit classification, sky
// and emitter emission with MIS, the optics of the hit (coverage null events, the
// dielectric lobe), surface, next-event sampling (direct_light, pathtrace.wgsl:471-558:
// every environment and sun, and the one selected area light, in scene order; each
// visibility test is handed to `emit`, which adds its radiance if the segment is
// clear) and BSDF continuation with Russian roulette. Writes first-hit depth/aux at
// bounce 0. In fog (pathtrace.wgsl:980-1011) the segment first adds its in-scattered
// emitter light, then a collision drawn along it may scatter the path (next events
// for the sky lights, phase-sampled continuation) before the hit is reached.
// `point_index` is the sample index and `point_stream` the pixel's rotation
// (point_stream_of) of the primary segment's points. A surface hit on a material with
// optics carries the refined hit and the normal of optical_refine_hit (optics.wgsl:
// 7-23) and normal_at(p, 1e-4), made by the trace. FEAT: as make_surface's (the
// optics and the footprint transport need SF_FEAT_RICH).
template <int FEAT = 0, class Emit>
static __device__ int bounce_body(const DevScene& S, PathState& ps, const HitInfo& h, Emit&& emit, float* first_depth,
                                  float4* first_aux, uint32_t point_index, uint32_t point_stream) {
    constexpr bool RICH = (FEAT & SF_FEAT_RICH) != 0;
    const bool optics = RICH && (S.rich & SF_RICH_OPTICS) != 0u;
    if (optics && ps.solid_medium) {  // inside a dielectric solid (pathtrace.wgsl:857-875)
        const DevOptics& medium = material_optics(S, ps.medium_slot);
        float distance = h.t;
        if (medium.subsurface[3] > 0.0f)
            distance = fminf(h.t, wdiv(-logf(fmaxf(1e-7f, 1.0f - rnd(ps.rng))), medium.subsurface[3]));
        ps.tp = ps.tp * exp3(mk3(-medium.absorption[0] * distance, -medium.absorption[1] * distance,
                                 -medium.absorption[2] * distance));
        if (distance < h.t) {
            if (ps.bounce == S.max_bounces) return PATH_DONE;
            ps.tp = ps.tp * ld3(medium.subsurface);
            const float r1 = rnd(ps.rng);
            const float r2 = rnd(ps.rng);
            ps.o = ps.o + ps.d * distance;
            ps.d = hg_sample(ps.d, 0.0f, r1, r2);
            // no MIS after a subsurface collision: emitters reached next count in full
            ps.prev_from_bsdf = false;
            ps.prev_from_volume = false;
            ps.prev_pdf = 0.0f;
            ps.tex_spread = fmaxf(ps.tex_spread, 0.25f);
            ps.bounce += 1;
            return PATH_CONTINUE;
        }
    }
    if (h.hit && ps.bounce == 0 && first_depth) {
        *first_depth = h.t;
        const float3 en = h.light_index != SF_NO_LIGHT
                              ? emitter_normal(light_of(S, h.light_index), e_add(ps.o, e_mul(ps.d, h.t)))
                              : h.n;
        *first_aux = make_float4(en.x, en.y, en.z, float(h.steps));
    }
    const bool fog = S.fog[0] > 0.0f && !(RICH && ps.solid_medium);
    if (fog) {
        const float t_end = h.hit ? h.t : S.extent;
        fog_segment_direct(S, ps.tp, ps.o, ps.d, t_end, ps.rng, point_index, point_stream,
                           ps.bounce == 0 && (!RICH || ps.null_surfaces == 0), emit);
        const float t_s = fog_free_flight(S, ps.o, ps.d, t_end, ps.rng);
        if (t_s < t_end) {
            if (ps.bounce == 0) ps.volume_path = true;
            if (RICH) {
                ps.tex_width += t_s * ps.tex_spread;
                ps.tex_spread = fmaxf(ps.tex_spread, 0.25f);
            }
            if (ps.bounce == 0 && !h.hit && first_depth) *first_depth = t_s;
            const float3 p_s = ps.o + ps.d * t_s;
            const float volume_area_total = area_total_weight(S, p_s, mk3(0.f, 0.f, 0.f));
            const bool last = ps.bounce == S.max_bounces;
            const float3 tpc = ps.tp * ld3(S.fog_color);
            fog_direct_light(S, tpc, p_s, ps.d, volume_area_total, last, ps.rng, emit);
            ps.tp = tpc;
            if (last) return PATH_DONE;
            const float r1 = rnd(ps.rng);
            const float r2 = rnd(ps.rng);
            const float3 nd = hg_sample(ps.d, S.fog[3], r1, r2);
            ps.prev_pdf = hg_phase(dot3(ps.d, nd), S.fog[3]);
            ps.prev_from_bsdf = true;
            ps.prev_from_volume = true;
            ps.prev_normal = mk3(0.f, 0.f, 0.f);
            ps.prev_area_total = volume_area_total;
            ps.o = p_s;
            ps.d = nd;
            ps.bounce += 1;
            return PATH_CONTINUE;
        }
    }
    if (!h.hit) {
        if (!h.exhausted) {  // the sky, the panoramas, the suns (pathtrace.wgsl:1026-1040)
            ps.L = ps.L + ps.tp * environment_emission(S, ps.d, ps.prev_pdf, ps.prev_from_bsdf, ps.prev_normal,
                                                       ps.prev_from_volume, ps.prev_area_total);
            ps.L = ps.L + ps.tp * hdri_emission(S, ps.d, ps.prev_pdf, ps.prev_from_bsdf);
            ps.L = ps.L + ps.tp * sun_radiance(S, ps.d, ps.prev_pdf, ps.prev_from_bsdf);
        }
        return PATH_DONE;
    }
    float3 p = ps.o + ps.d * h.t;
    if (h.light_index != SF_NO_LIGHT) {
        // after a fog scattering point its segment estimate already holds the emitters
        if (!ps.prev_from_volume)
            ps.L = ps.L + ps.tp * area_emission(S, ps.o, ps.d, h.t, ps.prev_pdf, ps.prev_from_bsdf, ps.prev_normal,
                                                ps.prev_area_total);
        return PATH_DONE;
    }
    float3 n = h.n;
    bool optical = false, entering = true;
    if (optics) {  // pathtrace.wgsl:1053-1066
        const DevOptics& o = material_optics(S, h.sample.material);
        optical = optics_enabled(o);
        entering = dot3(ps.d, h.n) < 0.0f;
        if (optical && !entering) n = -n;
        if (optical && o.surface[0] < 1.0f && rnd(ps.rng) >= o.surface[0]) {
            // a coverage null event: the path passes the surface within the same bounce
            ps.null_surfaces += 1;
            if (ps.null_surfaces > 32u) return PATH_DONE;
            ps.o = p + ps.d * fmaxf(h.t * S.pixel_cone * 0.15f * S.pixel_tolerance, 1e-4f);
            if (ps.bounce == 0 && first_depth) {
                *first_depth = -1.0f;
                *first_aux = make_float4(0.f, 0.f, 0.f, -1.0f);
            }
            return PATH_CONTINUE;
        }
        if (optical && ps.bounce == 0 && first_depth) *first_aux = make_float4(n.x, n.y, n.z, float(h.steps));
    }
    if (ps.bounce == 0) {
        float x = fminf(fmaxf(float(h.steps) / 96.0f, 0.0f), 1.0f);
        ps.tp = ps.tp * (1.0f - S.cavity * (x * x * (3.0f - 2.0f * x)));
    }
    float3 v = -ps.d;
    if (RICH) ps.tex_width += h.t * ps.tex_spread;
    Surface s = make_surface<FEAT>(S, p, n, v, h.sample, fmaxf(ps.tex_width, 1e-4f));
    ps.L = ps.L + ps.tp * s.emission;
    float offset = fmaxf(h.t * S.pixel_cone * 2.0f, 1e-3f) * S.pixel_tolerance;
    if (optical) {
        const DevOptics& o = material_optics(S, h.sample.material);
        if (o.surface[1] > 0.0f && rnd(ps.rng) < o.surface[1]) {  // the dielectric lobe (:1088-1107)
            if (ps.bounce == S.max_bounces) return PATH_DONE;
            const OpticalBounce b = optical_bounce(o, n, ps.d, s.alpha, entering, ps.rng);
            if (!b.valid) return PATH_DONE;
            ps.tp = ps.tp * b.weight;
            const float bias = fmaxf(1e-4f, fminf(offset, 0.001f));
            ps.o = p + b.direction * bias;
            ps.d = b.direction;
            if (b.transmitted && o.surface[3] == 0.0f) {
                ps.solid_medium = entering;
                ps.medium_slot = h.sample.material;
            }
            ps.prev_from_bsdf = false;
            ps.prev_from_volume = false;
            ps.prev_pdf = 0.0f;
            ps.tex_spread = fmaxf(ps.tex_spread, s.alpha * 0.1f);
            ps.bounce += 1;
            return PATH_CONTINUE;
        }
    }
    float3 p_off = p + n * offset;
    float nv = fmaxf(dot3(s.n, v), 1e-4f);
    float p_spec = spec_probability(s, nv);
    float area_total = area_total_weight(S, p_off, s.n);
    bool last = ps.bounce == S.max_bounces;
    // direct_light: the area light selected by weight, then every light in order
    uint32_t selected = SF_NO_LIGHT;
    float selected_weight = 0.0f;
    if (area_total > 0.0f) {
        float threshold = rnd(ps.rng) * area_total;
        float sum = 0.0f;
        for (uint32_t i = 0; i < S.light_count; ++i) {
            if (!is_emitter(light_of(S, i))) continue;
            float w = area_weight(p_off, s.n, light_of(S, i));
            sum += w;
            if (w > 0.0f) {
                selected = i;
                selected_weight = w;
                if (threshold < sum) break;
            }
        }
    }
    for (uint32_t i = 0; i < S.light_count; ++i) {
        const DevLight& l = light_of(S, i);
        if (l.kind == SF_LIGHT_ENVIRONMENT) {
            if (l.peak <= 0.0f) continue;
            const float probability = environment_probability(l, area_total);
            if (rnd(ps.rng) >= probability) continue;
            const float r1 = rnd(ps.rng);
            const float r2 = rnd(ps.rng);
            const float3 ldir = cosine_sample(s.n, r1, r2);
            const float nl = fmaxf(dot3(s.n, ldir), 0.0f);
            if (dot3(n, ldir) <= 0.0f || nl <= 0.0f) continue;
            const float pl = probability * nl * (1.0f / SF_PI);
            const float pb = last ? 0.0f : bsdf_pdf(s, v, ldir, p_spec);
            const float w = last ? 1.0f : mis_power(pl, pb);
            ShadowReq sh;
            sh.o = p_off;
            sh.dir = ldir;
            sh.t_end = S.extent;
            const float tr = fog ? fog_transmittance(S, p_off, ldir, S.extent) : 1.0f;
            sh.contrib = ps.tp * (brdf_eval(s, v, ldir) * nl * environment_value(l, ldir) * tr * wdiv(w, pl));
            emit(sh);
        } else if (l.kind == SF_LIGHT_HDRI) {
            if (l.color[0] <= 0.0f) continue;
            const float r0 = rnd(ps.rng);
            const float r1 = rnd(ps.rng);
            const float r2 = rnd(ps.rng);
            const float3 ldir = hdri_sample(l, r0, r1, r2);
            const float nl = dot3(s.n, ldir);
            if (nl <= 0.0f || dot3(n, ldir) <= 0.0f) continue;
            const float pl = hdri_pdf(l, ldir);
            const float pb = last ? 0.0f : bsdf_pdf(s, v, ldir, p_spec);
            const float w = last ? 1.0f : mis_power(pl, pb);
            ShadowReq sh;
            sh.o = p_off;
            sh.dir = ldir;
            sh.t_end = S.extent;
            const float tr = fog ? fog_transmittance(S, p_off, ldir, S.extent) : 1.0f;
            sh.contrib = ps.tp * (brdf_eval(s, v, ldir) * nl * hdri_lookup(l, ldir) * tr * wdiv(w, pl));
            emit(sh);
        } else if (l.kind == SF_LIGHT_SUN) {
            const float r1 = rnd(ps.rng);
            const float r2 = rnd(ps.rng);
            const float3 ldir = cone_sample(ld3(l.a), l.cos_max, r1, r2);
            const float nl = dot3(s.n, ldir);
            if (nl <= 0.0f || dot3(n, ldir) <= 0.0f) continue;
            const float pl = sun_pdf(l.cos_max);
            const float pb = last ? 0.0f : bsdf_pdf(s, v, ldir, p_spec);
            const float w = last ? 1.0f : mis_power(pl, pb);
            ShadowReq sh;
            sh.o = p_off;
            sh.dir = ldir;
            sh.t_end = S.extent;
            const float tr = fog ? fog_transmittance(S, p_off, ldir, S.extent) : 1.0f;
            sh.contrib = ps.tp * (brdf_eval(s, v, ldir) * nl * ld3(l.color) * w * tr);
            emit(sh);
        } else if (i == selected) {
            // sample_emitter: two numbers for a rectangle, three for a tube
            float u1 = rnd(ps.rng);
            float u2 = rnd(ps.rng);
            float u3 = l.kind == SF_LIGHT_TUBE ? rnd(ps.rng) : 0.0f;
            const EmitterPoint emitter = sample_emitter_point(l, u1, u2, u3);
            float3 q = emitter.position;
            float3 ln = emitter.normal;
            float3 to_q = q - p_off;
            float dist2 = dot3(to_q, to_q);
            if (dist2 < 1e-8f) continue;
            const float inv_dist = rsqrtf(dist2);
            float dist = dist2 * inv_dist;
            float3 ldir = to_q * inv_dist;
            float nl = dot3(s.n, ldir);
            float cos_l = dot3(ln, -ldir);
            if (nl <= 0.0f || cos_l <= 0.0f || dot3(n, ldir) <= 0.0f) continue;
            float pl = wdiv(selected_weight, area_total) * wdiv(dist2, fmaxf(l.area * cos_l, 1e-20f));
            float pb = last ? 0.0f : bsdf_pdf(s, v, ldir, p_spec);
            float w = last ? 1.0f : mis_power(pl, pb);
            const float tr = fog ? fog_transmittance(S, p_off, ldir, dist) : 1.0f;
            float3 Ld = brdf_eval(s, v, ldir) * nl * emitter_radiance(l, -ldir) * tr * wdiv(w, pl);
            ShadowReq sh;
            sh.o = p_off;
            sh.dir = ldir;
            sh.t_end = fmaxf(0.0f, dist - fmaxf(1e-5f, dist * 1e-6f));
            sh.contrib = ps.tp * Ld;
            emit(sh);
        }
    }
    if (last) return PATH_DONE;
    float r0 = rnd(ps.rng), r1 = rnd(ps.rng), r2 = rnd(ps.rng);
    float3 ldir;
    if (r0 < p_spec) {
        float3 hh = sample_ggx_h(s.n, v, s.alpha, r1, r2);
        float3 i = -v;
        ldir = i - hh * (2.0f * dot3(hh, i));
    } else {
        ldir = cosine_sample(s.n, r1, r2);
    }
    float nl = dot3(s.n, ldir);
    if (nl <= 0.0f || dot3(n, ldir) <= 0.0f) return PATH_DONE;
    float pdf = bsdf_pdf(s, v, ldir, p_spec);
    if (pdf <= 1e-6f) return PATH_DONE;
    ps.tp = ps.tp * (brdf_eval(s, v, ldir) * wdiv(nl, pdf));
    ps.prev_pdf = pdf;
    ps.prev_from_bsdf = true;
    ps.prev_from_volume = false;
    ps.prev_normal = s.n;
    ps.prev_area_total = area_total;
    if (ps.bounce >= 2) {
        float q = fminf(fmaxf(fmaxf(ps.tp.x, fmaxf(ps.tp.y, ps.tp.z)), 0.05f), 0.95f);
        if (rnd(ps.rng) > q) return PATH_DONE;
        ps.tp = ps.tp * wdiv(1.0f, q);
    }
    ps.o = p_off;
    ps.d = ldir;
    if (RICH) ps.tex_spread = fmaxf(ps.tex_spread, s.alpha * 0.25f);
    ps.bounce += 1;
    return PATH_CONTINUE;
}

// Tetrahedral stencil (common.wgsl:376-387).
__device__ __forceinline__ float3 tetra_offset(uint32_t i) {
    return i == 0 ? mk3(1.f, -1.f, -1.f) : (i == 1 ? mk3(-1.f, -1.f, 1.f) : (i == 2 ? mk3(-1.f, 1.f, -1.f) : mk3(1.f, 1.f, 1.f)));
}

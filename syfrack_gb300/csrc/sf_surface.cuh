// Surface detail of make_surface on sm_103a: the world-space finish patterns of
// finish_detail.wgsl (:1-160), the ramps (palette_sample) and the volumetric fractal
// texture (texture.wgsl, pattern.wgsl). A finish pattern returns its analytic
// gradient (xyz) and height (w) from one evaluation; patterns and textures are
// filtered by the pixel footprint the path transports (pathtrace.wgsl:811-814, :1075).
#pragma once
#include "sf_de.cuh"
#include "sf_program.h"

#define SF_PI 3.14159265358979f  // common.wgsl:6

// WGSL's scalar helpers: smoothstep, fract, mix (x*(1-t) + y*t).
__device__ __forceinline__ float sstep(float e0, float e1, float x) {
    const float t = fminf(fmaxf((x - e0) / (e1 - e0), 0.0f), 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
__device__ __forceinline__ float fractf(float x) { return x - floorf(x); }
__device__ __forceinline__ float mixf(float x, float y, float t) { return fmaf(x, 1.0f - t, y * t); }
__device__ __forceinline__ float4 mix4(float4 x, float4 y, float t) {
    return make_float4(mixf(x.x, y.x, t), mixf(x.y, y.y, t), mixf(x.z, y.z, t), mixf(x.w, y.w, t));
}
__device__ __forceinline__ float4 f4(float3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
__device__ __forceinline__ float3 xyz(float4 v) { return mk3(v.x, v.y, v.z); }
__device__ __forceinline__ float4 scale4(float4 v, float s) { return make_float4(v.x * s, v.y * s, v.z * s, v.w * s); }
__device__ __forceinline__ float4 add4(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float signf(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
// modf_euclid (common.wgsl:255-257): x - m * floor(x / m).
__device__ __forceinline__ float modf_euclid(float x, float m) { return x - m * floorf(x / m); }

__device__ __forceinline__ uint32_t pcg_hash(uint32_t v) {
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
// finish_hash (finish_detail.wgsl:3-7): the lattice cell's bits hashed with the seed.
__device__ __forceinline__ float finish_hash(int cx, int cy, int cz, uint32_t seed) {
    const uint32_t h = pcg_hash(uint32_t(cx) ^ pcg_hash(uint32_t(cy) + 0x9e3779b9u) ^ pcg_hash(uint32_t(cz) + seed));
    return float(h >> 8u) * (1.0f / 16777216.0f);
}
// finish_noise (:8-21): trilinear value noise with the smoothstep fade and its
// analytic gradient.
static __device__ float4 finish_noise(float3 p, uint32_t seed) {
    const float3 fl = mk3(floorf(p.x), floorf(p.y), floorf(p.z));
    const int x = __float2int_rz(fl.x), y = __float2int_rz(fl.y), z = __float2int_rz(fl.z);
    const float3 f = p - fl;
    const float3 t = f * f * (mk3(3.f, 3.f, 3.f) - f * 2.0f);
    const float3 dt = f * (mk3(1.f, 1.f, 1.f) - f) * 6.0f;
    const float a0 = finish_hash(x, y, z, seed), a1 = finish_hash(x + 1, y, z, seed);
    const float b0 = finish_hash(x, y + 1, z, seed), b1 = finish_hash(x + 1, y + 1, z, seed);
    const float c0 = finish_hash(x, y, z + 1, seed), c1 = finish_hash(x + 1, y, z + 1, seed);
    const float d0 = finish_hash(x, y + 1, z + 1, seed), d1 = finish_hash(x + 1, y + 1, z + 1, seed);
    const float a = mixf(a0, a1, t.x), b = mixf(b0, b1, t.x);
    const float c = mixf(c0, c1, t.x), d = mixf(d0, d1, t.x);
    const float e = mixf(a, b, t.y), g = mixf(c, d, t.y);
    const float dx = mixf(mixf(a1 - a0, b1 - b0, t.y), mixf(c1 - c0, d1 - d0, t.y), t.z);
    return make_float4(dx * dt.x, mixf(b - a, d - c, t.z) * dt.y, (g - e) * dt.z, mixf(e, g, t.z));
}
// finish_fbm (:22-33): three octaves, each faded out where the footprint exceeds its period.
static __device__ float4 finish_fbm(float3 p, float width, uint32_t seed) {
    float frequency = 1.0f, weight = 0.5f;
    float4 result = make_float4(0.f, 0.f, 0.f, 0.f);
    for (uint32_t i = 0; i < 3u; ++i) {
        const float visible = 1.0f - sstep(0.35f, 0.85f, width * frequency);
        if (visible > 0.0f) {
            const float4 n = finish_noise(p * frequency, seed + i * 97u);
            result = add4(result, scale4(f4(xyz(n) * (frequency * visible), mixf(0.5f, n.w, visible)), weight));
        } else {
            result.w += weight * 0.5f;
        }
        frequency *= 2.13f;
        weight *= 0.5f;
    }
    return scale4(result, 1.0f / 0.875f);
}
__device__ __forceinline__ float finish_smooth_derivative(float a, float b, float x) {
    const float t = fminf(fmaxf((x - a) / (b - a), 0.0f), 1.0f);
    return 6.0f * t * (1.0f - t) / (b - a);
}
__device__ __forceinline__ float2 rot2(float2 v, float a) {
    float s, c;
    sincosf(a, &s, &c);
    return make_float2(c * v.x - s * v.y, s * v.x + c * v.y);
}

// finish_eval (:37-154): the pattern of finish `d` at p, footprint-filtered. Returns
// (gradient, height). `wind` is the dunes' wind direction in radians (Sand). The
// coastal rock's sea-level wet band needs an ocean, which this path does not have.
static __device__ float4 finish_eval(const DevDetail& d, float3 p, float footprint, float wind) {
    const float scale = d.mapping[0];
    const float3 q = p * scale;
    const float width = footprint * scale;
    const uint32_t seed = d.seed, kind = d.kind;
    if (kind == 12u) {  // WetConcrete: rain fills broad depressions
        const float4 basin = finish_fbm(q * mk3(0.31f, 0.31f, 0.22f), width * 0.31f, seed + 911u);
        const float wet = sstep(0.47f, 0.59f, basin.w);
        const float4 grit = finish_fbm(q * 16.0f, width * 16.0f, seed + 113u);
        const float visible = 1.0f - sstep(0.15f, 0.6f, width * 3.0f);
        const float phase = fmaf(q.z, 4.1f, q.x * 2.8f);
        const float3 ripple = mk3(2.8f, 0.0f, 4.1f) * (cosf(phase) * 0.018f * visible);
        const float3 g = xyz(grit) * 16.0f;
        return f4(mk3(mixf(g.x, ripple.x, wet), mixf(g.y, ripple.y, wet), mixf(g.z, ripple.z, wet)) * scale, wet);
    }
    if (kind == 10u || kind == 11u) {  // Concrete / WeatheredConcrete
        const float4 stains = finish_fbm(q * 0.14f, width * 0.14f, seed + 17u);
        const float4 aggregate = finish_fbm(q * 7.0f, width * 7.0f, seed + 113u);
        const float4 pore = finish_noise(q * 23.0f, seed + 307u);
        const float visible = 1.0f - sstep(0.25f, 0.75f, width * 23.0f);
        const float pit = 1.0f - sstep(0.24f, 0.43f, pore.w);
        const float3 pit_gradient = xyz(pore) * (-finish_smooth_derivative(0.24f, 0.43f, pore.w) * 23.0f * visible);
        const float phase = fractf(q.y / 1.25f + 0.5f) - 0.5f;
        const float board_visible = 1.0f - sstep(0.03f, 0.15f, width);
        const float joint = (1.0f - sstep(0.006f, 0.027f, fabsf(phase))) * board_visible;
        const float joint_gradient =
            -finish_smooth_derivative(0.006f, 0.027f, fabsf(phase)) * signf(phase) / 1.25f * board_visible;
        const float height = 0.18f * stains.w + 0.65f * aggregate.w - 0.14f * mixf(0.2f, pit, visible) - 0.09f * joint;
        const float3 gradient = (xyz(stains) * (0.18f * 0.14f) + xyz(aggregate) * (0.65f * 7.0f) -
                                 pit_gradient * 0.14f - mk3(0.0f, 0.09f * joint_gradient, 0.0f)) * scale;
        if (kind == 11u) {
            const float3 axes = mk3(1.9f, 0.055f, 1.9f);
            const float4 rain = finish_fbm(q * axes, width * 1.9f, seed + 601u);
            const float deposit = sstep(0.33f, 0.68f, rain.w);
            const float3 rain_gradient = xyz(rain) * axes * (scale * finish_smooth_derivative(0.33f, 0.68f, rain.w));
            return f4(gradient + rain_gradient * 0.12f, fminf(fmaxf(0.72f * deposit + 0.28f * stains.w, 0.0f), 1.0f));
        }
        return f4(gradient, fminf(fmaxf(height + 0.12f, 0.0f), 1.0f));
    }
    if (kind == 9u) {  // Dust: domain-warped deposits with an analytic Jacobian
        const float4 wa = finish_fbm(q * 0.17f, width * 0.17f, seed + 17u);
        const float4 wb = finish_fbm(q * 0.17f, width * 0.17f, seed + 53u);
        const float3 warped = q + mk3(wa.w - 0.5f, 0.0f, wb.w - 0.5f) * 2.8f;
        const float4 cloud = finish_fbm(warped * 0.16f, width * 0.48f, seed + 211u);
        const float3 axes = mk3(0.65f, 0.18f, 0.09f);
        const float4 streak = finish_fbm(warped * axes, width * 1.95f, seed + 397u);
        const float density = 0.78f * cloud.w + 0.22f * streak.w;
        const float3 g = xyz(cloud) * (0.78f * 0.16f) + axes * xyz(streak) * 0.22f;
        const float3 density_gradient = (g + (xyz(wa) * g.x + xyz(wb) * g.z) * (2.8f * 0.17f)) * scale;
        const float deposit = sstep(0.36f, 0.64f, density);
        const float3 deposit_gradient = density_gradient * finish_smooth_derivative(0.36f, 0.64f, density);
        const float4 grain = finish_fbm(p * 48.0f, footprint * 48.0f, seed + 739u);
        const float powder = 0.85f + 0.15f * grain.w;
        return f4(deposit_gradient * powder + xyz(grain) * (deposit * 0.15f * 48.0f), deposit * powder);
    }
    if (kind == 8u) {  // Sand: wind-aligned ripples and grains
        const float2 r = rot2(make_float2(p.x, p.z), wind);
        const float2 s = make_float2(r.x * scale, r.y * scale);
        const float4 warp = finish_noise(mk3(s.x * 0.045f, 0.0f, s.y * 0.045f), seed);
        const float phase = 2.0f * SF_PI * (s.x + 1.7f * warp.w + 0.12f * sinf(s.y * 0.22f));
        const float w3 = width * 3.0f;
        const float visible = expf(-(w3 * w3));
        const float ripple = 0.5f + 0.36f * sinf(phase) + 0.10f * sinf(2.0f * phase);
        const float amp = 2.0f * SF_PI * (0.36f * cosf(phase) + 0.20f * cosf(2.0f * phase));
        const float k = amp * scale * visible;
        const float2 gradient = make_float2((1.0f + 0.0765f * warp.x) * k,
                                            (0.0264f * cosf(s.y * 0.22f) + 0.0765f * warp.z) * k);
        const float4 grain = finish_fbm(p * 90.0f, footprint * 90.0f, seed + 139u);
        const float2 grad = rot2(gradient, -wind);
        return f4(mk3(grad.x, 0.0f, grad.y) + xyz(grain) * 2.5f, 0.70f * mixf(0.5f, ripple, visible) + 0.30f * grain.w);
    }
    if (kind == 6u) {  // Rosettes: carved flowers in a square lattice on xz
        const float tx = fractf(q.x + 0.5f) - 0.5f, ty = fractf(q.z + 0.5f) - 0.5f;
        const float r = fmaxf(sqrtf(tx * tx + ty * ty), 1e-5f);
        const float angle = atan2f(ty, tx);
        const float flower = r - 0.25f - 0.07f * cosf(angle * 8.0f);
        const float ring = r - 0.45f;
        const float ax = -ty / (r * r), ay = tx / (r * r);
        const float sf = signf(flower), k8 = 0.56f * sinf(angle * 8.0f);
        float gx = sf * (tx / r + k8 * ax), gy = sf * (ty / r + k8 * ay);
        float distance = fabsf(flower);
        if (fabsf(ring) < distance) {
            distance = fabsf(ring);
            const float sr = signf(ring);
            gx = sr * tx / r;
            gy = sr * ty / r;
        }
        const float visible = 1.0f - sstep(0.10f, 0.40f, width);
        const float carving = 1.0f - sstep(0.012f, 0.045f, distance);
        const float k = -finish_smooth_derivative(0.012f, 0.045f, distance) * visible * scale;
        return make_float4(gx * k, 0.0f, gy * k, mixf(0.2f, carving, visible));
    }
    if (kind == 3u) {  // BrushedMetal: stretched noise
        const float3 axes = mk3(18.0f, 0.45f, 3.0f);
        const float4 n = finish_fbm(q * axes, width * 18.0f, seed);
        return f4(xyz(n) * axes * scale, n.w);
    }
    const float4 n = finish_fbm(q, width, seed);
    float4 result = n;
    if (kind == 1u) {  // VeinedStone
        const float3 axis = mk3(0.16f, 0.11f, 0.08f);
        const float phase = (dot3(q, axis) + n.w * 2.8f) * SF_PI * 2.0f;
        const float wave = sinf(phase);
        const float veins = 1.0f - sstep(0.035f, 0.19f, fabsf(wave));
        const float3 gradient = (axis + xyz(n) * 2.8f) *
                                (-finish_smooth_derivative(0.035f, 0.19f, fabsf(wave)) * signf(wave) * cosf(phase) *
                                 SF_PI * 2.0f);
        const float visible = 1.0f - sstep(0.18f, 0.45f, width);
        result = mix4(n, add4(scale4(n, 0.65f), scale4(f4(gradient, veins), 0.35f)), visible);
    } else if (kind == 2u) {  // Patina
        result = f4(xyz(n) * finish_smooth_derivative(0.35f, 0.67f, n.w), sstep(0.35f, 0.67f, n.w));
    } else if (kind == 4u || kind == 7u) {  // Basalt, CoastalRock
        const float4 grain = finish_fbm(q * 3.7f, width * 3.7f, seed + 53u);
        result = add4(scale4(n, 0.8f), scale4(f4(xyz(grain) * 3.7f, grain.w), 0.2f));
    } else if (kind == 5u) {  // Ripples
        const float a = q.x + 0.75f * n.w;
        const float b = fmaf(q.z, 1.37f, q.x * 0.4f);
        const float visible = 1.0f - sstep(0.35f, 1.0f, width);
        const float3 gradient = ((mk3(1.f, 0.f, 0.f) + xyz(n) * 0.75f) * (0.32f * cosf(a)) +
                                 mk3(0.4f, 0.0f, 1.37f) * (0.18f * cosf(b))) * visible;
        result = f4(gradient, 0.5f + (0.32f * sinf(a) + 0.18f * sinf(b)) * visible);
    }
    return f4(xyz(result) * scale, result.w);
}
// finish_normal (:155-159): the gradient's tangential part bends the normal, limited
// so the slope stays below 0.75.
__device__ __forceinline__ float3 finish_normal(float bump, float3 n, float3 gradient) {
    const float3 slope = gradient - n * dot3(gradient, n);
    const float limit = 0.75f / fmaxf(len3(slope), 1e-5f);
    return safe_normalize3(n - slope * fminf(fmaxf(bump, -limit), limit));
}

// ------------------------------------------------------------------ ramps
// palette_sample (common.wgsl:331-362).
static __device__ float3 ramp_sample(const DevRamp& r, float value) {
    const uint32_t n = r.n;
    if (n == 0) return mk3(1.f, 1.f, 1.f);
    if (n == 1) return ld3(r.stops[0]);
    auto mixs = [&](uint32_t a, uint32_t b, float amount) {
        float f = fminf(fmaxf(amount, 0.0f), 1.0f);
        if (r.smooth) f = f * f * (3.0f - 2.0f * f);
        const float g = 1.0f - f;
        return mk3(fmaf(r.stops[a][0], g, r.stops[b][0] * f), fmaf(r.stops[a][1], g, r.stops[b][1] * f),
                   fmaf(r.stops[a][2], g, r.stops[b][2] * f));
    };
    float t = value * r.map[0] + r.map[1];
    if (r.cyclic) t = t - floorf(t);
    else t = fminf(fmaxf(t, 0.0f), 1.0f);
    if (r.map[2] != 1.0f) t = powf(t, r.map[2]);
    if (!r.positioned && !r.cyclic) {
        const float x = t * float(n - 1);
        const uint32_t i = min(uint32_t(floorf(x)), n - 2);
        return mixs(i, i + 1, x - float(i));
    }
    const float first = r.stops[0][3], last = r.stops[n - 1][3];
    if (r.cyclic && (t < first || t >= last)) {
        const float x = t < first ? t + 1.0f : t;
        return mixs(n - 1, 0, (x - last) / fmaxf(1.0f + first - last, 1e-8f));
    }
    if (t <= first) return ld3(r.stops[0]);
    if (t >= last) return ld3(r.stops[n - 1]);
    for (uint32_t i = 0; i + 1 < n; ++i)
        if (t < r.stops[i + 1][3]) return mixs(i, i + 1, (t - r.stops[i][3]) / (r.stops[i + 1][3] - r.stops[i][3]));
    return ld3(r.stops[n - 1]);
}
// OrbitColoring::value (material.rs:39-55) and pathtrace.wgsl:277-282: the weighted
// traps, iteration fraction and normal term, optionally log-remapped.
__device__ __forceinline__ float orbit_mix(const float* w, const float* extra, const float* traps, float iter_frac,
                                           float normal_term) {
    float v = w[0] * traps[0] + w[1] * traps[1] + w[2] * traps[2] + w[3] * traps[3] + extra[0] * iter_frac +
              extra[1] * normal_term;
    const float gain = extra[2];
    if (gain > 0.0f) v = signf(v) * logf(1.0f + gain * fabsf(v)) / logf(1.0f + gain);
    return v;
}

// ------------------------------------------------------------------ textures
// pattern_value (pattern.wgsl:2-49): octaves of the texture graph's exact sample at
// the mapped point (or its fan mapping), the channel's value, contrast.
static __device__ float texture_value(const DevTexture& T, float3 p) {
    const DeProgram& TP = *reinterpret_cast<const DeProgram*>(T.prog);
    const float3 rot = mk3(T.rotation[0], T.rotation[1], T.rotation[2]);
    const float3 off = mk3(T.mapping[0], T.mapping[1], T.mapping[2]);
    const float scale = T.mapping[3];
    float3 q = rotate_euler_xyz(p * scale, rot) + off;
    float fan_angle = 0.0f, fan_radius = 0.0f;
    if (T.fan[3] > 0.0f) {
        q = rotate_euler_xyz(p, rot) + off;
        const float row = floorf(q.z / T.fan[1]);
        const float x = modf_euclid(q.x + modf_euclid(row, 2.0f) * T.fan[0] * 0.5f, T.fan[0]) - T.fan[0] * 0.5f;
        const float z = modf_euclid(q.z, T.fan[1]) + 0.03f;
        fan_angle = atan2f(x, z);
        fan_radius = sqrtf(x * x + z * z);
        q = mk3(fan_angle * T.fan[2] / SF_PI, q.y, fan_radius) * scale;
    }
    const bool orbit = T.channel == 7u;
    const float budget = fmaxf(float(T.budget), 1.0f);
    float total = 0.0f, weights = 0.0f, weight = 1.0f;
    for (uint32_t octave = 0; octave < T.octaves; ++octave) {
        const DeSampleF smp = de_finalize(TP, de_raw_exact(TP, q));
        float value;
        if (orbit) value = orbit_mix(T.weights, T.extra, smp.traps, float(smp.iter) / budget, 0.5f);
        else if (T.channel < 4u) value = smp.traps[T.channel];
        else if (T.channel == 4u) value = float(smp.iter) / budget;
        else value = 0.5f + 0.5f * smp.d / (1.0f + fabsf(smp.d));
        if (!(value >= -3.4028235e38f && value <= 3.4028235e38f)) value = 0.5f;  // NaN and infinities
        total += (orbit ? value : fminf(fmaxf(value, 0.0f), 1.0f)) * weight;
        weights += weight;
        q = q * 2.0f + mk3(0.73f, 1.17f, 0.91f);
        weight *= 0.5f;
    }
    const float fractal = total / fmaxf(weights, 1e-6f);
    float value = fractal;
    if (T.fan[3] > 0.0f) {
        const float spoke = powf(1.0f - fabsf(sinf(fan_angle * T.fan[2] + 0.16f * (fractal - 0.5f))), 4.0f);
        const float arc = powf(1.0f - fabsf(sinf(fan_radius * scale * SF_PI + 0.35f * fractal)), 6.0f);
        value = 0.16f + 0.28f * fractal + 0.42f * spoke + 0.22f * arc;
    }
    const float result = (value - 0.5f) * T.rotation[3] + 0.5f;
    return orbit ? result : fminf(fmaxf(result, 0.0f), 1.0f);
}
// texture_mask (texture.wgsl:17-21): 1 - smoothstep over |trap - value|.
__device__ __forceinline__ float texture_mask(const DevTexture& T, const float* traps) {
    if (T.mask[3] == 0.0f) return 1.0f;
    return 1.0f - sstep(T.mask[2] * 0.5f, T.mask[2], fabsf(traps[uint32_t(T.mask[0]) & 3u] - T.mask[1]));
}
// texture_filtered_value (texture.wgsl:27-31): fades to 0.5 as the footprint grows.
__device__ __forceinline__ float texture_filtered_value(const DevTexture& T, float3 p, float footprint) {
    const float fade = sstep(0.25f, 0.75f, footprint * T.mapping[3]);
    if (fade >= 1.0f) return 0.5f;
    return mixf(texture_value(T, p), 0.5f, fade);
}
// texture_parallax (texture.wgsl:35-55): the height field's ray intersection in the
// tangent plane, by linear search over the layers with a secant refinement.
static __device__ float3 texture_parallax(const DevTexture& T, float3 p, float3 n, float3 v, float footprint) {
    const float depth = T.parallax[0] / T.mapping[3];
    if (depth <= 0.0f || depth < footprint * 0.25f) return p;
    const float nv = fmaxf(dot3(n, v), 0.15f);
    const float3 direction = (v - n * dot3(n, v)) / nv + n;
    const uint32_t layers = uint32_t(mixf(4.0f, T.parallax[1], 1.0f - fminf(fmaxf(nv, 0.0f), 1.0f)));
    const uint32_t count = max(layers, 4u);
    const float step = 1.0f / float(count);
    float previous = texture_value(T, p) - 1.0f;
    float layer = 0.0f;
    for (uint32_t i = 0; i < count; ++i) {
        layer += step;
        const float3 q = p - direction * (depth * layer);
        const float crossing = layer + texture_value(T, q) - 1.0f;
        if (crossing >= 0.0f) {
            const float fraction = fminf(fmaxf(-previous / fmaxf(crossing - previous, 1e-6f), 0.0f), 1.0f);
            return p - direction * (depth * (layer - step + step * fraction));
        }
        previous = crossing;
    }
    return p - direction * depth;
}
// texture_normal (texture.wgsl:57-72): the footprint-filtered tetrahedral gradient of
// the texture bends the normal, at most 45 degrees from it.
static __device__ float3 texture_normal(const DevTexture& T, float3 p, float3 n, float footprint) {
    const float fade = sstep(0.25f, 0.75f, footprint * T.mapping[3]);
    if (fade >= 1.0f) return n;
    const float h = fmaxf(footprint, 0.005f / T.mapping[3]);
    const float3 a = mk3(1.f, -1.f, -1.f), b = mk3(-1.f, -1.f, 1.f), c = mk3(-1.f, 1.f, -1.f), d = mk3(1.f, 1.f, 1.f);
    const float3 gradient = (a * texture_value(T, p + a * h) + b * texture_value(T, p + b * h) +
                             c * texture_value(T, p + c * h) + d * texture_value(T, p + d * h)) / (4.0f * h);
    float3 tangent = (gradient - n * dot3(n, gradient)) * (T.effects[2] * (1.0f - fade) / T.mapping[3]);
    tangent = tangent / fmaxf(1.0f, len3(tangent));
    return safe_normalize3(n - tangent);
}

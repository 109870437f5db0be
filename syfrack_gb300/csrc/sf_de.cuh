// Distance-estimator evaluation on sm_103a.
//
// Device twin of the reference's CPU interpreter (crates/syfrack-core/src/
// scene/graph/eval.rs:346-826) and of the generated WGSL `de_sample`
// (crates/syfrack-render/src/graph_wgsl.rs:385-681). FP32 throughout.
// Three iterated forms have straight-line routines selected on the host; every
// other supported graph runs through the postfix interpreter at the end.
#pragma once
#include <math.h>
#include <stdint.h>

#include "../../include/syfrack_gpu.h"
#include "sf_program.h"

#define SF_INF __int_as_float(0x7f800000)

// ------------------------------------------------------------------ float3 helpers
__device__ __forceinline__ float3 mk3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return mk3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float3 operator/(float3 a, float3 b) { return mk3(a.x / b.x, a.y / b.y, a.z / b.z); }
// Sums of products are written as explicit fused multiply-adds: contraction of
// a*b + c*d may fuse either product, and the choice can differ between the kernels
// a routine is inlined into. Fixed fusion gives every kernel the same bits.
__device__ __forceinline__ float dot3(float3 a, float3 b) { return fmaf(a.z, b.z, fmaf(a.x, b.x, a.y * b.y)); }
__device__ __forceinline__ float diff_of_products(float a, float b, float c, float d) { return fmaf(a, b, -(c * d)); }
__device__ __forceinline__ float sum_of_products(float a, float b, float c, float d) { return fmaf(a, b, c * d); }
__device__ __forceinline__ float len3(float3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ float3 abs3(float3 a) { return mk3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return mk3(diff_of_products(a.y, b.z, a.z, b.y), diff_of_products(a.z, b.x, a.x, b.z),
               diff_of_products(a.x, b.y, a.y, b.x));
}
__device__ __forceinline__ float3 ld3(const float* f) { return mk3(f[0], f[1], f[2]); }
__device__ __forceinline__ float max3(float3 a) { return fmaxf(fmaxf(a.x, a.y), a.z); }
__device__ __forceinline__ float min3(float3 a) { return fminf(fminf(a.x, a.y), a.z); }
__device__ __forceinline__ float3 clamp3(float3 v, float lo, float hi) {
    return mk3(fminf(fmaxf(v.x, lo), hi), fminf(fmaxf(v.y, lo), hi), fminf(fmaxf(v.z, lo), hi));
}
__device__ __forceinline__ float3 normalize3(float3 v) { return v / len3(v); }
// glam try_normalize().unwrap_or(Y) (common.wgsl:241-246).
__device__ __forceinline__ float3 safe_normalize3(float3 v) {
    float l = len3(v);
    float rcp = 1.0f / l;
    if (!(l > 0.0f) || !(rcp > 0.0f) || !(rcp <= 3.4028235e38f)) return mk3(0.f, 1.f, 0.f);
    return v * rcp;
}
__device__ __forceinline__ float rem_euclid(float x, float m) {
    float r = fmodf(x, m);
    return r < 0.0f ? r + fabsf(m) : r;
}

// Raw DE state before normalisation (eval.rs DistState :14-19).
struct DeRaw {
    float d;
    float t0, t1, t2, t3;  // raw trap slots (+inf = unwritten)
    uint32_t iter;
    uint32_t material;
    uint32_t flags;  // bit 0: d is a skipped Bounded branch's conservative bound (DeSample.flags)
};

// Normalised sample (PreparedGraph::evaluate, eval.rs:98-114).
struct DeSampleF {
    float d;
    float traps[4];
    uint32_t iter;
    uint32_t material;
};

// (t / scale).min(1): the quotient in WGSL's division accuracy class (<= 2 ulp).
__device__ __forceinline__ float trap_norm(float t, float scale) {
    float q;
    asm("div.approx.ftz.f32 %0, %1, %2;" : "=f"(q) : "f"(t), "f"(scale));
    return isfinite(t) ? fminf(q, 1.0f) : 1.0f;
}
__device__ __forceinline__ DeSampleF de_finalize(const DeProgram& P, const DeRaw& r) {
    DeSampleF s;
    s.d = r.d;
    s.traps[0] = trap_norm(r.t0, P.trap_scales[0]);
    s.traps[1] = trap_norm(r.t1, P.trap_scales[1]);
    s.traps[2] = trap_norm(r.t2, P.trap_scales[2]);
    s.traps[3] = trap_norm(r.t3, P.trap_scales[3]);
    s.iter = min(r.iter, P.iteration_product);
    s.material = r.material;
    return s;
}

// measure (eval.rs:299-331).
__device__ __forceinline__ float trap_measure(uint32_t m, float3 p) {
    const float TAU = 6.2831855f;
    switch (m) {
    case SF_MEASURE_AXIS_X: return sqrtf(p.y * p.y + p.z * p.z);
    case SF_MEASURE_AXIS_Y: return sqrtf(p.x * p.x + p.z * p.z);
    case SF_MEASURE_AXIS_Z: return sqrtf(p.x * p.x + p.y * p.y);
    case SF_MEASURE_PLANE_Y: return fabsf(p.y);
    case SF_MEASURE_ANGLE_XY: return (p.x == 0.f && p.y == 0.f) ? 0.5f : atan2f(p.y, p.x) / TAU + 0.5f;
    case SF_MEASURE_ANGLE_XZ: return (p.x == 0.f && p.z == 0.f) ? 0.5f : atan2f(p.z, p.x) / TAU + 0.5f;
    case SF_MEASURE_ANGLE_YZ: return (p.y == 0.f && p.z == 0.f) ? 0.5f : atan2f(p.z, p.y) / TAU + 0.5f;
    case SF_MEASURE_LOG_NORM: return log1pf(len3(p));
    default: return len3(p);
    }
}
// Trap slot update (eval.rs:533-552) on four named registers (no local memory).
__device__ __forceinline__ float trap_mode_apply(uint32_t mode, float old, float v) {
    if (mode == SF_TRAP_LAST) return v;
    if (mode == SF_TRAP_MAXIMUM) return old >= 1e30f ? v : fmaxf(old, v);
    return fminf(old, v);
}
__device__ __forceinline__ void trap_update(DeRaw& s, uint32_t slot, uint32_t mode, float v) {
    if (slot == 0) s.t0 = trap_mode_apply(mode, s.t0, v);
    else if (slot == 1) s.t1 = trap_mode_apply(mode, s.t1, v);
    else if (slot == 2) s.t2 = trap_mode_apply(mode, s.t2, v);
    else s.t3 = trap_mode_apply(mode, s.t3, v);
}

// A Norm trap kept as |p|^2 (Minimum / Last modes): sqrtf is monotonic, so the
// root of the minimum (or of the last value) equals the reference's minimum of roots.
__device__ __forceinline__ void trap_sqrt(DeRaw& s, uint32_t slot) {
    if (slot == 0) s.t0 = sqrtf(s.t0);
    else if (slot == 1) s.t1 = sqrtf(s.t1);
    else if (slot == 2) s.t2 = sqrtf(s.t2);
    else s.t3 = sqrtf(s.t3);
}

// Square root and quotient in the accuracy class WGSL gives its own sqrt and
// division (a few ulp): one MUFU reciprocal square root / reciprocal and a multiply.
__device__ __forceinline__ float sqrt_fast(float x) { return x > 0.0f && x < SF_INF ? x * rsqrtf(x) : x; }
// 1/x by the hardware approximation (PTX rcp.approx.ftz.f32, max error 1 ulp):
// (a.x * b + c.x, a.y * b + c.y) as one packed FMA (fma.rn.f32x2, sm_100 and later):
// each lane rounds exactly as fmaf does, in one issue slot instead of two.
__device__ __forceinline__ float2 fma2_scalar(float ax, float ay, float b, float cx, float cy) {
    unsigned long long ra, rb, rc, rd;
    asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(ax), "f"(ay));
    asm("mov.b64 %0, {%1, %1};" : "=l"(rb) : "f"(b));
    asm("mov.b64 %0, {%1, %2};" : "=l"(rc) : "f"(cx), "f"(cy));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(rd) : "l"(ra), "l"(rb), "l"(rc));
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(rd));
    return r;
}

// x / y as x * rcp_approx(y) is within 2 ulp for normal y.
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// integral_spherical_power (eval.rs:129-178): complex powers of the polar and
// azimuthal unit vectors; n = 6, 8 by repeated squaring, other n by binary powers.
// The quotients by r and rho use the hardware reciprocal (WGSL's division accuracy
// class, as the reference's bulb_power68 on the GPU).
__device__ __forceinline__ void spherical_power(float3 p, float r, uint32_t n, float3& out, float& deriv) {
    if (n == 1) { out = p; deriv = 1.0f; return; }
    const float rho = sqrt_fast(fmaf(p.x, p.x, p.y * p.y));
    const float ir = rcp_approx(r);
    float tx = fminf(fmaxf(p.z * ir, -1.0f), 1.0f), ty = rho * ir;
    float fx = 1.0f, fy = 0.0f;
    if (rho > 0.0f) {
        const float irho = rcp_approx(rho);
        fx = p.x * irho;
        fy = p.y * irho;
    }
    if (n == 8 || n == 6) {
        float t2x = diff_of_products(tx, tx, ty, ty), t2y = 2.0f * tx * ty;
        float f2x = diff_of_products(fx, fx, fy, fy), f2y = 2.0f * fx * fy;
        float t4x = diff_of_products(t2x, t2x, t2y, t2y), t4y = 2.0f * t2x * t2y;
        float f4x = diff_of_products(f2x, f2x, f2y, f2y), f4y = 2.0f * f2x * f2y;
        float r2 = r * r, r4 = r2 * r2;
        float ax, ay, bx, by, prev;
        if (n == 6) {
            ax = diff_of_products(t2x, t4x, t2y, t4y); ay = sum_of_products(t2x, t4y, t2y, t4x);
            bx = diff_of_products(f2x, f4x, f2y, f4y); by = sum_of_products(f2x, f4y, f2y, f4x);
            prev = r4 * r;
        } else {
            ax = diff_of_products(t4x, t4x, t4y, t4y); ay = 2.0f * t4x * t4y;
            bx = diff_of_products(f4x, f4x, f4y, f4y); by = 2.0f * f4x * f4y;
            prev = r4 * r2 * r;
        }
        float m = prev * r;
        out = mk3(ay * bx * m, ay * by * m, ax * m);
        deriv = float(n) * prev;
        return;
    }
    float ax = 1.f, ay = 0.f, bx = 1.f, by = 0.f;
    uint32_t e = n;
    while (e != 0) {
        if (e & 1u) {
            float nx = diff_of_products(ax, tx, ay, ty), ny = sum_of_products(ax, ty, ay, tx); ax = nx; ay = ny;
            nx = diff_of_products(bx, fx, by, fy); ny = sum_of_products(bx, fy, by, fx); bx = nx; by = ny;
        }
        e >>= 1;
        if (e != 0) {
            float nx = diff_of_products(tx, tx, ty, ty), ny = sum_of_products(tx, ty, ty, tx); tx = nx; ty = ny;
            nx = diff_of_products(fx, fx, fy, fy); ny = sum_of_products(fx, fy, fy, fx); fx = nx; fy = ny;
        }
    }
    float prev = 1.0f;
    for (uint32_t i = 1; i < n; ++i) prev *= r;
    float m = prev * r;
    out = mk3(ay * bx * m, ay * by * m, ax * m);
    deriv = float(n) * prev;
}

// Power node (eval.rs:456-476), including the trigonometric path for
// non-integer exponents and radii below 1e-12.
__device__ __forceinline__ void power_op(float3& p, float& dr, float radius, float power, uint32_t power_int) {
    if (radius >= 1e-12f && power_int != 0) {
        float3 q;
        float dv;
        spherical_power(p, radius, power_int, q, dv);
        p = q;
        dr *= dv;
        return;
    }
    float r = fmaxf(radius, 1e-12f);
    float theta = radius >= 1e-12f ? atan2f(sqrtf(p.x * p.x + p.y * p.y), p.z)
                                   : acosf(fminf(fmaxf(p.z / r, -1.0f), 1.0f));
    float phi = atan2f(p.y, p.x);
    dr *= powf(r, power - 1.0f) * power;
    float zr = powf(r, power);
    float st, ct, sp, cp;
    sincosf(theta * power, &st, &ct);
    sincosf(phi * power, &sp, &cp);
    p = mk3(st * cp, st * sp, ct) * zr;
}

__device__ __forceinline__ float bulb_fence(float3 p, float dr) {
    float r = fmaxf(sqrt_fast(dot3(p, p)), 1e-12f);
    return 0.5f * logf(r) * r * rcp_approx(dr);
}
__device__ __forceinline__ float box_fence(float3 p, float3 half, float dr) {
    float3 q = abs3(p) - half;
    float3 qm = mk3(fmaxf(q.x, 0.f), fmaxf(q.y, 0.f), fmaxf(q.z, 0.f));
    return (sqrt_fast(dot3(qm, qm)) + fminf(fmaxf(q.x, fmaxf(q.y, q.z)), 0.0f)) * rcp_approx(dr);
}

__device__ __forceinline__ DeRaw raw_empty() {
    DeRaw r;
    r.d = SF_INF; r.t0 = r.t1 = r.t2 = r.t3 = SF_INF; r.iter = 0; r.material = 0; r.flags = 0;
    return r;
}

// ------------------------------------------------------------------ specialised forms
// Mandelbulb: Iterate{Trap, Power, AddOrigin} -> BulbFence (graphs/mandelbulb.ron).
__device__ __forceinline__ DeRaw de_bulb(const FormParams& f, float3 p) {
    DeRaw s = raw_empty();
    const float3 c = p;
    float dr = 1.0f;
    const uint32_t n = f.iterations;
    for (uint32_t i = 0; i < n; ++i) {
        // |p| correctly rounded: the power raises it to the n-th, which would multiply
        // any error by n
        float r = len3(p);
        if (r > f.bailout) break;
        float v = f.trap_measure == SF_MEASURE_NORM ? r : trap_measure(f.trap_measure, p);
        trap_update(s, f.trap_slot, f.trap_mode, v);
        power_op(p, dr, r, f.power, f.power_int);
        p = p + c;
        dr += 1.0f;
        s.iter++;
    }
    s.d = bulb_fence(p, dr);
    s.material = f.material;
    return s;
}


// (a.x * b.x, a.y * b.y) as one packed multiply (mul.rn.f32x2): each lane rounds as
// a binary32 multiply.
__device__ __forceinline__ float2 mul2(float ax, float ay, float bx, float by) {
    unsigned long long ra, rb, rd;
    asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(ax), "f"(ay));
    asm("mov.b64 %0, {%1, %2};" : "=l"(rb) : "f"(bx), "f"(by));
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(rd));
    return r;
}

// (a.x + b.x, a.y + b.y) as one packed add (add.rn.f32x2): each lane rounds as a
// binary32 add.
__device__ __forceinline__ float2 add2(float ax, float ay, float bx, float by) {
    unsigned long long ra, rb, rd;
    asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(ax), "f"(ay));
    asm("mov.b64 %0, {%1, %2};" : "=l"(rb) : "f"(bx), "f"(by));
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(rd));
    return r;
}

// Mandelbox: Iterate{BoxFold, Trap, SphereFold, Scale, AddOrigin} -> NormFence.
// NORM_MIN0: the bundled trap (slot 0, Norm, Minimum) kept as min |p|^2.
// The sphere fold's fr^2 / r^2 uses the fast reciprocal division (<= 2 ulp, the
// accuracy class WGSL allows for its own division). CLAMPED (fr >= mr): the
// reference's three cases (eval.rs:408-414) are min(fr^2/mr^2, max(fr^2/r^2, 1)),
// two min/max instead of a compare and a select; otherwise the factor for
// r^2 >= min_radius^2 is max(fr^2 / r^2, 1), which covers r^2 >= fixed_radius^2.
// The factor's products with the scale and with |scale| share one packed multiply.
template <bool NORM_MIN0, bool CLAMPED>
__device__ __forceinline__ DeRaw de_box_t(const FormParams& f, float3 p) {
    DeRaw s = raw_empty();
    float dr = 1.0f;
    const uint32_t n = f.iterations;
    const float l = f.limit, bt = f.bailout_t, mr2 = f.min_radius2, fr2 = f.fixed_radius2, kmin = f.fold_k_min;
    const float sc = f.scale, asc = f.abs_scale;
    const bool sq = f.trap_squared != 0;
    float t0 = SF_INF;
    // The loop carries w = -p: the box fold 2 clamp(p) - p is then fma(clamp(w), -2, w)
    // (clamp(-p) = -clamp(p) exactly), one packed FMA for x and y, and the next -p is
    // fold * (-k scale) + (-c). Every result is the exact negation of the same
    // operation on p, so the iteration rounds as it does on p.
    const float ncx = -p.x, ncy = -p.y, ncz = -p.z;
    float wx = ncx, wy = ncy, wz = ncz;
    uint32_t i = 0;
#pragma unroll 2
    for (; i < n; ++i) {
        if (fmaf(wz, wz, fmaf(wx, wx, wy * wy)) > bt) break;  // dot3(p, p)
        const float2 fxy = fma2_scalar(fminf(fmaxf(wx, -l), l), fminf(fmaxf(wy, -l), l), -2.0f, wx, wy);
        const float fz = fmaf(fminf(fmaxf(wz, -l), l), -2.0f, wz);
        const float3 q = mk3(fxy.x, fxy.y, fz);  // the folded point
        float r2 = dot3(q, q);
        if (NORM_MIN0) {
            t0 = fminf(t0, r2);
        } else {
            float v = sq ? r2 : trap_measure(f.trap_measure, q);
            trap_update(s, f.trap_slot, f.trap_mode, v);
        }
        const float qk = fr2 * rcp_approx(r2);
        const float k = CLAMPED ? fminf(kmin, fmaxf(qk, 1.0f)) : (r2 < mr2 ? kmin : fmaxf(qk, 1.0f));
        // sphere fold, Scale and AddOrigin as one multiply-add per component
        const float2 kk = mul2(k, k, -sc, asc);  // (-k * scale, k * |scale|)
        const float2 wxy = fma2_scalar(q.x, q.y, kk.x, ncx, ncy);
        wx = wxy.x;
        wy = wxy.y;
        wz = fmaf(q.z, kk.x, ncz);
        dr = fmaf(dr, kk.y, 1.0f);
    }
    s.iter = i;
    s.d = (sqrt_fast(fmaf(wz, wz, fmaf(wx, wx, wy * wy))) - f.fence[0]) * rcp_approx(fabsf(dr));
    s.material = f.material;
    if (NORM_MIN0) s.t0 = sqrt_fast(t0);
    else if (sq) trap_sqrt(s, f.trap_slot);
    return s;
}
__device__ __forceinline__ DeRaw de_box(const FormParams& f, float3 p) {
    if (f.trap_squared && f.trap_slot == 0 && f.trap_mode == SF_TRAP_MINIMUM)
        return f.fold_clamped ? de_box_t<true, true>(f, p) : de_box_t<true, false>(f, p);
    return f.fold_clamped ? de_box_t<false, true>(f, p) : de_box_t<false, false>(f, p);
}

// Menger: Iterate{MengerFold, Trap} -> Box (graphs/menger.ron).
__device__ __forceinline__ DeRaw de_menger(const FormParams& f, float3 p) {
    DeRaw s = raw_empty();
    float dr = 1.0f;
    const uint32_t n = f.iterations;
    const float sc = f.scale;
    const float3 off = mk3(f.offset[0], f.offset[1], f.offset[2]);
    const bool sq = f.trap_squared != 0;
    for (uint32_t i = 0; i < n; ++i) {
        if (dot3(p, p) > f.bailout_t) break;
        float3 z = abs3(p);
        if (z.x < z.y) z = mk3(z.y, z.x, z.z);
        if (z.x < z.z) z = mk3(z.z, z.y, z.x);
        if (z.y < z.z) z = mk3(z.x, z.z, z.y);
        z = z * sc - off * (sc - 1.0f);
        if (z.z < -0.5f * off.z * (sc - 1.0f)) z.z += off.z * (sc - 1.0f);
        p = z;
        dr *= sc;
        float v = sq ? dot3(p, p) : trap_measure(f.trap_measure, p);
        trap_update(s, f.trap_slot, f.trap_mode, v);
        s.iter++;
    }
    s.d = box_fence(p, mk3(f.fence[0], f.fence[1], f.fence[2]), dr);
    s.material = f.material;
    if (sq) trap_sqrt(s, f.trap_slot);
    return s;
}

// ------------------------------------------------------------------ generic interpreter
struct PState {
    float3 p;
    float dr;
    uint32_t iter;
    float t0, t1, t2, t3;
};

__device__ __forceinline__ float3 rotate_euler_xyz(float3 p, float3 a) {
    float3 q = p;
    q = mk3(cosf(a.z) * q.x - sinf(a.z) * q.y, sinf(a.z) * q.x + cosf(a.z) * q.y, q.z);
    q = mk3(cosf(a.y) * q.x + sinf(a.y) * q.z, q.y, -sinf(a.y) * q.x + cosf(a.y) * q.z);
    q = mk3(q.x, cosf(a.x) * q.y - sinf(a.x) * q.z, sinf(a.x) * q.y + cosf(a.x) * q.z);
    return q;
}
__device__ __forceinline__ float to_rad(float d) { return d * (3.14159265358979323846f / 180.0f); }

__device__ __forceinline__ float terrain_hash(int cx, int cy, int cz, uint32_t seed) {
    uint32_t h = (uint32_t(cx) * 0x8da6b343u) ^ (uint32_t(cy) * 0xd8163841u) ^ (uint32_t(cz) * 0xcb1ab31fu) ^ seed;
    h = (h ^ (h >> 16)) * 0x7feb352du;
    h = (h ^ (h >> 15)) * 0x846ca68bu;
    h ^= h >> 16;
    return float(h >> 8) / 16777216.0f;
}
static __device__ float terrain_noise(float3 p, uint32_t seed) {
    float3 base = mk3(floorf(p.x), floorf(p.y), floorf(p.z));
    float3 f = p - base;
    float3 t = f * f * (mk3(3.f, 3.f, 3.f) - f * 2.0f);
    int c0 = int(base.x), c1 = int(base.y), c2 = int(base.z);
#define SF_MIX(a, b, t) ((a) + ((b) - (a)) * (t))
    float a = SF_MIX(terrain_hash(c0, c1, c2, seed), terrain_hash(c0 + 1, c1, c2, seed), t.x);
    float b = SF_MIX(terrain_hash(c0, c1 + 1, c2, seed), terrain_hash(c0 + 1, c1 + 1, c2, seed), t.x);
    float d = SF_MIX(terrain_hash(c0, c1, c2 + 1, seed), terrain_hash(c0 + 1, c1, c2 + 1, seed), t.x);
    float e = SF_MIX(terrain_hash(c0, c1 + 1, c2 + 1, seed), terrain_hash(c0 + 1, c1 + 1, c2 + 1, seed), t.x);
    float r = SF_MIX(SF_MIX(a, b, t.y), SF_MIX(d, e, t.y), t.z);
#undef SF_MIX
    return r;
}

static __device__ void apply_point_op(const DeOp& op, PState& s, float3 c, float3 seed_p, float seed_dr) {
    switch (op.code) {
    case SF_NODE_TRANSLATE: s.p = s.p + ld3(op.f); break;
    case SF_NODE_ROTATE: s.p = rotate_euler_xyz(s.p, mk3(to_rad(op.f[0]), to_rad(op.f[1]), to_rad(op.f[2]))); break;
    case SF_NODE_SCALE: s.p = s.p * op.f[0]; s.dr *= fabsf(op.f[0]); break;
    case SF_NODE_SCALE_AXES: { float3 f = ld3(op.f); s.p = s.p * f; s.dr *= max3(f); break; }
    case SF_NODE_MIRROR: {
        float3 nn = safe_normalize3(ld3(op.f));
        float h = dot3(s.p, nn) - op.f[3];
        if (h < 0.0f) s.p = s.p - nn * (2.0f * h);
        break;
    }
    case SF_NODE_BOX_FOLD: s.p = clamp3(s.p, -op.f[0], op.f[0]) * 2.0f - s.p; break;
    case SF_NODE_BOX_FOLD_AXES: {
        float3 l = ld3(op.f);
        float3 fo = mk3(fminf(fmaxf(s.p.x, -l.x), l.x), fminf(fmaxf(s.p.y, -l.y), l.y), fminf(fmaxf(s.p.z, -l.z), l.z)) * 2.0f - s.p;
        if (op.a & 1u) s.p.x = fo.x;
        if (op.a & 2u) s.p.y = fo.y;
        if (op.a & 4u) s.p.z = fo.z;
        break;
    }
    case SF_NODE_SPHERE_INVERSION: {
        float k = op.f[0] * op.f[0] / fmaxf(dot3(s.p, s.p), op.f[1] * op.f[1]);
        s.p = s.p * k; s.dr *= k;
        break;
    }
    case SF_NODE_SPHERE_FOLD: {
        float r2 = dot3(s.p, s.p);
        float mr2 = op.f[0] * op.f[0], fr2 = op.f[1] * op.f[1];
        float k = r2 < mr2 ? fr2 / mr2 : (r2 < fr2 ? fr2 / r2 : 1.0f);
        s.p = s.p * k; s.dr *= k;
        break;
    }
    case SF_NODE_ABS:
        if (op.a & 1u) s.p.x = fabsf(s.p.x);
        if (op.a & 2u) s.p.y = fabsf(s.p.y);
        if (op.a & 4u) s.p.z = fabsf(s.p.z);
        break;
    case SF_NODE_MENGER_FOLD: {
        float sc = op.f[0];
        float3 off = mk3(op.f[1], op.f[2], op.f[3]);
        float3 z = abs3(s.p);
        if (z.x < z.y) z = mk3(z.y, z.x, z.z);
        if (z.x < z.z) z = mk3(z.z, z.y, z.x);
        if (z.y < z.z) z = mk3(z.x, z.z, z.y);
        z = z * sc - off * (sc - 1.0f);
        if (z.z < -0.5f * off.z * (sc - 1.0f)) z.z += off.z * (sc - 1.0f);
        s.p = z; s.dr *= sc;
        break;
    }
    case SF_NODE_KALEIDO: {
        float sector = 6.2831855f / float(op.a > 0 ? op.a : 1u);
        float a = atan2f(s.p.z, s.p.x) + to_rad(op.f[0]);
        a = fabsf(rem_euclid(a + sector * 0.5f, sector) - sector * 0.5f);
        float r = sqrtf(s.p.x * s.p.x + s.p.z * s.p.z);
        float sn, cs;
        sincosf(a, &sn, &cs);
        s.p.x = r * cs; s.p.z = r * sn;
        break;
    }
    case SF_NODE_POWER: power_op(s.p, s.dr, len3(s.p), op.f[0], op.a); break;
    case SF_NODE_ADD_ORIGIN: s.p = s.p + c; s.dr += 1.0f; break;
    case SF_NODE_ADD_SEED: { float3 m = ld3(op.f); s.p = s.p + seed_p * m; s.dr += seed_dr * max3(abs3(m)); break; }
    case SF_NODE_ADD_CONSTANT: {
        float3 m = ld3(op.f);
        s.p = s.p + (c * m + ld3(op.f + 3));
        s.dr += max3(abs3(m));
        break;
    }
    case SF_NODE_TWIST: {
        float sn, cs; sincosf(op.f[0] * s.p.y, &sn, &cs);
        float x = cs * s.p.x - sn * s.p.z, z = sn * s.p.x + cs * s.p.z;
        s.p.x = x; s.p.z = z;
        break;
    }
    case SF_NODE_BEND: {
        float sn, cs; sincosf(op.f[0] * s.p.x, &sn, &cs);
        float x = cs * s.p.x - sn * s.p.y, y = sn * s.p.x + cs * s.p.y;
        s.p.x = x; s.p.y = y;
        break;
    }
    case SF_NODE_TILE: {
        float3 per = ld3(op.f), h = per * 0.5f;
        s.p = mk3(rem_euclid(s.p.x + h.x, per.x) - h.x, rem_euclid(s.p.y + h.y, per.y) - h.y,
                  rem_euclid(s.p.z + h.z, per.z) - h.z);
        break;
    }
    case SF_NODE_REPEAT_FINITE: {
        float3 per = ld3(op.f);
        float3 last = mk3(float(op.a) - 1.0f, float(op.b) - 1.0f, float(op.c) - 1.0f);
        float3 h = last * 0.5f;
        float3 q = s.p / per + h + mk3(0.5f, 0.5f, 0.5f);
        float3 cell = mk3(fminf(fmaxf(floorf(q.x), 0.f), last.x), fminf(fmaxf(floorf(q.y), 0.f), last.y),
                          fminf(fmaxf(floorf(q.z), 0.f), last.z)) - h;
        s.p = s.p - cell * per;
        break;
    }
    case SF_NODE_TRAP: {
        float v = trap_measure(op.b, s.p);
        DeRaw tmp;
        tmp.t0 = s.t0; tmp.t1 = s.t1; tmp.t2 = s.t2; tmp.t3 = s.t3;
        trap_update(tmp, op.a, op.c, v);
        s.t0 = tmp.t0; s.t1 = tmp.t1; s.t2 = tmp.t2; s.t3 = tmp.t3;
        break;
    }
    default: break;
    }
}

// fence (eval.rs:558-599).
static __device__ float fence_op(const DeOp& op, const PState& s) {
    switch (op.code) {
    case SF_NODE_SPHERE: return (len3(s.p) - op.f[0]) / s.dr;
    case SF_NODE_TORUS: {
        float q = sqrtf(s.p.x * s.p.x + s.p.z * s.p.z) - op.f[0];
        return (sqrtf(q * q + s.p.y * s.p.y) - op.f[1]) / s.dr;
    }
    case SF_NODE_CYLINDER: {
        float qx = sqrtf(s.p.x * s.p.x + s.p.z * s.p.z) - op.f[0], qy = fabsf(s.p.y) - op.f[1];
        float mx = fmaxf(qx, 0.f), my = fmaxf(qy, 0.f);
        return (sqrtf(mx * mx + my * my) + fminf(fmaxf(qx, qy), 0.0f)) / s.dr;
    }
    case SF_NODE_BOX: return box_fence(s.p, ld3(op.f), s.dr);
    case SF_NODE_ROUND_BOX: {
        float3 half = ld3(op.f);
        float r = fminf(op.f[3], min3(half));
        float3 q = abs3(s.p) - (half - mk3(r, r, r));
        float3 qm = mk3(fmaxf(q.x, 0.f), fmaxf(q.y, 0.f), fmaxf(q.z, 0.f));
        return (len3(qm) + fminf(max3(q), 0.0f) - r) / s.dr;
    }
    case SF_NODE_ROCK: {
        float3 half = ld3(op.f);
        float e = op.f[3];
        float h = min3(half);
        float3 q = s.p * (1.15f / h);
        float relief = 0.57f * terrain_noise(q, op.a) + 0.29f * terrain_noise(q * 2.03f, op.a + 97u) +
                       0.14f * terrain_noise(q * 4.17f, op.a + 193u) - 0.5f;
        return ((len3(s.p / half) - 1.0f - e * relief) * h / (1.0f + 5.22f * e)) / s.dr;
    }
    case SF_NODE_PLANE: return (dot3(s.p, safe_normalize3(ld3(op.f))) - op.f[3]) / s.dr;
    case SF_NODE_NORM_FENCE: return (len3(s.p) - op.f[0]) / fabsf(s.dr);
    case SF_NODE_BULB_FENCE: return bulb_fence(s.p, s.dr);
    default: return SF_INF;
    }
}

__device__ __forceinline__ DeRaw dist_from(const PState& s, float d) {
    DeRaw r;
    r.d = d; r.material = 0; r.iter = s.iter; r.flags = 0;
    r.t0 = s.t0; r.t1 = s.t1; r.t2 = s.t2; r.t3 = s.t3;
    return r;
}

// combine (eval.rs:601-657).
static __device__ DeRaw combine_op(uint32_t kind, float k, DeRaw a, DeRaw b) {
    auto blend = [&](float h, float d) {
        DeRaw r;
        float ta[4] = {a.t0, a.t1, a.t2, a.t3}, tb[4] = {b.t0, b.t1, b.t2, b.t3}, tr[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            bool fa = isfinite(ta[i]), fb = isfinite(tb[i]);
            tr[i] = (fa && fb) ? tb[i] + (ta[i] - tb[i]) * h : (fa ? ta[i] : (fb ? tb[i] : SF_INF));
        }
        r.t0 = tr[0]; r.t1 = tr[1]; r.t2 = tr[2]; r.t3 = tr[3];
        r.d = d;
        r.material = h >= 0.5f ? a.material : b.material;
        r.iter = h >= 0.5f ? a.iter : b.iter;
        return r;
    };
    // flags (graph_wgsl.rs:845-852): a union keeps its winner's, the others join both
    const uint32_t both = a.flags | b.flags;
    DeRaw r;
    switch (kind) {
    case SF_NODE_UNION: { r = a.d <= b.d ? a : b; r.d = fminf(a.d, b.d); return r; }
    case SF_NODE_INTERSECTION: { r = a.d >= b.d ? a : b; r.d = fmaxf(a.d, b.d); break; }
    case SF_NODE_SUBTRACTION: { r = a; r.d = fmaxf(a.d, -b.d); break; }
    case SF_NODE_SMOOTH_UNION: {
        if (a.d >= 1e30f) { r = b; break; }
        if (b.d >= 1e30f) { r = a; break; }
        float h = fminf(fmaxf(0.5f + 0.5f * (b.d - a.d) / k, 0.0f), 1.0f);
        r = blend(h, b.d + (a.d - b.d) * h - k * h * (1.0f - h));
        break;
    }
    case SF_NODE_SMOOTH_INTERSECTION: {
        if (a.d >= 1e30f) { r = b; r.d = SF_INF; break; }
        if (b.d >= 1e30f) { r = a; r.d = SF_INF; break; }
        float h = fminf(fmaxf(0.5f - 0.5f * (b.d - a.d) / k, 0.0f), 1.0f);
        r = blend(h, b.d + (a.d - b.d) * h + k * h * (1.0f - h));
        break;
    }
    default: return a;
    }
    r.flags = both;
    return r;
}

// ------------------------------------------------------------------ instances
// box_distance (common.wgsl) without the derivative.
__device__ __forceinline__ float box_dist(float3 p, float3 half) {
    const float3 q = abs3(p) - half;
    const float3 qm = mk3(fmaxf(q.x, 0.f), fmaxf(q.y, 0.f), fmaxf(q.z, 0.f));
    return sqrt_fast(dot3(qm, qm)) + fminf(max3(q), 0.0f);
}
// A hierarchy node's signed box distance (bvh.rs:19-24; WGSL _cluster_bound).
__device__ __forceinline__ float cluster_bound(const float* nd, float3 p) {
    return box_dist(p - mk3(__ldg(nd), __ldg(nd + 1), __ldg(nd + 2)), mk3(__ldg(nd + 3), __ldg(nd + 4), __ldg(nd + 5)));
}
// The search over one Instances node's copies (graph_wgsl.rs:760-790): seeded at
// the nearest leaf by a greedy descent, then a stackless preorder walk that skips
// subtrees whose bound exceeds the best distance; ties go to the lower placement.
struct InstFrame {
    const float* rows;  // 12 floats per placement
    const float* bvh;   // 8 floats per hierarchy node
    float3 c, half, q;  // the point the node is evaluated at; fence half; current local point
    float margin, w, fence;
    uint32_t cursor, seed, end, chosen, j;
    bool seed_pass, skip;
    DeRaw best;
};
// Next copy whose template must run (its local point in F.q): true; or false when
// the walk has ended (F.best holds the result). Copies skipped by their fence
// (fast mode, fence > margin) are folded into F.best here.
__device__ __forceinline__ bool inst_next(InstFrame& F) {
    while (F.cursor < F.end) {
        const uint32_t cur = F.cursor;
        const bool first = F.seed_pass;
        F.seed_pass = false;
        F.cursor = first ? 0u : cur + 1u;
        const float* nd = F.bvh + size_t(cur) * 8u;
        if (cluster_bound(nd, F.c) > F.best.d) {
            if (!first) F.cursor = uint32_t(__ldg(nd + 6));
            continue;
        }
        const float leaf = __ldg(nd + 7);
        if (leaf < 0.0f || (!first && cur == F.seed)) continue;
        const uint32_t j = uint32_t(leaf);
        // the copy's inverse affine rows: local point, per-axis scale and its minimum
        const float* r = F.rows + size_t(j) * 12u;
        const float4 x = make_float4(__ldg(r), __ldg(r + 1), __ldg(r + 2), __ldg(r + 3));
        const float4 y = make_float4(__ldg(r + 4), __ldg(r + 5), __ldg(r + 6), __ldg(r + 7));
        const float4 z = make_float4(__ldg(r + 8), __ldg(r + 9), __ldg(r + 10), __ldg(r + 11));
        const float3 q = mk3(dot3(mk3(x.x, x.y, x.z), F.c) + x.w, dot3(mk3(y.x, y.y, y.z), F.c) + y.w,
                             dot3(mk3(z.x, z.y, z.z), F.c) + z.w);
        const float3 sc = mk3(rsqrtf(fmaf(x.z, x.z, fmaf(x.x, x.x, x.y * x.y))),
                              rsqrtf(fmaf(y.z, y.z, fmaf(y.x, y.x, y.y * y.y))),
                              rsqrtf(fmaf(z.z, z.z, fmaf(z.x, z.x, z.y * z.y))));
        const float fence = box_dist(q * sc, F.half * sc);
        if (fence > F.best.d) continue;
        if (F.skip && fence > F.margin) {
            DeRaw d = raw_empty();
            d.d = fence;
            d.flags = 1;
            if (d.d < F.best.d || (d.d == F.best.d && j < F.chosen)) { F.best = d; F.chosen = j; }
            continue;
        }
        F.j = j;
        F.w = min3(sc);
        F.fence = fence;
        F.q = q;
        return true;
    }
    return false;
}

// Evaluation modes of the generic interpreter.
enum : uint32_t {
    SF_EVAL_FAST = 0,   // de_sample: skippable branches skipped outside their margin, the sample flagged
    SF_EVAL_EXACT = 1,  // de_sample_exact: every branch evaluated
    // the union probe (graph_wgsl.rs:1124-1136, bounds_only): every skippable Bounded
    // pushes its bound and every skippable Instances its root fence, flagged, whatever
    // the margin; a sample without the flag took no skip and is exact
    SF_EVAL_PROBE = 2
};

// Postfix interpreter over the ops [pc0, pc1) of DeProgram.ops (generic graphs) in
// one of the SF_EVAL_* modes; the whole program is [0, n_ops). Inlined into the two
// entry points below, so the whole-program one keeps its constant range and modes.
__device__ __forceinline__ DeRaw de_run(const DeProgram& P, float3 c, uint32_t mode, uint32_t pc0, uint32_t pc1) {
    const bool exact = mode == SF_EVAL_EXACT, probe = mode == SF_EVAL_PROBE;
    // the copy searches in flight, one per nesting level (eval.rs:808 recurses into the
    // template of each copy; here the template's ops run between INST_BEGIN and INST_END)
    InstFrame frames[SF_MAX_INST_DEPTH];
    int fd = -1;
    PState s;
    s.p = c; s.dr = 1.0f; s.iter = 0; s.t0 = s.t1 = s.t2 = s.t3 = SF_INF;
    uint32_t loop_count[SF_MAX_LOOP_DEPTH];
    float3 loop_seed[SF_MAX_LOOP_DEPTH];
    float loop_seed_dr[SF_MAX_LOOP_DEPTH];
    int depth = 0;
    DeRaw stack[SF_MAX_DIST_STACK];
    int sp = 0;
    float3 seed_p = c;
    float seed_dr = 1.0f;
    for (uint32_t pc = pc0; pc < pc1; ++pc) {
        const DeOp& op = P.ops[pc];
        switch (op.code) {
        case SF_OP_BEGIN:
            s.p = c; s.dr = 1.0f; s.iter = 0; s.t0 = s.t1 = s.t2 = s.t3 = SF_INF;
            seed_p = c; seed_dr = 1.0f; depth = 0;
            break;
        case SF_OP_ITER_BEGIN:
            if (op.a == 0 || dot3(s.p, s.p) > op.f[1] || depth >= SF_MAX_LOOP_DEPTH) { pc = op.b; break; }
            loop_count[depth] = 0;
            loop_seed[depth] = s.p;
            loop_seed_dr[depth] = s.dr;
            seed_p = s.p; seed_dr = s.dr;
            depth++;
            break;
        case SF_OP_ITER_END: {
            const DeOp& b = P.ops[op.a];
            s.iter += 1;
            uint32_t cnt = ++loop_count[depth - 1];
            if (cnt < b.a && !(dot3(s.p, s.p) > b.f[1])) {
                pc = op.a;  // continue at the first body op (pc++ follows)
                seed_p = loop_seed[depth - 1];
                seed_dr = loop_seed_dr[depth - 1];
            } else {
                depth--;
                if (depth > 0) { seed_p = loop_seed[depth - 1]; seed_dr = loop_seed_dr[depth - 1]; }
                else { seed_p = s.p; seed_dr = s.dr; }
            }
            break;
        }
        case SF_OP_FENCE_OFF:
            if (sp < SF_MAX_DIST_STACK) stack[sp++] = dist_from(s, SF_INF);
            break;
        case SF_OP_EMPTY:
            if (sp < SF_MAX_DIST_STACK) stack[sp++] = raw_empty();
            break;
        case SF_OP_TAG:
            if (sp > 0) stack[sp - 1].material = op.a;
            break;
        case SF_OP_BOUND:
            if (sp > 0) stack[sp - 1].d = fmaxf(stack[sp - 1].d, box_fence(s.p, ld3(op.f), s.dr));
            break;
        case SF_OP_BOUND_FAST: {
            if (sp >= SF_MAX_DIST_STACK) break;
            DeRaw b = raw_empty();
            b.d = box_fence(s.p, ld3(op.f), s.dr);
            if (!exact && (probe || b.d > op.f[3])) {
                b.flags = 1;
                stack[sp++] = b;
                pc = op.b;  // past BOUND_END
                break;
            }
            stack[sp++] = b;
            break;
        }
        case SF_OP_INST_BEGIN: {
            if (sp >= SF_MAX_DIST_STACK || fd + 1 >= SF_MAX_INST_DEPTH) { pc = op.b; break; }
            InstFrame& F = frames[++fd];
            const float* base = reinterpret_cast<const float*>(P.inst_data) + op.c;
            F.rows = base;
            F.bvh = base + size_t(op.a) * 12u;
            F.c = c;
            F.half = ld3(op.f);
            F.margin = op.f[3];
            F.skip = op.f[4] != 0.0f && !exact;
            F.end = 2u * op.a - 1u;
            if (F.skip) {
                // empty space needs only the root fence (graph_wgsl.rs:769-771)
                const float env = cluster_bound(F.bvh, c);
                if (probe || env > F.margin) {
                    DeRaw e = raw_empty();
                    e.d = env;
                    e.flags = 1;
                    stack[sp++] = e;
                    pc = op.b;
                    fd--;
                    break;
                }
            }
            uint32_t seed = 0;
            while (seed + 1u < F.end && __ldg(F.bvh + size_t(seed) * 8u + 7u) < 0.0f) {
                const uint32_t left = seed + 1u, right = uint32_t(__ldg(F.bvh + size_t(left) * 8u + 6u));
                seed = (right >= F.end || cluster_bound(F.bvh + size_t(left) * 8u, c) <=
                                              cluster_bound(F.bvh + size_t(right) * 8u, c))
                           ? left
                           : right;
            }
            F.seed = F.cursor = seed;
            F.seed_pass = true;
            F.chosen = op.a;
            F.best = raw_empty();
            F.best.d = 1e30f;
            if (inst_next(F)) { c = F.q; break; }  // the template follows with the copy's point
            stack[sp++] = F.best;
            pc = op.b;
            fd--;
            break;
        }
        case SF_OP_INST_END: {
            if (sp < 1 || fd < 0) break;
            InstFrame& F = frames[fd];
            DeRaw d = stack[--sp];
            d.d = fmaxf(d.d * F.w, F.fence);
            if (d.d < F.best.d || (d.d == F.best.d && F.j < F.chosen)) { F.best = d; F.chosen = F.j; }
            if (inst_next(F)) { c = F.q; pc = op.a; break; }  // next copy: the template again
            c = F.c;  // the point the search ran at (an outer copy's local point, nested)
            stack[sp++] = F.best;
            fd--;
            break;
        }
        case SF_OP_BOUND_END:
            if (sp >= 2) {
                DeRaw r = stack[sp - 1];
                r.d = fmaxf(stack[sp - 2].d, r.d);
                stack[sp - 2] = r;
                sp--;
            }
            break;
        case SF_OP_COMBINE:
            if (sp >= 2) { stack[sp - 2] = combine_op(op.a, op.f[0], stack[sp - 2], stack[sp - 1]); sp--; }
            break;
        default:
            if (op.code >= SF_NODE_SPHERE && op.code <= SF_NODE_BULB_FENCE) {
                if (sp < SF_MAX_DIST_STACK) stack[sp++] = dist_from(s, fence_op(op, s));
            } else {
                // outside any Iterate, AddSeed reinjects the point entering this node
                if (depth == 0) { seed_p = s.p; seed_dr = s.dr; }
                apply_point_op(op, s, c, seed_p, seed_dr);
            }
            break;
        }
    }
    return sp > 0 ? stack[sp - 1] : raw_empty();
}
// The whole program: exact = false is the reference's de_sample (skippable Bounded
// branches skipped outside their margin, the sample flagged); exact = true is
// de_sample_exact (every branch evaluated).
static __device__ __noinline__ DeRaw de_generic(const DeProgram& P, float3 c, bool exact) {
    return de_run(P, c, exact ? SF_EVAL_EXACT : SF_EVAL_FAST, 0, P.n_ops);
}
// One union leaf's op range, probed or exact.
static __device__ __noinline__ DeRaw de_generic_leaf(const DeProgram& P, float3 c, uint32_t mode, uint32_t leaf) {
    return de_run(P, c, mode, P.leaf_begin[leaf], P.leaf_end[leaf]);
}

// The exact sample of a wide union by branch and bound (graph_wgsl.rs:1112-1154): every
// leaf is probed for its conservative distance (a probe that took no skip is the
// leaf's exact sample), then the unsettled leaf with the lowest bound is evaluated
// exactly, lowest index first on ties, until no bound can reach the best. Skippable
// bounds are lower bounds (a bound reached through a Subtraction's second input is
// never skippable), so every leaf left out is strictly farther than the winner and the
// result is the union's own: the nearest leaf, the first in depth-first order on ties
// (a Union keeps its first input when a.d <= b.d). The search starts from the empty
// state rather than the WGSL's 1e30 sentinel, so a union of empty leaves stays +inf
// as the union itself does.
static __device__ __noinline__ DeRaw de_union_exact(const DeProgram& P, float3 c) {
    const uint32_t k = P.union_leaves;
    float lower[SF_MAX_UNION_LEAVES];
    uint32_t settled = 0;  // bit i: leaf i's exact sample is known
    DeRaw best = raw_empty();
    uint32_t winner = k;
    for (uint32_t i = 0; i < k; ++i) {
        const DeRaw s = de_generic_leaf(P, c, SF_EVAL_PROBE, i);
        lower[i] = s.d;
        if (s.flags == 0) {
            settled |= 1u << i;
            if (s.d < best.d || (s.d == best.d && i < winner)) { best = s; winner = i; }
        }
    }
    for (uint32_t step = 0; step < k; ++step) {
        uint32_t chosen = k;
        float bound = SF_INF;
        for (uint32_t i = 0; i < k; ++i)
            if (!((settled >> i) & 1u) && (lower[i] < bound || (lower[i] == bound && i < chosen))) {
                chosen = i;
                bound = lower[i];
            }
        if (chosen == k || bound > best.d) break;
        settled |= 1u << chosen;
        const DeRaw s = de_generic_leaf(P, c, SF_EVAL_EXACT, chosen);
        if (s.d < best.d || (s.d == best.d && chosen < winner)) { best = s; winner = chosen; }
    }
    return best;
}

// Entry point: raw DE at p for the program's form.
__device__ __forceinline__ DeRaw de_raw(const DeProgram& P, float3 p) {
    switch (P.form) {
    case SF_FORM_BULB: return de_bulb(P.fp, p);
    case SF_FORM_BOX: return de_box(P.fp, p);
    case SF_FORM_MENGER: return de_menger(P.fp, p);
    default: return de_generic(P, p, false);
    }
}
// de_sample_exact: the generic program with every Bounded branch evaluated; the
// specialised forms have no bounds. The path tracers take this whole-program form:
// their exact samples (normals, acceptance, refinement) are a small share of their
// work, and the search's call would raise their register allocation.
__device__ __forceinline__ DeRaw de_raw_exact(const DeProgram& P, float3 p) {
    if (P.form != SF_FORM_GENERIC) return de_raw(P, p);
    return de_generic(P, p, true);
}
// The same sample, with a union of SF_UNION_SEARCH_MIN or more leaves searched by
// branch and bound: for the kernels whose work is exact samples (the batched probe,
// the preview's march on the exact field), where each one would otherwise evaluate
// every leaf's detail. Two leaves are left to the whole program: their search saves at
// most one leaf for two probes (a bounded Mandelbulb beside a sphere previews 25%
// slower searched, while a nine-leaf union previews 28% faster).
#define SF_UNION_SEARCH_MIN 3
__device__ __forceinline__ DeRaw de_raw_exact_search(const DeProgram& P, float3 p) {
    if (P.form != SF_FORM_GENERIC) return de_raw(P, p);
    if (P.union_leaves >= SF_UNION_SEARCH_MIN) return de_union_exact(P, p);
    return de_generic(P, p, true);
}
// The march's sample (pathtrace.wgsl:100-106, lights.wgsl:234): a flagged sample
// whose radius is within five hit cones of acceptance is replaced by the exact one.
// absolute selects the fixed-epsilon rule of the primary-ray configuration.
__device__ __forceinline__ bool needs_exact(const DeRaw& s, float t, float safety, float accept, bool absolute) {
    if (!s.flags) return false;
    const float radius = fabsf(s.d) * safety;
    return absolute ? radius <= accept * 5.0f : radius / fmaxf(t, 1e-6f) <= accept * 5.0f;
}

// Escape-time sampling: PlanarFractal::sample (planar.rs:77-194) at probe points
// (k_planar) and over the flat canvas (k_escape2d, pathtrace.wgsl:1226-1239).
//
// The orbit is evaluated in explicitly rounded binary32 operations (no
// contraction), so iteration counts and the smooth time equal the reference's f32
// arithmetic exactly. Two changes keep those results while doing less work:
//  * the bailout test |z| > b is made on |z|^2 against the largest float whose
//    correctly rounded square root is <= b (bail_t, computed on the host), which
//    selects exactly the same iterations without a square root;
//  * z^n starts from z instead of 1 * z, and the twist rotation is skipped when the
//    twist is zero; both are exact up to the sign of a zero component.
// The traps (ring, stripe bands, final angle) are tolerance quantities (the
// reference's own GPU parity bound is 0.006): for an integer stripe count k the
// per-iteration sin(k atan2(y, x)) comes from the Chebyshev recurrence on
// cos(theta), sin(theta) = z/|z|, and the ring distance uses |z| = |z|^2 rsqrt(|z|^2). With TRAPS = false only the
// iteration count, smooth time and distance are produced.
#include <cuda_runtime.h>

#include "sf_kernels.cuh"
#include "sf_trace.cuh"
#include "sf_warp.cuh"

#define FM(a, b) __fmul_rn((a), (b))
#define FA(a, b) __fadd_rn((a), (b))
#define FS(a, b) __fsub_rn((a), (b))

static __device__ __forceinline__ void cmul_rn(float ax, float ay, float bx, float by, float& rx, float& ry) {
    rx = FS(FM(ax, bx), FM(ay, by));
    ry = FA(FM(ax, by), FM(ay, bx));
}
// z^n for n >= 1, multiplying an accumulator by z on the right (planar.rs complex power).
static __device__ __forceinline__ void cpow_rn(float zx, float zy, uint32_t n, float& rx, float& ry) {
    float x = zx, y = zy;
    for (uint32_t i = 1; i < n; ++i) {
        float nx, ny;
        cmul_rn(x, y, zx, zy, nx, ny);
        x = nx;
        y = ny;
    }
    rx = x;
    ry = y;
}
static __device__ __forceinline__ float len2_rn(float x, float y) { return __fsqrt_rn(FA(FM(x, x), FM(y, y))); }

// PlanarFractal's map of a sample point (planar.rs:79-100): rotate, /zoom, inversion, +centre.
static __device__ __forceinline__ void planar_map(const PlanarDev& f, float ix, float iy, float& px, float& py) {
    px = __fdiv_rn(FS(FM(f.angle_cos, ix), FM(f.angle_sin, iy)), f.zoom);
    py = __fdiv_rn(FA(FM(f.angle_sin, ix), FM(f.angle_cos, iy)), f.zoom);
    if (f.inversion != 0.0f) {
        float k = __fdiv_rn(f.inversion, fmaxf(FA(FM(px, px), FM(py, py)), 1e-8f));
        px = FM(px, k);
        py = FM(py, k);
    }
    px = FA(px, f.center[0]);
    py = FA(py, f.center[1]);
}

// Orbit of the escape families (Julia, Mandelbrot, Burning Ship, Phoenix):
// z <- rot * z^n + c (+ memory * previous z), planar.rs:101-130.
struct EscOrbit {
    float zx, zy, qx, qy, cx, cy, ring, stripe;
    uint32_t count;
    bool escaped;
};

static __device__ __forceinline__ void esc_init(const PlanarDev& f, float px, float py, EscOrbit& o) {
    const bool parameter_plane = f.family == 1 || f.family == 2;
    o.cx = parameter_plane ? px : f.julia[0];
    o.cy = parameter_plane ? py : f.julia[1];
    o.zx = parameter_plane ? 0.0f : px;
    o.zy = parameter_plane ? 0.0f : py;
    o.qx = o.qy = 0.0f;
    o.ring = 1e20f;
    o.stripe = 0.0f;
    o.count = 0;
    o.escaped = false;
}

// The descriptor fields the iteration reads, held in registers.
struct EscParams {
    float bail_t, trap_radius, twist_cos, twist_sin, memory, stripes;
    uint32_t iterations, power;
    int stripe_k;
    bool ship, phoenix, rotate;
};

static __device__ __forceinline__ EscParams esc_params(const PlanarDev& f) {
    EscParams p;
    p.bail_t = f.bail_t;
    p.trap_radius = f.trap_radius;
    p.twist_cos = f.twist_cos;
    p.twist_sin = f.twist_sin;
    p.memory = f.memory;
    p.stripes = f.stripes;
    p.iterations = f.iterations;
    p.power = f.power;
    p.stripe_k = f.stripe_k;
    p.ship = f.family == 2;
    p.phoenix = f.family == 5;
    p.rotate = !(f.twist_cos == 1.0f && f.twist_sin == 0.0f);
    return p;
}

// sin(k theta) for integer k from cos theta and sin theta: the Chebyshev recurrence
// s_j = 2 cos(theta) s_(j-1) - s_(j-2), s_0 = 0, s_1 = sin(theta).
static __device__ __forceinline__ float sin_multiple(float c, float s, int k) {
    float sign = 1.0f;
    if (k < 0) {
        k = -k;
        sign = -1.0f;
    }
    if (k == 0) return 0.0f;
    const float c2 = 2.0f * c;
    float a = 0.0f, b = s;
    for (int j = 1; j < k; ++j) {
        float t = fmaf(c2, b, -a);
        a = b;
        b = t;
    }
    return sign * b;
}

// sin(12 theta), the default stripe count of PlanarFractal: the recurrence unrolled.
static __device__ __forceinline__ float sin_12(float c, float s) {
    const float c2 = 2.0f * c;
    float a = 0.0f, b = s;
#pragma unroll
    for (int j = 1; j < 12; ++j) {
        float t = fmaf(c2, b, -a);
        a = b;
        b = t;
    }
    return b;
}

// One iteration; true once the orbit has escaped or spent its iteration budget.
// POW2: the power is 2 (z^2 as one complex square). SK12: the stripe count is 12.
// o.stripe accumulates sin(k theta); the bands use 0.5 n + 0.5 * that sum.
template <bool TRAPS, bool POW2, bool SK12 = false>
static __device__ __forceinline__ bool esc_step(const EscParams& p, EscOrbit& o) {
    if (o.count >= p.iterations) return true;
    float r2 = FA(FM(o.zx, o.zx), FM(o.zy, o.zy));
    if (r2 > p.bail_t) {
        o.escaped = true;
        return true;
    }
    if (TRAPS) {
        float rinv = rsqrtf(r2);
        float radius = r2 > 0.0f ? r2 * rinv : 0.0f;
        o.ring = fminf(o.ring, fabsf(radius - p.trap_radius));
        float s = 0.0f;
        if (r2 > 0.0f) {
            if (SK12) s = sin_12(o.zx * rinv, o.zy * rinv);
            else if (p.stripe_k != SF_STRIPES_GENERAL) s = sin_multiple(o.zx * rinv, o.zy * rinv, p.stripe_k);
            else s = sinf(p.stripes * atan2f(o.zy, o.zx));
        }
        o.stripe += s;
    }
    float bx = p.ship ? fabsf(o.zx) : o.zx, by = p.ship ? fabsf(o.zy) : o.zy;
    float nx, ny;
    if (POW2) cmul_rn(bx, by, bx, by, nx, ny);
    else cpow_rn(bx, by, p.power, nx, ny);
    if (p.rotate) {
        float wx = nx, wy = ny;
        cmul_rn(p.twist_cos, p.twist_sin, wx, wy, nx, ny);
    }
    nx = FA(nx, o.cx);
    ny = FA(ny, o.cy);
    if (p.phoenix) {
        nx = FA(nx, FM(o.qx, p.memory));
        ny = FA(ny, FM(o.qy, p.memory));
        o.qx = o.zx;
        o.qy = o.zy;
    }
    o.zx = nx;
    o.zy = ny;
    o.count += 1;
    return false;
}

// Smooth time, distance and traps of a finished orbit (planar.rs:173-194).
template <bool TRAPS>
static __device__ __forceinline__ void planar_finish(const PlanarDev& f, float zx, float zy, bool escaped, bool root,
                                                     uint32_t count, uint32_t measured, float smooth, float ring,
                                                     float stripe, float& dist, float* traps) {
    const float bail = f.bailout;
    float radius = fminf(len2_rn(zx, zy), 1e20f);
    escaped = escaped || radius > bail;
    float lnp = logf(float(f.power));
    if (escaped && !root) smooth = float(count) + 1.0f - logf(logf(fmaxf(radius, 1.0001f))) / lnp;
    else if (escaped) smooth = float(count);
    dist = radius / (1.0f + radius);
    traps[0] = fminf(fmaxf(smooth / float(f.iterations), 0.0f), 1.0f);
    if (TRAPS) {
        const float TAU = 6.2831855f;
        float final_angle = radius == 0.0f ? 0.5f : atan2f(zy, zx) / TAU + 0.5f;
        float bands = stripe / float(measured > 1 ? measured : 1);
        if (escaped && !root && measured > 0) {
            float angle = radius == 0.0f ? 0.0f : atan2f(zy, zx);
            float last = 0.5f + 0.5f * sinf(f.stripes * angle);
            float full = (stripe + last) / float(measured + 1);
            float t = fminf(fmaxf(1.0f + (logf(logf(bail)) - logf(logf(fmaxf(radius, 1.0001f)))) / lnp, 0.0f), 1.0f);
            bands += (full - bands) * t;
        }
        traps[1] = ring / (1.0f + ring);
        traps[2] = bands;
        traps[3] = final_angle;
    } else {
        traps[1] = traps[2] = traps[3] = 0.0f;
    }
}

template <bool TRAPS>
static __device__ __forceinline__ void planar_sample_dev(const PlanarDev& f, float ix, float iy, float& dist,
                                                         float* traps, uint32_t& iterations, uint32_t& measured_out) {
    float px, py;
    planar_map(f, ix, iy, px, py);
    const uint32_t fam = f.family;
    if (fam != 3 && fam != 4) {
        EscOrbit o;
        esc_init(f, px, py, o);
        const EscParams p = esc_params(f);
        while (!esc_step<TRAPS, false>(p, o)) {
        }
        planar_finish<TRAPS>(f, o.zx, o.zy, o.escaped, false, o.count, o.count, float(f.iterations), o.ring,
                             0.5f * float(o.count) + 0.5f * o.stripe, dist, traps);
        iterations = measured_out = o.count;
        return;
    }
    // Newton / Nova: root finding with relaxation (planar.rs:131-172)
    const float rcs = f.twist_cos, rsn = f.twist_sin;
    const float lx = FM(rcs, f.relaxation), ly = FM(rsn, f.relaxation);
    const float cx = f.julia[0], cy = f.julia[1];
    float zx = px, zy = py;
    float ring = 1e20f, stripe = 0.0f, previous_error = 1.0f;
    uint32_t count = 0, measured = 0;
    float smooth = float(f.iterations);
    bool escaped = false;
    for (uint32_t it = 0; it < f.iterations; ++it) {
        float radius = len2_rn(zx, zy);
        if (radius > f.bailout) {
            escaped = true;
            break;
        }
        if (TRAPS) {
            ring = fminf(ring, fabsf(radius - f.trap_radius));
            float angle = radius == 0.0f ? 0.0f : atan2f(zy, zx);
            stripe += 0.5f + 0.5f * sinf(f.stripes * angle);
        }
        measured += 1;
        float rx, ry;
        cpow_rn(zx, zy, f.power, rx, ry);
        rx = FS(rx, 1.0f);
        float rl2 = FA(FM(rx, rx), FM(ry, ry));
        if (fam == 3 && rl2 < 1e-12f) {
            float error = fmaxf(__fsqrt_rn(rl2), 1e-20f);
            float fraction = fminf(fmaxf(logf(1e-6f / previous_error) / logf(error / previous_error), 0.0f), 1.0f);
            smooth = count == 0 ? 0.0f : float(count) - 1.0f + fraction;
            break;
        }
        previous_error = fmaxf(__fsqrt_rn(rl2), 1e-20f);
        float ox = zx, oy = zy;
        float dx = 1.0f, dy = 0.0f;
        if (f.power > 1) cpow_rn(zx, zy, f.power - 1, dx, dy);
        dx = FM(dx, float(f.power));
        dy = FM(dy, float(f.power));
        // cdiv(residual, derivative) = residual * conj(derivative) / max(|derivative|^2, 1e-24)
        float nx, ny;
        cmul_rn(rx, ry, dx, -dy, nx, ny);
        float den = fmaxf(FA(FM(dx, dx), FM(dy, dy)), 1e-24f);
        nx = __fdiv_rn(nx, den);
        ny = __fdiv_rn(ny, den);
        float sx, sy;
        cmul_rn(lx, ly, nx, ny, sx, sy);
        zx = FS(zx, sx);
        zy = FS(zy, sy);
        if (fam == 4) {
            zx = FA(zx, cx);
            zy = FA(zy, cy);
            float ex = FS(zx, ox), ey = FS(zy, oy);
            if (FA(FM(ex, ex), FM(ey, ey)) < 1e-12f) {
                count += 1;
                smooth = float(count);
                break;
            }
        }
        count += 1;
    }
    planar_finish<TRAPS>(f, zx, zy, escaped, true, count, measured, smooth, ring, stripe, dist, traps);
    iterations = count;
    measured_out = measured;
}

__global__ void __launch_bounds__(256) k_planar(const PlanarDev* __restrict__ fg, const float* __restrict__ x,
                                                const float* __restrict__ y, size_t n, float* dist, float* traps,
                                                uint32_t* iters) {
    __shared__ PlanarDev F;
    stage_pod(F, fg);
    __syncthreads();
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float tr[4];
        uint32_t it, ms;
        float d;
        planar_sample_dev<true>(F, x[i], y[i], d, tr, it, ms);
        dist[i] = d;
        traps[i] = tr[0];
        traps[n + i] = tr[1];
        traps[2 * n + i] = tr[2];
        traps[3 * n + i] = tr[3];
        iters[i] = it;
    }
}

// Flat-canvas pixel mapping (pathtrace.wgsl:1226-1239): jittered (or centred,
// sample = 0xffffffff) uv -> p = (u - 0.5, (0.5 - v) / aspect) * 6 / zoom, rotated, + centre.
static __device__ __forceinline__ void canvas_point(const CanvasDev& K, float scale, uint32_t px, uint32_t py,
                                                    uint32_t sample, float& qx, float& qy) {
    float jx = 0.5f, jy = 0.5f;
    if (sample != 0xffffffffu) {
        uint32_t rng = rng_init(px, py, sample, K.seed);
        jx = rnd(rng);
        jy = rnd(rng);
    }
    float u = __fdiv_rn(FA(float(px), jx), float(K.width));
    float v = __fdiv_rn(FA(float(py), jy), float(K.height));
    float ax = FM(FS(u, 0.5f), scale);
    float ay = FM(__fdiv_rn(FS(0.5f, v), K.aspect), scale);
    qx = FA(K.center[0], FS(FM(K.rot_cos, ax), FM(K.rot_sin, ay)));
    qy = FA(K.center[1], FA(FM(K.rot_sin, ax), FM(K.rot_cos, ay)));
}

static __device__ __forceinline__ void store_pixel(float* dist, float* traps, uint32_t* iters, uint32_t n, uint32_t i,
                                                   float d, const float* tr, uint32_t it, bool with_traps) {
    dist[i] = d;
    traps[i] = tr[0];
    if (with_traps) {
        traps[n + i] = tr[1];
        traps[2 * n + i] = tr[2];
        traps[3 * n + i] = tr[3];
    }
    iters[i] = it;
}

// One tile of the canvas, Newton and Nova: one pixel per thread (grid-stride).
template <bool TRAPS>
__global__ void __launch_bounds__(256) k_escape2d_root(const PlanarDev* __restrict__ fg,
                                                       const CanvasDev* __restrict__ cg, uint32_t tile_x,
                                                       uint32_t tile_y, uint32_t tile_w, uint32_t tile_h,
                                                       uint32_t sample, float* dist, float* traps, uint32_t* iters,
                                                       unsigned long long* stats) {
    __shared__ PlanarDev F;
    __shared__ CanvasDev K;
    stage_pod(F, fg);
    stage_pod(K, cg);
    __syncthreads();
    const uint32_t n = tile_w * tile_h;
    unsigned long long total_iters = 0;
    const float scale = __fdiv_rn(6.0f, K.zoom);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float qx, qy, tr[4], d;
        canvas_point(K, scale, tile_x + i % tile_w, tile_y + i / tile_w, sample, qx, qy);
        uint32_t it, ms;
        planar_sample_dev<TRAPS>(F, qx, qy, d, tr, it, ms);
        store_pixel(dist, traps, iters, n, i, d, tr, it, TRAPS);
        total_iters += ms;
    }
    warp_stat(&stats[SF_STAT_DE_ITERS], total_iters);
}

// One tile of the canvas, escape families: each lane owns one pixel at a time and
// takes the next pixel of the tile (warp-aggregated atomic on *work, which starts at
// 0) as soon as its orbit ends, checking every ESC_CHUNK iterations, so lanes whose
// pixels escape early do not idle beside interior pixels that run the whole budget.
// Without TRAPS only dist, traps[0 .. n) (smooth time) and iters are written.
constexpr int ESC_CHUNK = 16;

// Up to ESC_CHUNK iterations; true once the orbit has ended.
template <bool TRAPS, bool POW2, bool SK12>
static __device__ __forceinline__ bool esc_chunk(const EscParams& p, EscOrbit& o) {
    for (int j = 0; j < ESC_CHUNK; ++j)
        if (esc_step<TRAPS, POW2, SK12>(p, o)) return true;
    return false;
}

// The common tile: z^2 without twist (Julia, Mandelbrot or, SHIP, Burning Ship), the
// default 12 stripes. The budget is checked once per chunk instead of per iteration.
// The orbit's arithmetic rounds as esc_step's, bit for bit, with fewer instructions:
// the squares x*x, y*y of |z|^2 serve the new real part (|x|*|x| = x*x exactly), the
// imaginary part is fl(x*y) doubled (fl(x*y) + fl(y*x) = 2 fl(x*y), and
// fl(|x|*|y|) = |fl(x*y)|), and the paired products and the sum with c are packed
// f32x2 operations, each lane rounded as a binary32 multiply or add.
template <bool TRAPS, bool SHIP>
static __device__ __forceinline__ bool esc_chunk_z2(const EscParams& p, EscOrbit& o) {
    const uint32_t left = p.iterations - o.count;  // count <= iterations
    const int n = left < (uint32_t)ESC_CHUNK ? (int)left : ESC_CHUNK;
    float zx = o.zx, zy = o.zy, ring = o.ring, stripe = o.stripe;
    const float cx = o.cx, cy = o.cy, bt = p.bail_t, tr = p.trap_radius;
    int j = 0;
    bool escaped = false;
    for (; j < n; ++j) {
        const float2 sq = mul2(zx, zy, zx, zy);  // (x*x, y*y)
        const float r2 = FA(sq.x, sq.y);
        if (r2 > bt) {
            escaped = true;
            break;
        }
        if (TRAPS) {
            const float rinv = rsqrtf(r2);
            ring = fminf(ring, fabsf((r2 > 0.0f ? r2 * rinv : 0.0f) - tr));
            if (r2 > 0.0f) {
                const float2 u = mul2(zx, zy, rinv, rinv);  // z / |z|
                stripe += sin_12(u.x, u.y);
            }
        }
        const float m = FM(zx, zy);
        const float mm = SHIP ? fabsf(m) : m;
        const float2 z = add2(FS(sq.x, sq.y), FA(mm, mm), cx, cy);
        zx = z.x;
        zy = z.y;
    }
    o.zx = zx;
    o.zy = zy;
    o.ring = ring;
    o.stripe = stripe;
    o.count += (uint32_t)j;
    o.escaped = escaped;
    return escaped || o.count >= p.iterations;
}

template <bool TRAPS>
__global__ void __launch_bounds__(256, 5) k_escape2d(const PlanarDev* __restrict__ fg,
                                                     const CanvasDev* __restrict__ cg, uint32_t tile_x,
                                                     uint32_t tile_y, uint32_t tile_w, uint32_t tile_h,
                                                     uint32_t sample, float* dist, float* traps, uint32_t* iters,
                                                     unsigned long long* stats, uint32_t* work) {
    __shared__ PlanarDev F;
    __shared__ CanvasDev K;
    stage_pod(F, fg);
    stage_pod(K, cg);
    __syncthreads();
    const uint32_t n = tile_w * tile_h;
    unsigned long long total_iters = 0;
    const float scale = __fdiv_rn(6.0f, K.zoom);
    const EscParams p = esc_params(F);
    const bool pow2 = p.power == 2, sk12 = p.stripe_k == 12;
    const bool z2 = pow2 && sk12 && !p.rotate && !p.phoenix;
    EscOrbit o;
    uint32_t pix = 0;
    bool busy = false, live = true;
    for (;;) {
        // every lane of the warp reaches this point together
        bool want = live && !busy;
        uint32_t got = warp_fetch(work, want);
        if (want) {
            if (got < n) {
                pix = got;
                float px, py, qx, qy;
                canvas_point(K, scale, tile_x + pix % tile_w, tile_y + pix / tile_w, sample, qx, qy);
                planar_map(F, qx, qy, px, py);
                esc_init(F, px, py, o);
                busy = true;
            } else {
                live = false;
            }
        }
        if (!__any_sync(FULL_MASK, busy)) break;
        if (busy) {
            bool done;
            if (z2 && p.ship) done = esc_chunk_z2<TRAPS, true>(p, o);
            else if (z2) done = esc_chunk_z2<TRAPS, false>(p, o);
            else if (pow2 && sk12) done = esc_chunk<TRAPS, true, true>(p, o);
            else if (pow2) done = esc_chunk<TRAPS, true, false>(p, o);
            else done = esc_chunk<TRAPS, false, false>(p, o);
            if (done) {
                float tr[4], d;
                planar_finish<TRAPS>(F, o.zx, o.zy, o.escaped, false, o.count, o.count, float(F.iterations), o.ring,
                                     0.5f * float(o.count) + 0.5f * o.stripe, d, tr);
                store_pixel(dist, traps, iters, n, pix, d, tr, o.count, TRAPS);
                total_iters += o.count;
                busy = false;
            }
        }
    }
    warp_stat(&stats[SF_STAT_DE_ITERS], total_iters);
}

static unsigned escape_grid(size_t n, unsigned per_sm) {
    size_t want = (n + 255) / 256;
    size_t cap = (size_t)sf_device_sm_count() * per_sm;
    if (want > cap) want = cap;
    return (unsigned)(want ? want : 1);
}

cudaError_t sf_launch_planar(const PlanarDev* f, const float* x, const float* y, size_t n, float* dist, float* traps,
                             uint32_t* iters, cudaStream_t st) {
    if (!n) return cudaSuccess;
    k_planar<<<escape_grid(n, 8), 256, 0, st>>>(f, x, y, n, dist, traps, iters);
    return cudaGetLastError();
}

cudaError_t sf_launch_escape2d(const PlanarDev* f, const CanvasDev* canvas, uint32_t tile_x, uint32_t tile_y,
                               uint32_t tile_w, uint32_t tile_h, uint32_t sample, float* dist, float* traps,
                               uint32_t* iters, unsigned long long* stats, uint32_t* work, int with_traps, int root,
                               cudaStream_t st) {
    size_t n = (size_t)tile_w * tile_h;
    if (!n) return cudaSuccess;
    if (root && with_traps)
        k_escape2d_root<true><<<escape_grid(n, 8), 256, 0, st>>>(f, canvas, tile_x, tile_y, tile_w, tile_h, sample,
                                                                  dist, traps, iters, stats);
    else if (root)
        k_escape2d_root<false><<<escape_grid(n, 8), 256, 0, st>>>(f, canvas, tile_x, tile_y, tile_w, tile_h, sample,
                                                                   dist, traps, iters, stats);
    else if (with_traps)
        k_escape2d<true><<<escape_grid(n, 5), 256, 0, st>>>(f, canvas, tile_x, tile_y, tile_w, tile_h, sample, dist,
                                                             traps, iters, stats, work);
    else
        k_escape2d<false><<<escape_grid(n, 5), 256, 0, st>>>(f, canvas, tile_x, tile_y, tile_w, tile_h, sample, dist,
                                                              traps, iters, stats, work);
    return cudaGetLastError();
}

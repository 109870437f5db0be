// TEST INFRASTRUCTURE -- NOT THE PRODUCT.
// C entry points of the CPU oracle (oracle_core.*), loaded with ctypes by the
// tests, the smoke check and the CPU-baseline leg of the benchmark. Every
// function takes a thread count; work is split in contiguous chunks.
#include <algorithm>
#include <atomic>
#include <thread>

#include "oracle_core.hpp"

#if defined(__x86_64__) || defined(__i386__)
typedef __float128 real128;  // IEEE binary128 (software arithmetic)
#else
typedef long double real128;  // IEEE binary128 on aarch64
#endif

using namespace orc;

template <class F> static void parallel_for(size_t n, int threads, F&& f) {
    if (threads <= 1 || n < 2) {
        for (size_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<size_t> next{0};
    const size_t chunk = 16;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&]() {
            for (;;) {
                size_t s = next.fetch_add(chunk);
                if (s >= n) break;
                size_t e = std::min(n, s + chunk);
                for (size_t i = s; i < e; ++i) f(i);
            }
        });
    for (auto& th : pool) th.join();
}

// Primary rays through pixel centres (control.wgsl:270-273), march (pathtrace.wgsl:78-145)
// with the absolute (rule 1) or cone-relative (rule 0) hit test, then a 6-tap central
// (normal_mode 0) or 4-tap tetrahedral (normal_mode 1) normal with
// h = max(t * pixel_cone * 0.5, 1e-4) * tolerance.
template <class R>
static void primary_one(const Graph& g, const sf_camera& cam, uint32_t w, uint32_t h, uint32_t idx, uint32_t max_steps,
                        int rule, double eps, double t_far, double tol, int normal_mode, double* t_out,
                        uint32_t* steps_out, double* n_out, uint64_t* evals) {
    uint32_t px = idx % w, py = idx / w;
    R ndcx = ((R(float(px)) + R(0.5)) / R(float(w))) * R(2) - R(1);
    R ndcy = ((R(float(py)) + R(0.5)) / R(float(h))) * R(2) - R(1);
    V3<R> fw(cam.forward[0], cam.forward[1], cam.forward[2]);
    V3<R> rt(cam.right[0], cam.right[1], cam.right[2]);
    V3<R> up(cam.up[0], cam.up[1], cam.up[2]);
    V3<R> ro(cam.origin[0], cam.origin[1], cam.origin[2]);
    R th = R(cam.tan_half_fov), asp = R(cam.aspect);
    V3<R> rd = normalize(fw + rt * (ndcx * th) + up * (-ndcy * th / asp));
    R cone = th * R(2) / R(float(w));
    Hit<R> hit = march_segment(g, ro, rd, R(g.step_scale), cone * R(tol), R(t_far), max_steps, rule == 1, R(eps), evals);
    steps_out[idx] = hit.steps;
    if (!hit.hit) {
        t_out[idx] = -1.0;
        n_out[3 * idx] = n_out[3 * idx + 1] = n_out[3 * idx + 2] = 0.0;
        return;
    }
    t_out[idx] = double(hit.t);
    R hh = r_max(hit.t * cone * R(0.5), R(1e-4)) * R(tol);
    V3<R> p = ro + rd * hit.t;
    V3<R> n = normal_mode == 0 ? normal_central(g, p, hh) : normal_tetra(g, p, hh);
    *evals += normal_mode == 0 ? 6 : 4;
    n_out[3 * idx] = n.x;
    n_out[3 * idx + 1] = n.y;
    n_out[3 * idx + 2] = n.z;
}

// Film planes of main (pathtrace.wgsl:1243-1266) over `samples` samples from
// sample_start, each pixel's planes starting at zero: volume (sums, count), its
// Welford moments (sums of max(0, delta * (v - new_mean)), count) and surface
// (sums of radiance - volume, count), accumulated in the oracle's precision.
template <class R> struct FilmAcc {
    R acc[3] = {0, 0, 0}, vol[4] = {0, 0, 0, 0}, mom[4] = {0, 0, 0, 0}, surf[4] = {0, 0, 0, 0};
    void add(const PixelResult& r) {
        for (int c = 0; c < 3; ++c) acc[c] += R(r.L[c]);
        const R n = vol[3];
        for (int c = 0; c < 3; ++c) {
            const R v = R(r.V[c]);
            const R old_mean = vol[c] / std::max(n, R(1));
            const R delta = v - old_mean;
            const R new_mean = old_mean + delta / (n + R(1));
            mom[c] += std::max(R(0), delta * (v - new_mean));
            vol[c] += v;
            surf[c] += R(r.L[c]) - v;
        }
        vol[3] += R(1);
        mom[3] += R(1);
        surf[3] += R(1);
    }
};

extern "C" {

void* or_graph_new(const sf_graph_desc* d) {
    if (!d) return nullptr;
    Graph* g = new Graph();
    g->nodes.assign(d->nodes, d->nodes + d->node_count);
    g->links.assign(d->links, d->links + d->link_count);
    if (d->body_ids && d->body_id_count) g->body.assign(d->body_ids, d->body_ids + d->body_id_count);
    if (d->placements && d->placement_count) g->placements.assign(d->placements, d->placements + d->placement_count);
    g->safety = d->safety;
    g->hint = d->bounding_radius_hint;
    if (!prepare(*g)) { delete g; return nullptr; }
    return g;
}

void or_graph_free(void* g) { delete static_cast<Graph*>(g); }

// A panorama's tables, registered under the key scenes carry in their environment field;
// writes w*h*4 floats into texels when not NULL.
int or_panorama(uint64_t key, const float* rgb, uint32_t width, uint32_t height, float* texels, uint32_t* w,
                uint32_t* h) {
    Panorama p;
    if (!panorama_tables(rgb, width, height, p)) return 0;
    if (w) *w = p.w;
    if (h) *h = p.h;
    if (texels) std::memcpy(texels, p.texels.data(), p.texels.size() * sizeof(float));
    if (key) panorama_register(key, p);
    return 1;
}

// The fence hierarchy of `count` placements: 8 floats per node (centre, half, escape,
// placement or -1) into out (2 * count - 1 nodes).
void or_bvh_build(const sf_placement* pl, uint32_t count, const float* half, float* out) {
    auto nodes = bvh_build(pl, count, half);
    for (size_t i = 0; i < nodes.size(); ++i) {
        for (int k = 0; k < 3; ++k) {
            out[8 * i + k] = nodes[i].center[k];
            out[8 * i + 3 + k] = nodes[i].half[k];
        }
        out[8 * i + 6] = float(nodes[i].escape);
        out[8 * i + 7] = float(nodes[i].placement);
    }
}

void or_graph_info(void* gp, float* step_scale, float* lipschitz, float* trap_scales, uint32_t* iteration_product) {
    Graph* g = static_cast<Graph*>(gp);
    *step_scale = g->step_scale;
    *lipschitz = g->lipschitz;
    for (int i = 0; i < 4; ++i) trap_scales[i] = g->trap_scales[i];
    *iteration_product = g->iteration_product;
}

// DE at n points (xyz interleaved). precision 32 = reference f32, 64 = oracle f64.
void or_de_eval(void* gp, int precision, const double* xyz, size_t n, double* dist, double* traps,
                uint32_t* iters, uint32_t* mats, int threads) {
    const Graph& g = *static_cast<Graph*>(gp);
    parallel_for(n, threads, [&](size_t i) {
        if (precision == 32) {
            auto s = evaluate<float>(g, V3<float>(float(xyz[3 * i]), float(xyz[3 * i + 1]), float(xyz[3 * i + 2])));
            dist[i] = s.distance;
            for (int k = 0; k < 4; ++k) traps[4 * i + k] = s.traps[k];
            iters[i] = s.iterations;
            mats[i] = s.material;
        } else {
            auto s = evaluate<double>(g, V3<double>(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]));
            dist[i] = s.distance;
            for (int k = 0; k < 4; ++k) traps[4 * i + k] = s.traps[k];
            iters[i] = s.iterations;
            mats[i] = s.material;
        }
    });
}

// The exact sample through the union search (graph_wgsl.rs:1112-1154), as or_de_eval.
// exact_leaves[i]: the leaves point i evaluated exactly after the probes.
void or_de_eval_search(void* gp, int precision, const double* xyz, size_t n, double* dist, double* traps,
                       uint32_t* iters, uint32_t* mats, uint32_t* exact_leaves, int threads) {
    const Graph& g = *static_cast<Graph*>(gp);
    parallel_for(n, threads, [&](size_t i) {
        exact_leaves[i] = 0;
        if (precision == 32) {
            auto s = evaluate_union_search<float>(
                g, V3<float>(float(xyz[3 * i]), float(xyz[3 * i + 1]), float(xyz[3 * i + 2])), &exact_leaves[i]);
            dist[i] = s.distance;
            for (int k = 0; k < 4; ++k) traps[4 * i + k] = s.traps[k];
            iters[i] = s.iterations;
            mats[i] = s.material;
        } else {
            auto s = evaluate_union_search<double>(g, V3<double>(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]),
                                                   &exact_leaves[i]);
            dist[i] = s.distance;
            for (int k = 0; k < 4; ++k) traps[4 * i + k] = s.traps[k];
            iters[i] = s.iterations;
            mats[i] = s.material;
        }
    });
}
// The union search's leaves (union_leaves, graph_wgsl.rs:18-26) and whether the graph
// has a skippable Bounded or Instances node.
uint32_t or_union_leaves(void* gp, uint32_t* any_fast) {
    const Graph& g = *static_cast<Graph*>(gp);
    *any_fast = g.fast_bounds.empty() ? 0u : 1u;
    return uint32_t(g.union_leaves.size());
}

// The GPU's fast sample (de_sample, graph_wgsl.rs:800-814): distance and flags.
void or_de_eval_fast(void* gp, int precision, const double* xyz, size_t n, double* dist, uint32_t* flags,
                     int threads) {
    const Graph& g = *static_cast<Graph*>(gp);
    parallel_for(n, threads, [&](size_t i) {
        if (precision == 32) {
            auto s = evaluate<float>(g, V3<float>(float(xyz[3 * i]), float(xyz[3 * i + 1]), float(xyz[3 * i + 2])),
                                     true);
            dist[i] = s.distance;
            flags[i] = s.flags;
        } else {
            auto s = evaluate<double>(g, V3<double>(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]), true);
            dist[i] = s.distance;
            flags[i] = s.flags;
        }
    });
}

uint64_t or_primary(void* gp, int precision, const sf_camera* cam, uint32_t w, uint32_t h, uint32_t first,
                    uint32_t count, uint32_t max_steps, int rule, double eps, double t_far, double tol,
                    int normal_mode, double* t_out, uint32_t* steps_out, double* n_out, int threads) {
    const Graph& g = *static_cast<Graph*>(gp);
    std::atomic<uint64_t> total{0};
    parallel_for(count, threads, [&](size_t i) {
        uint64_t ev = 0;
        uint32_t idx = first + uint32_t(i);
        if (precision == 32)
            primary_one<float>(g, *cam, w, h, idx, max_steps, rule, eps, t_far, tol, normal_mode, t_out, steps_out, n_out, &ev);
        else
            primary_one<double>(g, *cam, w, h, idx, max_steps, rule, eps, t_far, tol, normal_mode, t_out, steps_out, n_out, &ev);
        total += ev;
    });
    return total.load();
}

// Path-traced film for a list of pixels: per pixel, samples [sample_start, sample_start+samples)
// are added in ascending order into an accumulator of the working precision (the
// reference's accum += (L, 1), pathtrace.wgsl:1243-1245 / wavefront.wgsl:240).
// depth/aux come from sample 0 when sample_start == 0. Returns the number of traced segments.
uint64_t or_render(void* gp, int precision, const sf_scene_desc* scene, const sf_render_config* cfg,
                   const uint32_t* pixels, size_t n, uint32_t sample_start, uint32_t samples, double* accum,
                   double* depth, double* aux, uint64_t* de_evals, int threads, double* volume, double* moments,
                   double* surface) {
    const Graph& g = *static_cast<Graph*>(gp);
    std::atomic<uint64_t> segs{0}, evals{0};
    Scene<float> s32;
    Scene<double> s64;
    if (precision == 32) s32 = make_scene<float>(g, *scene, *cfg);
    else s64 = make_scene<double>(g, *scene, *cfg);
    parallel_for(n, threads, [&](size_t i) {
        uint32_t px = pixels[2 * i], py = pixels[2 * i + 1];
        FilmAcc<float> af;
        FilmAcc<double> ad;
        uint64_t sg = 0, ev = 0;
        for (uint32_t k = 0; k < samples; ++k) {
            uint32_t sample = sample_start + k;
            PixelResult r = precision == 32 ? radiance<float>(g, s32, px, py, sample) : radiance<double>(g, s64, px, py, sample);
            sg += r.segments;
            ev += r.de_evals;
            if (precision == 32) af.add(r);
            else ad.add(r);
            if (sample == 0) {
                depth[i] = r.depth;
                for (int c = 0; c < 4; ++c) aux[4 * i + c] = r.aux[c];
            }
        }
        for (int c = 0; c < 4; ++c) {
            if (c < 3) accum[3 * i + c] = precision == 32 ? double(af.acc[c]) : ad.acc[c];
            if (volume) volume[4 * i + c] = precision == 32 ? double(af.vol[c]) : ad.vol[c];
            if (moments) moments[4 * i + c] = precision == 32 ? double(af.mom[c]) : ad.mom[c];
            if (surface) surface[4 * i + c] = precision == 32 ? double(af.surf[c]) : ad.surf[c];
        }
        segs += sg;
        evals += ev;
    });
    if (de_evals) *de_evals = evals.load();
    return segs.load();
}

// Escape-time sample at n plane points (xy interleaved); outputs DeSample fields.
void or_planar(int precision, const PlanarParams* f, const double* xy, size_t n, double* dist, double* traps,
               uint32_t* iters, int threads) {
    parallel_for(n, threads, [&](size_t i) {
        if (precision == 32) {
            auto s = planar_sample<float>(*f, V2<float>(float(xy[2 * i]), float(xy[2 * i + 1])));
            dist[i] = s.distance;
            for (int k = 0; k < 4; ++k) traps[4 * i + k] = s.traps[k];
            iters[i] = s.iterations;
        } else {
            auto s = planar_sample<double>(*f, V2<double>(xy[2 * i], xy[2 * i + 1]));
            dist[i] = s.distance;
            for (int k = 0; k < 4; ++k) traps[4 * i + k] = s.traps[k];
            iters[i] = s.iterations;
        }
    });
}

// Direct Mandelbrot escape count z <- z^2 + c, escape when |z|^2 > bailout^2.
// c = center + offset, with center given as a double-double (hi + lo) and the
// offsets as doubles. precision 64: double; 128: IEEE binary128 (the deep-zoom
// truth). Also returns |z|^2 at escape (as double) for smooth colouring.
// Reference orbit Z_0 = 0, Z_(n+1) = Z_n^2 + c_ref of c_ref = (cx, cy) in binary128
// (precision 128) or binary64, through the first n with |Z_n| > bailout or n = max_iter,
// as the perturbation kernel reads it: four floats per entry (Re hi, Im hi, Re lo,
// Im lo) with hi = float(Z_n) and lo = float(Z_n - hi). Returns the entry count.
uint32_t or_mandel_orbit(int precision, double cx, double cy, uint32_t max_iter, double bailout, float* out) {
    auto run = [&](auto zero) {
        using T = decltype(zero);
        const T x0 = T(cx), y0 = T(cy), b2 = T(bailout) * T(bailout);
        T zx = 0, zy = 0;
        uint32_t n = 0;
        for (;;) {
            const float hx = float(zx), hy = float(zy);
            out[4 * n] = hx;
            out[4 * n + 1] = hy;
            out[4 * n + 2] = float(zx - T(hx));
            out[4 * n + 3] = float(zy - T(hy));
            const T x2 = zx * zx, y2 = zy * zy;
            if (n >= max_iter || x2 + y2 > b2) break;
            const T nx = (x2 - y2) + x0;
            zy = (T(2) * zx) * zy + y0;
            zx = nx;
            ++n;
        }
        return n + 1;
    };
    return precision == 128 ? run(real128(0)) : run(double(0));
}

void or_mandel_escape(int precision, const double* center_hi, const double* center_lo, const double* offsets,
                      size_t n, uint32_t max_iter, double bailout, uint32_t* iters, double* mag2, int threads) {
    parallel_for(n, threads, [&](size_t i) {
        if (precision == 64) {
            double cx = (center_hi[0] + center_lo[0]) + offsets[2 * i];
            double cy = (center_hi[1] + center_lo[1]) + offsets[2 * i + 1];
            double zx = 0, zy = 0, b2 = bailout * bailout;
            uint32_t k = 0;
            double m = 0;
            for (; k < max_iter; ++k) {
                double x2 = zx * zx, y2 = zy * zy;
                m = x2 + y2;
                if (m > b2) break;
                double nx = x2 - y2 + cx;
                zy = 2.0 * zx * zy + cy;
                zx = nx;
            }
            if (k == max_iter) m = zx * zx + zy * zy;
            iters[i] = k;
            mag2[i] = m;
        } else {
            real128 cx = ((real128)center_hi[0] + (real128)center_lo[0]) + (real128)offsets[2 * i];
            real128 cy = ((real128)center_hi[1] + (real128)center_lo[1]) + (real128)offsets[2 * i + 1];
            real128 zx = 0, zy = 0, b2 = (real128)bailout * (real128)bailout;
            uint32_t k = 0;
            real128 m = 0;
            for (; k < max_iter; ++k) {
                real128 x2 = zx * zx, y2 = zy * zy;
                m = x2 + y2;
                if (m > b2) break;
                real128 nx = x2 - y2 + cx;
                zy = 2 * zx * zy + cy;
                zx = nx;
            }
            if (k == max_iter) m = zx * zx + zy * zy;
            iters[i] = k;
            mag2[i] = (double)m;
        }
    });
}

// Escape label for the deep-zoom centre search: 1 if c escapes within max_iter.
int or_mandel_escapes(int precision, double cx_hi, double cx_lo, double cy_hi, double cy_lo, uint32_t max_iter) {
    double off[2] = {0, 0};
    double hi[2] = {cx_hi, cy_hi}, lo[2] = {cx_lo, cy_lo};
    uint32_t it;
    double m;
    or_mandel_escape(precision, hi, lo, off, 1, max_iter, 2.0, &it, &m, 1);
    return it < max_iter ? 1 : 0;
}

// The scene's texture value (pattern_value) at n points; sf_texture.graph carries an
// oracle graph handle.
void or_texture_values(const sf_scene_desc* scene, int precision, const double* xyz, size_t n, double* out) {
    sf_render_config cfg{};
    cfg.width = cfg.height = 1;
    const Graph& tg = *reinterpret_cast<const Graph*>(scene->texture.graph);
    if (precision == 32) {
        const Scene<float> s = make_scene<float>(tg, *scene, cfg);
        for (size_t i = 0; i < n; ++i)
            out[i] = texture_value_at<float>(s, V3<float>(float(xyz[3 * i]), float(xyz[3 * i + 1]), float(xyz[3 * i + 2])));
    } else {
        const Scene<double> s = make_scene<double>(tg, *scene, cfg);
        for (size_t i = 0; i < n; ++i) out[i] = texture_value_at<double>(s, V3<double>(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]));
    }
}

}  // extern "C"

// Wavefront stage bodies shared by the single-job kernels (sf_kernels.cu) and the
// batched multi-job kernels (sf_batch.cu).
#pragma once
#include "sf_kernels.cuh"
#include "sf_trace.cuh"
#include "sf_warp.cuh"

static __device__ __forceinline__ void path_pixel(const DispatchGeom& g, uint32_t path, uint32_t& px, uint32_t& py,
                                                  uint32_t& sample) {
    uint32_t tile_px = g.tile_w * g.tile_h;
    uint32_t local = path % tile_px;
    sample = g.sample_start + path / tile_px;
    px = g.tile_x + local % g.tile_w;
    py = g.tile_y + local / g.tile_w;
}

template <int FEAT = 0>
static __device__ __forceinline__ void store_path(PathSoA& soa, uint32_t path, const PathState& ps, uint32_t flags) {
    soa.o[path] = make_float4(ps.o.x, ps.o.y, ps.o.z, ps.prev_pdf);
    soa.d[path] = make_float4(ps.d.x, ps.d.y, ps.d.z, ps.prev_area_total);
    soa.tp[path] = make_float4(ps.tp.x, ps.tp.y, ps.tp.z, __uint_as_float(ps.rng));
    uint32_t f = flags | (ps.prev_from_bsdf ? SF_PF_FROM_BSDF : 0u) | (ps.prev_from_volume ? SF_PF_FROM_VOLUME : 0u);
    soa.L[path] = make_float4(ps.L.x, ps.L.y, ps.L.z, __uint_as_float(ps.bounce | (f << 16)));
    soa.pn[path] = make_float4(ps.prev_normal.x, ps.prev_normal.y, ps.prev_normal.z, 0.f);
    if ((FEAT & SF_FEAT_RICH) && soa.ex) {
        const float4 e = soa.ex[path];  // keeps a pending initial-medium flag (set by generate)
        const uint32_t keep = __float_as_uint(e.z) & SF_EX_INIT;
        soa.ex[path] = make_float4(ps.tex_width, ps.tex_spread,
                                   __uint_as_float(ps.medium_slot | (ps.solid_medium ? SF_EX_SOLID : 0u) | keep),
                                   __uint_as_float(ps.null_surfaces));
    }
}
template <int FEAT = 0>
static __device__ __forceinline__ uint32_t load_path(const PathSoA& soa, uint32_t path, PathState& ps) {
    float4 o = soa.o[path], d = soa.d[path], tp = soa.tp[path], L = soa.L[path], pn = soa.pn[path];
    ps.o = mk3(o.x, o.y, o.z);
    ps.prev_pdf = o.w;
    ps.d = mk3(d.x, d.y, d.z);
    ps.prev_area_total = d.w;
    ps.tp = mk3(tp.x, tp.y, tp.z);
    ps.rng = __float_as_uint(tp.w);
    ps.L = mk3(L.x, L.y, L.z);
    uint32_t bits = __float_as_uint(L.w);
    ps.bounce = bits & 0xffffu;
    uint32_t flags = bits >> 16;
    ps.prev_from_bsdf = (flags & SF_PF_FROM_BSDF) != 0;
    ps.prev_from_volume = (flags & SF_PF_FROM_VOLUME) != 0;
    ps.prev_normal = mk3(pn.x, pn.y, pn.z);
    ps.tex_width = 0.0f;
    ps.tex_spread = 0.0f;
    ps.solid_medium = false;
    ps.medium_slot = 0;
    ps.null_surfaces = 0;
    if ((FEAT & SF_FEAT_RICH) && soa.ex) {
        const float4 e = soa.ex[path];
        ps.tex_width = e.x;
        ps.tex_spread = e.y;
        const uint32_t m = __float_as_uint(e.z);
        ps.medium_slot = m & 0xffu;
        ps.solid_medium = (m & SF_EX_SOLID) != 0u;
        ps.null_surfaces = __float_as_uint(e.w);
    }
    return flags;
}

// A segment's march state at its start -- the nearest emitter on the ray
// (lights.wgsl:183-209) bounds it, then march_begin's fields -- written to the path's
// continuation row (row = path) or shadow row (row = path + capacity) by the stage
// that creates the ray, so the trace kernel only loads it.
static __device__ __forceinline__ void begin_segment(const DevScene& S, PathSoA& soa, uint32_t row, float3 ro,
                                                     float3 rd, float t_end) {
    uint32_t li;
    const float te = nearest_emitter(S, ro, rd, t_end, li);
    soa.m0[row] = make_float4(0.0f, 1.2f, 0.0f, 0.0f);    // t, omega, previous radius, step
    soa.m1[row] = make_float4(te, 0.0f, 1e30f, 0.0f);     // t_end, candidate t, candidate error, steps (0)
    soa.m2[row] = li;
}

// wf_generate (wavefront.wgsl:160-179) for one path: camera ray and RNG.
// `local` indexes the path within its job (g), `path` its row in the SoA.
static __device__ __forceinline__ void generate_path(const DevScene& S, PathSoA& soa, const DispatchGeom& g,
                                                     uint32_t local, uint32_t path) {
    uint32_t px, py, sample;
    path_pixel(g, local, px, py, sample);
    PathState ps;
    path_begin(S, ps, px, py, sample);
    if (soa.ex)  // the camera's footprint; the trace kernel samples the initial medium of optics scenes first
        soa.ex[path] = make_float4(ps.tex_width, ps.tex_spread,
                                   __uint_as_float((S.rich & SF_RICH_OPTICS) ? SF_EX_INIT : 0u), 0.f);
    store_path(soa, path, ps, SF_PF_CONT);
    if (soa.pv) soa.pv[path] = make_float4(0.f, 0.f, 0.f, 0.f);
    begin_segment(S, soa, path, ps.o, ps.d, S.extent);
}

// wf_shade + wf_compact (wavefront.wgsl:196-223) for one path: resolve last round's
// shadow segment, run the bounce body on this round's hit, return the next flags.
template <int FEAT = 0>
static __device__ __forceinline__ uint32_t shade_path(const DevScene& S, PathSoA& soa, const DispatchGeom& g,
                                                      const FilmPlanes& film, uint32_t local, uint32_t path,
                                                      uint32_t* status, int final_round) {
    PathState ps;
    // The hit record is read with the path state, one round trip rather than one more
    // after the flags (every path owns the row; a path without a hit this round ignores
    // it). The traps and normal stay behind the hit test: read up front as well, they
    // made the shading kernels slower, 15.90 against 15.78 ms per 64-spp frame.
    const uint4 hr = soa.hit[path];
    uint32_t flags = load_path<FEAT>(soa, path, ps);
    const size_t cap = soa.capacity;
    // the volume layer split (fog scenes): the camera segment's in-scattered light and
    // the volume tags of last round's shadow slots
    uint32_t vbits = 0;
    ps.pv = mk3(0.f, 0.f, 0.f);
    ps.volume_path = false;
    if (soa.pv) {
        const float4 v = soa.pv[path];
        ps.pv = mk3(v.x, v.y, v.z);
        vbits = __float_as_uint(v.w);
        ps.volume_path = (vbits >> 8) & 1u;
    }
    if (flags & SF_PF_SHADOW) {  // last round's shadow segments, in slot order
        const uint32_t mask = (flags >> SF_PF_SHADOW_SHIFT) & 0xffu;
        for (uint32_t k = 0; k < soa.shadow_slots; ++k) {
            const size_t row = k * cap + path;
            if (!((mask >> k) & 1u)) continue;
            const float4 c4 = soa.sh_c[row];  // read beside the visibility, not after it
            if (soa.vis[row]) {
                float3 c = mk3(c4.x, c4.y, c4.z);
                if ((FEAT & SF_FEAT_RICH) && (S.rich & SF_RICH_OPTICS))
                    c = c * soa.sh_d[row].w;  // the coverage of crossed surfaces
                ps.L = add_rn(ps.L, c);
                if ((vbits >> k) & 1u) ps.pv = add_rn(ps.pv, c);
            }
        }
    }
    uint32_t vmask = 0;  // volume tags of this bounce's shadow slots
    uint32_t nf = 0;
    if (flags & SF_PF_CONT) {
        HitInfo h;
        h.t = __uint_as_float(hr.x);
        h.steps = hr.y;
        h.light_index = hr.z;
        h.hit = (hr.w & SF_HF_HIT) != 0;
        h.exhausted = (hr.w & SF_HF_EXHAUSTED) != 0;
        if (h.hit && h.light_index == SF_NO_LIGHT) {
            const float4 tr = soa.hit_tr[path], hn = soa.hit_n[path];
            h.sample.traps[0] = tr.x; h.sample.traps[1] = tr.y; h.sample.traps[2] = tr.z; h.sample.traps[3] = tr.w;
            uint32_t im = __float_as_uint(hn.w);
            h.sample.iter = im & 0xffffu;
            h.sample.material = im >> 16;
            h.sample.d = 0.f;
            h.n = mk3(hn.x, hn.y, hn.z);
        }
        uint32_t px, py, sample;
        path_pixel(g, local, px, py, sample);
        float* fd = nullptr;
        float4* fa = nullptr;
        if (sample == 0 && ps.bounce == 0) {
            const size_t idx = film_index(film, px, py);
            fd = film.depth + idx;
            fa = film.aux + idx;
        }
        uint32_t n_sh = 0, sh_mask = 0;
        auto emit = [&](const ShadowReq& sh) {  // the k-th shadow segment of this bounce
            if (n_sh >= soa.shadow_slots) {  // more segments than the arena's slots: a host sizing error
                atomicOr(status, SF_WF_SHADOW_OVERFLOW);
                return;
            }
            const size_t row = n_sh * cap + path;
            soa.sh_o[row] = make_float4(sh.o.x, sh.o.y, sh.o.z, sh.t_end);
            soa.sh_d[row] = make_float4(sh.dir.x, sh.dir.y, sh.dir.z, 1.f);  // w: visibility weight
            soa.sh_c[row] = make_float4(sh.contrib.x, sh.contrib.y, sh.contrib.z, 0.f);
            begin_segment(S, soa, uint32_t(cap + row), sh.o, sh.dir, sh.t_end);
            sh_mask |= 1u << n_sh;
            if (sh.volume) vmask |= 1u << n_sh;
            n_sh++;
        };
        int r = bounce_body<FEAT>(S, ps, h, emit, fd, fa, sample, point_stream_of(S, px, py));
        if (sh_mask) nf |= SF_PF_SHADOW | (sh_mask << SF_PF_SHADOW_SHIFT);
        if (r == PATH_CONTINUE) nf |= SF_PF_CONT;
    }
    if (final_round && nf) {
        atomicOr(status, SF_WF_ALIVE_AT_COMMIT);
        nf = 0;
    }
    store_path<FEAT>(soa, path, ps, nf);
    if (nf & SF_PF_CONT) begin_segment(S, soa, path, ps.o, ps.d, S.extent);
    if (!nf) soa.Ls[path] = make_float4(ps.L.x, ps.L.y, ps.L.z, 1.0f);
    if (soa.pv) {
        if (!nf) {  // the sample's volume part (pathtrace.wgsl:1198)
            const float3 v = path_volume(ps);
            soa.pv[path] = make_float4(v.x, v.y, v.z, 0.f);
        } else {
            soa.pv[path] = make_float4(ps.pv.x, ps.pv.y, ps.pv.z,
                                       __uint_as_float(vmask | (ps.volume_path ? 256u : 0u)));
        }
    }
    return nf;
}

static __device__ __forceinline__ void enqueue_next(const RoundQueues& q, const PathSoA& soa, uint32_t nf,
                                                    uint32_t path) {
    warp_append(&q.next_counts[0], q.next_active, nf != 0, path);
    warp_append(&q.next_counts[1], q.next_cont, (nf & SF_PF_CONT) != 0, path);
    const uint32_t mask = (nf & SF_PF_SHADOW) ? (nf >> SF_PF_SHADOW_SHIFT) & 0xffu : 0u;
    for (uint32_t k = 0; k < soa.shadow_slots; ++k)
        warp_append(&q.next_counts[2], q.next_shadow, ((mask >> k) & 1u) != 0, k * soa.capacity + path);
}

// wf_commit (wavefront.wgsl:232-260) for one pixel: ordered per-sample film add in
// ascending sample order; non-finite samples contribute (0, 1).
static __device__ __forceinline__ void commit_pixel(const PathSoA& soa, const DispatchGeom& g, const FilmPlanes& film,
                                                    uint32_t local, uint32_t path_base) {
    uint32_t tile_px = g.tile_w * g.tile_h;
    uint32_t px = g.tile_x + local % g.tile_w, py = g.tile_y + local / g.tile_w;
    const size_t idx = film_index(film, px, py);
    float4 acc = film.accum[idx];
    const bool split = film.vol != nullptr;
    float4 vol = make_float4(0.f, 0.f, 0.f, 0.f), mom = vol, surf = vol;
    if (split) {
        vol = film.vol[idx];
        mom = film.vmom[idx];
        surf = film.surf[idx];
    }
    for (uint32_t s = 0; s < g.samples; ++s) {
        const size_t row = path_base + (size_t)s * tile_px + local;
        float4 L = soa.Ls[row];
        bool ok = L.x == L.x && L.y == L.y && L.z == L.z && fabsf(L.x) < 1e30f && fabsf(L.y) < 1e30f &&
                  fabsf(L.z) < 1e30f;
        acc.x += ok ? L.x : 0.0f;
        acc.y += ok ? L.y : 0.0f;
        acc.z += ok ? L.z : 0.0f;
        acc.w += 1.0f;
        if (split) {  // volume Welford moments and the surface sums (pathtrace.wgsl:1246-1266)
            const float4 pv = soa.pv[row];
            const float3 v = ok ? mk3(pv.x, pv.y, pv.z) : mk3(0.f, 0.f, 0.f);
            const float3 sv = ok ? mk3(L.x - pv.x, L.y - pv.y, L.z - pv.z) : mk3(0.f, 0.f, 0.f);
            const float nm = fmaxf(vol.w, 1.0f), n1 = vol.w + 1.0f;
            const float3 old_mean = mk3(__fdiv_rn(vol.x, nm), __fdiv_rn(vol.y, nm), __fdiv_rn(vol.z, nm));
            const float3 delta = v - old_mean;
            const float3 new_mean = old_mean + mk3(__fdiv_rn(delta.x, n1), __fdiv_rn(delta.y, n1), __fdiv_rn(delta.z, n1));
            mom.x += fmaxf(0.0f, delta.x * (v.x - new_mean.x));
            mom.y += fmaxf(0.0f, delta.y * (v.y - new_mean.y));
            mom.z += fmaxf(0.0f, delta.z * (v.z - new_mean.z));
            mom.w += 1.0f;
            vol = make_float4(vol.x + v.x, vol.y + v.y, vol.z + v.z, vol.w + 1.0f);
            surf = make_float4(surf.x + sv.x, surf.y + sv.y, surf.z + sv.z, surf.w + 1.0f);
        }
    }
    film.accum[idx] = acc;
    if (split) {
        film.vol[idx] = vol;
        film.vmom[idx] = mom;
        film.surf[idx] = surf;
    }
}

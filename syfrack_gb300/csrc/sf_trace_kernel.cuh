// The persistent trace kernel of the wavefront integrator (the counterpart of
// wf_intersect, wavefront.wgsl:187-195, marching in resumable quanta), compiled
// once per form so that each instantiation carries only its own DE routine.
//
// Every lane holds one segment. A lane whose segment ends fetches the next work
// item at once (one atomic per warp), so the warp keeps evaluating the DE in
// lockstep instead of waiting for its longest march. Continuation hits run the
// four tetrahedral normal taps (common.wgsl:376-387) through the same DE call;
// a candidate accepted at the step budget (pathtrace.wgsl:137-141) is
// re-evaluated at its t, through that call too, for its sample. A segment still
// open after `quantum` steps saves its march state and is re-queued, bounding
// each launch's tail by one quantum.
#pragma once
#include "sf_kernels.cuh"
#include "sf_trace.cuh"
#include "sf_warp.cuh"

enum { TL_IDLE = 0, TL_MARCH = 1, TL_CAND = 2, TL_NORMAL = 3, TL_DONE = 4, TL_INIT = 5, TL_REFINE = 6, TL_FINAL = 7 };
#define SF_FORM_ANY 99u
#define SF_FORM_MIXED 98u  // any of the three iterated forms, chosen per lane

template <int FORM>
__device__ __forceinline__ DeRaw de_form(const DeProgram& P, float3 p) {
    if constexpr (FORM == SF_FORM_BULB) return de_bulb(P.fp, p);
    else if constexpr (FORM == SF_FORM_BOX) return de_box(P.fp, p);
    else if constexpr (FORM == SF_FORM_MENGER) return de_menger(P.fp, p);
    else if constexpr (FORM == SF_FORM_MIXED) {
        switch (P.form) {
        case SF_FORM_BULB: return de_bulb(P.fp, p);
        case SF_FORM_BOX: return de_box(P.fp, p);
        default: return de_menger(P.fp, p);
        }
    } else return de_raw(P, p);
}

// Job of a batched path: binary search of the jobs' first paths (staged in shared memory).
static __device__ __forceinline__ uint32_t find_job(const uint32_t* begins, uint32_t n, uint32_t path) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (begins[mid] <= path) lo = mid;
        else hi = mid;
    }
    return lo;
}

// MULTI: the work items belong to the jobs of a batch (bt); each lane reads its job's
// program and scene (L1-cached global memory) when it takes an item.
// LANE_STATS: also count warp-level DE calls and, per call, the warp's longest
// iteration count times its active lanes (a diagnostic of SIMT lane use).
// OPTICS (scenes with dielectric materials): a path's first segment
// samples the field at its origin for the medium it starts in (pathtrace.wgsl:833-840);
// a hit on a material with optics is refined by Newton steps on the exact field
// (optical_refine_hit, optics.wgsl:7-23) and, for a continuation, its normal taken at
// 1e-4; a shadow segment crosses such surfaces, its weight (PathSoA.sh_d.w) times
// 1 - opacity at each, and marches on from just past them, up to 32 crossings
// (geometry_visibility_weight, lights.wgsl:263-283).
// THREADS: 256, or 128 for the shapes that fit more warps per SM at the same registers.
template <int FORM, int MIN_BLOCKS, bool MULTI = false, bool LANE_STATS = false, bool OPTICS = false,
          int THREADS = 256>
__global__ void __launch_bounds__(THREADS, MIN_BLOCKS) k_trace(const DeProgram* __restrict__ prog_g,
                                                           const DevScene* __restrict__ scene_g, PathSoA soa,
                                                           TraceLaunch tl, unsigned long long* stats,
                                                           BatchTable bt = BatchTable{}) {
    __shared__ DeProgram P;
    __shared__ DevScene S;
    __shared__ uint32_t begins[MULTI ? SF_BATCH_MAX_JOBS : 1];
    if constexpr (MULTI) {
        for (uint32_t i = threadIdx.x; i < bt.n_jobs; i += blockDim.x) begins[i] = bt.jobs[i].path_begin;
    } else {
        stage_program(P, prog_g);
        stage_pod(S, scene_g);
        stage_more_lights(scene_g);
    }
    __syncthreads();
    const bool first = tl.resume == nullptr;
    const uint32_t n_cont = first ? tl.q.counts[1] : 0u;
    const uint32_t total = first ? n_cont + tl.q.counts[2] : *tl.resume_count;
    const uint32_t quantum = tl.quantum ? tl.quantum : 0xffffffffu;
    const DeProgram* Pl = &P;
    const DevScene* Sl = &S;
    // a batch lane's job constants (registers); the single-job kernel reads the staged
    // scene (shared memory) at each use instead, which keeps them out of registers
    float accept_j = 0.f, safety_j = 0.f, cone_j = 0.f, tol_j = 0.f;
    uint32_t max_steps_j = 0;
    bool absolute_j = false;
#define TR_ACCEPT (MULTI ? accept_j : hit_accept(S))
#define TR_ABSOLUTE (MULTI ? absolute_j : hit_absolute(S))
#define TR_SAFETY (MULTI ? safety_j : S.step_scale)
#define TR_MAX_STEPS (MULTI ? max_steps_j : S.max_steps)
#define TR_CONE (MULTI ? cone_j : S.pixel_cone)
#define TR_TOL (MULTI ? tol_j : S.pixel_tolerance)
    const uint32_t cap = soa.capacity;

    // item: the continuation path, or the shadow row (k * cap + path) of a shadow segment
    uint32_t state = TL_IDLE, path = 0, item = 0, li = SF_NO_LIGHT, budget = 0;
    bool shadow = false;
    March m{};  // set by each refill before use
    // The normal taps of a surface hit overlay march fields that are dead once the hit
    // is recorded: the gradient (omega, previous radius, step length), the tap step
    // (candidate error), the hit word iterations | material << 16 (steps) and the tap
    // index (the quantum budget).
    float& gx = m.omega;
    float& gy = m.prev_radius;
    float& gz = m.step_len;
    float& hstep = m.cand_err;
    uint32_t& hit_w = m.i;
    uint32_t& tap = budget;
    uint32_t n_eval = 0, n_iter = 0, n_wcall = 0;
    // every item of a round's first launch is one segment: the queue counts are the
    // segment statistics (one thread adds them)
    if (first && blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(&stats[SF_STAT_SEGMENTS], (unsigned long long)total);
        atomicAdd(&stats[SF_STAT_SHADOW_SEGMENTS], (unsigned long long)(total - n_cont));
    }
    unsigned long long n_slots = 0;
    // LANE_STATS: the warp's cycles, and those after its first failed fetch (the tail,
    // when the launch's work is exhausted and lanes idle beside the last segments)
    long long t_start = 0, t_dry = 0;
    if constexpr (LANE_STATS) t_start = clock64();

    // End of a continuation or shadow segment without a surface sample.
    auto finish = [&](int r) {
        if (shadow) soa.vis[item] = (r == MARCH_MISS && li == SF_NO_LIGHT) ? 1u : 0u;
        else if (r == MARCH_MISS && li != SF_NO_LIGHT)
            soa.hit[path] = make_uint4(__float_as_uint(m.t_end), m.i, li, SF_HF_HIT);
        else
            soa.hit[path] = make_uint4(__float_as_uint(m.t_end), m.i, SF_NO_LIGHT,
                                       r == MARCH_EXHAUSTED ? SF_HF_EXHAUSTED : 0u);
        state = TL_IDLE;
    };
    // Surface hit of a continuation segment at m.t with sample s: record it, then the normal taps.
    auto surface_hit = [&](const DeRaw& s) {
        DeSampleF smp = de_finalize(*Pl, s);
        soa.hit[path] = make_uint4(__float_as_uint(m.t), m.i, SF_NO_LIGHT, SF_HF_HIT);
        soa.hit_tr[path] = make_float4(smp.traps[0], smp.traps[1], smp.traps[2], smp.traps[3]);
        hit_w = smp.iter | (smp.material << 16);  // stored with the normal after the last tap
        hstep = fmaxf(m.t * TR_CONE * 0.5f, 1e-4f) * TR_TOL;
        gx = gy = gz = 0.f;
        tap = 0;
        state = TL_NORMAL;
    };

    // OPTICS: a march that found a surface with sample s (at m.t): refine it when its
    // material has optics, else end a shadow segment or record a continuation's hit.
    auto on_hit = [&](const DeRaw& s) {
        if (OPTICS && optics_enabled(material_optics(*Sl, s.material))) {
            hstep = fmaxf(1e-5f, fminf(1e-3f, m.t * 1e-5f));  // the Newton step's difference
            tap = 0;                                           // iteration * 3 + tap of the step
            state = TL_REFINE;
        } else if (shadow) {
            finish(MARCH_HIT);
        } else {
            surface_hit(s);
        }
    };
    // OPTICS: the march of a fresh segment from its loaded state.
    auto start = [&]() {
        state = TL_MARCH;
        int r = march_check(m, TR_MAX_STEPS, TR_ACCEPT);
        if (r == MARCH_HIT) {
            if (shadow && !OPTICS) finish(MARCH_HIT);
            else { m.t = m.cand_t; state = TL_CAND; }
        } else if (r != MARCH_CONTINUE) {
            finish(r);
        }
    };

    const uint32_t regen = tl.regen ? tl.regen : 1u;
    while (true) {
        // One vote per DE call while every lane marches; when some lane is idle or done,
        // a second vote decides the warp's next move: all lanes done ends the loop; idle
        // lanes take new segments together once `regen` of them are idle (or no lane is
        // marching), so the segment set-up runs for many lanes at once and the fetch (a
        // vote and one atomic) only runs when the warp refills.
        const uint32_t quiet = __ballot_sync(FULL_MASK, state == TL_IDLE || state == TL_DONE);
        const uint32_t idle = quiet ? __ballot_sync(FULL_MASK, state == TL_IDLE) : 0u;  // warp-uniform
        if (quiet == FULL_MASK && idle == 0u) break;  // every lane done
        if (idle && ((uint32_t)__popc(idle) >= regen || quiet == FULL_MASK)) {  // warp-uniform
            const uint32_t w = warp_fetch(tl.work_counter, state == TL_IDLE);
            if constexpr (LANE_STATS) {
                if (t_dry == 0 && __any_sync(FULL_MASK, state == TL_IDLE && w >= total)) t_dry = clock64();
            }
            if (state == TL_IDLE) {
                if (w >= total) {
                    state = TL_DONE;
                } else {
                    if (first) {
                        shadow = w >= n_cont;
                        item = shadow ? tl.q.shadow[w - n_cont] : (tl.q.cont ? tl.q.cont[w] : w);
                    } else {
                        const uint32_t it = tl.resume[w];
                        item = it & 0x7fffffffu;
                        shadow = (it >> 31) != 0;
                    }
                    path = shadow ? item % cap : item;
                    if constexpr (MULTI) {
                        const BatchJob& job = bt.jobs[find_job(begins, bt.n_jobs, path)];
                        Pl = job.prog;
                        Sl = job.scene;
                        cone_j = Sl->pixel_cone;
                        tol_j = Sl->pixel_tolerance;
                        accept_j = hit_accept(*Sl);
                        absolute_j = hit_absolute(*Sl);
                        safety_j = Sl->step_scale;
                        max_steps_j = Sl->max_steps;
                    }
                    float4 o = shadow ? soa.sh_o[item] : soa.o[path];
                    float4 d = shadow ? soa.sh_d[item] : soa.d[path];
                    // the march state: set by the stage that made the ray, or saved by the
                    // previous launch at its step quantum
                    const uint32_t row = shadow ? cap + item : item;
                    const float4 a = soa.m0[row], b = soa.m1[row];
                    m.ro = mk3(o.x, o.y, o.z);
                    m.rd = mk3(d.x, d.y, d.z);
                    m.t = a.x; m.omega = a.y; m.prev_radius = a.z; m.step_len = a.w;
                    m.t_end = b.x; m.cand_t = b.y; m.cand_err = b.z; m.i = __float_as_uint(b.w);
                    li = soa.m2[row];
                    budget = quantum;
                    if (OPTICS && !shadow && first &&
                        (__float_as_uint(soa.ex[path].z) & SF_EX_INIT) != 0u) state = TL_INIT;
                    else start();
                }
            }
        }
        if (state != TL_IDLE && state != TL_DONE) {
            float3 q = m.ro + m.rd * m.t;
            if (state == TL_NORMAL) q = q + tetra_offset(tap) * hstep;
            if (OPTICS && state == TL_REFINE && tap % 3u != 0u) q = q + m.rd * (tap % 3u == 1u ? hstep : -hstep);
            // the single-job kernel reads the program from shared memory by name (LDS)
            DeRaw s;
            const bool exact_state = OPTICS && (state == TL_INIT || state == TL_REFINE || state == TL_FINAL);
            if constexpr (MULTI && FORM == SF_FORM_ANY && OPTICS)
                s = exact_state ? de_raw_exact(*Pl, q) : de_form<FORM>(*Pl, q);
            else if constexpr (MULTI) s = de_form<FORM>(*Pl, q);
            else if constexpr (FORM == SF_FORM_ANY && OPTICS) s = exact_state ? de_raw_exact(P, q) : de_form<FORM>(P, q);
            else s = de_form<FORM>(P, q);
            n_eval++;
            n_iter += s.iter;
            if constexpr (FORM == SF_FORM_ANY) {
                // a flagged march or candidate sample near acceptance: the exact sample
                if (state != TL_NORMAL && !exact_state && needs_exact(s, m.t, TR_SAFETY, TR_ACCEPT, TR_ABSOLUTE)) {
                    if constexpr (MULTI) s = de_raw_exact(*Pl, q);
                    else s = de_raw_exact(P, q);
                    n_eval++;
                    n_iter += s.iter;
                }
            }
            if constexpr (LANE_STATS) {
                // warp-level DE calls and, per call, the iterations the warp ran (its
                // longest lane) times its active lanes
                const uint32_t am = __activemask();
                const uint32_t mx = __reduce_max_sync(am, s.iter);
                if (lane_id() == (uint32_t)(__ffs(am) - 1)) {
                    n_wcall++;
                    n_slots += (unsigned long long)mx * __popc(am);
                }
            }
            if (state == TL_NORMAL) {
                const float3 off = tetra_offset(tap);
                gx = fmaf(off.x, s.d, gx);
                gy = fmaf(off.y, s.d, gy);
                gz = fmaf(off.z, s.d, gz);
                if (++tap == 4) {
                    // the taps of a hit end in the launch that found it (no quantum applies)
                    const float3 n = wnormalize(mk3(gx, gy, gz));
                    soa.hit_n[path] = make_float4(n.x, n.y, n.z, __uint_as_float(hit_w));
                    state = TL_IDLE;
                }
            } else if (state == TL_CAND) {
                if constexpr (OPTICS) on_hit(s);
                else surface_hit(s);
            } else if (OPTICS && state == TL_INIT) {
                // the medium the path starts in, then its first march
                const DevOptics& o = material_optics(*Sl, s.material);
                const bool solid = s.d < 0.0f && optics_enabled(o) && o.surface[1] > 0.0f && o.surface[3] == 0.0f;
                soa.ex[path].z = __uint_as_float(s.material | (solid ? SF_EX_SOLID : 0u));
                start();
            } else if (OPTICS && state == TL_REFINE) {
                const uint32_t k = tap % 3u;
                if (k == 0u) {
                    gx = s.d;
                    if (fabsf(s.d) < 1e-5f) state = TL_FINAL;
                    else tap++;
                } else if (k == 1u) {
                    gy = s.d;
                    tap++;
                } else {
                    const float derivative = (gy - s.d) / (2.0f * hstep);
                    if (fabsf(derivative) < 1e-5f) {
                        state = TL_FINAL;
                    } else {
                        m.t = fmaxf(0.0f, m.t - fminf(fmaxf(gx / derivative, -0.5f), 0.5f));
                        tap++;
                        if (tap == 24u) state = TL_FINAL;  // eight Newton steps
                    }
                }
            } else if (OPTICS && state == TL_FINAL) {
                const DevOptics& o = material_optics(*Sl, s.material);
                if (!shadow) {
                    // the refined hit, its sample and the normal taps (1e-4 on a dielectric)
                    const DeSampleF smp = de_finalize(*Pl, s);
                    soa.hit[path] = make_uint4(__float_as_uint(m.t), m.i, SF_NO_LIGHT, SF_HF_HIT);
                    soa.hit_tr[path] = make_float4(smp.traps[0], smp.traps[1], smp.traps[2], smp.traps[3]);
                    hit_w = smp.iter | (smp.material << 16);
                    hstep = optics_enabled(o) ? 1e-4f : fmaxf(m.t * TR_CONE * 0.5f, 1e-4f) * TR_TOL;
                    gx = gy = gz = 0.f;
                    tap = 0;
                    state = TL_NORMAL;
                } else if (!optics_enabled(o)) {
                    finish(MARCH_HIT);
                } else {
                    // cross the surface: its coverage weighs the segment, which marches on
                    float4 so = soa.sh_o[item];
                    float4 sd = soa.sh_d[item];
                    float4 sc = soa.sh_c[item];
                    sd.w *= 1.0f - o.surface[0];
                    sc.w += 1.0f;
                    const float distance = m.t + 1e-4f;
                    const float3 origin = m.ro + m.rd * distance;
                    const float remaining = so.w - distance;
                    if (sd.w < 1e-6f) {
                        soa.vis[item] = 0u;
                        state = TL_IDLE;
                    } else if (remaining <= 0.0f) {
                        soa.sh_d[item] = sd;
                        soa.vis[item] = 1u;
                        state = TL_IDLE;
                    } else if (sc.w >= 32.0f) {  // the 32 segments of the visibility loop spent
                        soa.vis[item] = 0u;
                        state = TL_IDLE;
                    } else {
                        soa.sh_o[item] = make_float4(origin.x, origin.y, origin.z, remaining);
                        soa.sh_d[item] = sd;
                        soa.sh_c[item] = sc;
                        const float te = nearest_emitter(*Sl, origin, m.rd, remaining, li);
                        march_begin(m, origin, m.rd, te);
                        start();
                    }
                }
            } else {
                int r = march_update(m, s.d, s.flags, TR_SAFETY, TR_ACCEPT, TR_ABSOLUTE);
                if (r == MARCH_HIT) {
                    if constexpr (OPTICS) on_hit(s);
                    else if (shadow) finish(MARCH_HIT);
                    else surface_hit(s);
                } else if (r != MARCH_CONTINUE) {
                    finish(r);
                } else {
                    r = march_check(m, TR_MAX_STEPS, TR_ACCEPT);
                    if (r == MARCH_HIT) {  // candidate accepted at the step budget
                        if (shadow && !OPTICS) finish(MARCH_HIT);
                        else { m.t = m.cand_t; state = TL_CAND; }
                    } else if (r != MARCH_CONTINUE) {
                        finish(r);
                    } else if (--budget == 0) {
                        // quantum spent: save the march and hand the segment to the next launch
                        const uint32_t row = shadow ? cap + item : item;
                        soa.m0[row] = make_float4(m.t, m.omega, m.prev_radius, m.step_len);
                        soa.m1[row] = make_float4(m.t_end, m.cand_t, m.cand_err, __uint_as_float(m.i));
                        soa.m2[row] = li;
                        warp_append(tl.next_resume_count, tl.next_resume, true, item | (shadow ? 0x80000000u : 0u));
                        state = TL_IDLE;
                    }
                }
            }
        }
    }
    warp_stat(&stats[SF_STAT_DE_EVALS], n_eval);
    warp_stat(&stats[SF_STAT_DE_ITERS], n_iter);
    if constexpr (LANE_STATS) {
        warp_stat(&stats[SF_STAT_WARP_DE_CALLS], n_wcall);
        warp_stat(&stats[SF_STAT_ITER_SLOTS], n_slots);
        if (lane_id() == 0) {
            const long long t_end = clock64();
            atomicAdd(&stats[SF_STAT_WARP_CYCLES], (unsigned long long)(t_end - t_start));
            atomicAdd(&stats[SF_STAT_TAIL_CYCLES], (unsigned long long)(t_dry ? t_end - t_dry : 0));
        }
    }
#undef TR_ACCEPT
#undef TR_ABSOLUTE
#undef TR_SAFETY
#undef TR_MAX_STEPS
#undef TR_CONE
#undef TR_TOL
}

template <int FORM>
static cudaError_t launch_trace_form(const DeProgram* prog, const DevScene* scene, PathSoA soa, TraceLaunch tl,
                                     unsigned long long* stats, int blocks, int min_blocks, uint32_t light_smem, cudaStream_t st) {
    if (tl.optics) {  // 6 blocks of 128 threads per SM (the host sizes the grid)
        k_trace<FORM, 6, false, false, true, 128><<<blocks, 128, light_smem, st>>>(prog, scene, soa, tl, stats);
        return cudaGetLastError();
    }
    if (tl.lane_stats && min_blocks == 3) {
        k_trace<FORM, 3, false, true><<<blocks, 256, light_smem, st>>>(prog, scene, soa, tl, stats);
        return cudaGetLastError();
    }
    if (tl.lane_stats && min_blocks == 7) {
        k_trace<FORM, 7, false, true, false, 128><<<blocks, 128, light_smem, st>>>(prog, scene, soa, tl, stats);
        return cudaGetLastError();
    }
    switch (min_blocks) {
    case 3: k_trace<FORM, 3><<<blocks, 256, light_smem, st>>>(prog, scene, soa, tl, stats); break;
    case 4: k_trace<FORM, 4><<<blocks, 256, light_smem, st>>>(prog, scene, soa, tl, stats); break;
    // 128-thread blocks: 6 or 7 per SM (24 or 28 warps at up to 85 or 73 registers)
    case 6: k_trace<FORM, 6, false, false, false, 128><<<blocks, 128, light_smem, st>>>(prog, scene, soa, tl, stats); break;
    case 7: k_trace<FORM, 7, false, false, false, 128><<<blocks, 128, light_smem, st>>>(prog, scene, soa, tl, stats); break;
    default: k_trace<FORM, 2><<<blocks, 256, light_smem, st>>>(prog, scene, soa, tl, stats); break;
    }
    return cudaGetLastError();
}

// Host side of the batched wavefront (sf_batch_*): many jobs rendered by one set of
// launches per round, captured once in a CUDA graph and replayed; the autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "sf_host_internal.h"

using namespace sfh;

// ------------------------------------------------------------------ batches

struct sf_batch {
    sf_context* ctx = nullptr;
    std::vector<sf_graph*> graphs;
    std::vector<BatchJob> jobs;  // host copy (initial sample_start)
    std::vector<sf_scene_desc> scenes;
    WaveArena a;
    cudaGraphExec_t exec = nullptr;
    uint32_t status_host = 0;
};

namespace sfh {

// Carves an arena for `capacity` paths and `max_jobs` jobs out of one allocation.
sf_status arena_alloc(sf_context* c, WaveArena& a, uint32_t capacity, uint32_t max_jobs, uint32_t rounds,
                      uint32_t shadow_slots, size_t extra_bytes, size_t* extra_offset) {
    const size_t N = capacity;
    const uint32_t K = std::max<uint32_t>(shadow_slots, 1);
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
    size_t o_jobs = take(size_t(max_jobs) * sizeof(BatchJob));
    size_t o_Ls = take(N * 16), o_soa = take(wave_soa_bytes(N, K)), o_lists = take(wave_lists_bytes(N, K));
    size_t o_march = take(wave_march_bytes(N, K)), o_resume = take(wave_resume_bytes(N, K));
    size_t o_counts = take(size_t(rounds + 1) * 16), o_qcounts = take(size_t(rounds) * 64 * 8), o_status = take(16);
    size_t o_extra = take(extra_bytes);
    sf_status st = ctx_alloc(c, off, &a.mem);
    if (st != SF_OK) return st;
    a.mem_bytes = off;
    char* base = static_cast<char*>(a.mem);
    a.bt.jobs = reinterpret_cast<BatchJob*>(base + o_jobs);
    a.capacity = capacity;
    a.max_jobs = max_jobs;
    a.rounds = rounds;
    wave_bind(a.soa, base + o_soa, base + o_march, capacity, K);
    a.soa.Ls = reinterpret_cast<float4*>(base + o_Ls);
    a.lists = reinterpret_cast<uint32_t*>(base + o_lists);
    a.resume = reinterpret_cast<uint32_t*>(base + o_resume);
    a.counts = reinterpret_cast<uint32_t*>(base + o_counts);
    a.qcounts = reinterpret_cast<uint32_t*>(base + o_qcounts);
    a.status = reinterpret_cast<uint32_t*>(base + o_status);
    if (extra_offset) *extra_offset = o_extra;
    return SF_OK;
}

// One pass of a batched wavefront on stream st: every job of a.bt renders its samples.
sf_status wave_record_pass(sf_context* c, const WaveArena& a, cudaStream_t st, bool timed) {
    const size_t N = a.capacity;
    const uint32_t R = a.rounds;
    const uint32_t Q = a.quantum ? std::min<uint32_t>((a.max_steps + a.quantum - 1) / a.quantum + 1, 64) : 1;
    CU(cudaMemsetAsync(a.counts, 0, size_t(R + 1) * 16, st));
    CU(cudaMemsetAsync(a.qcounts, 0, size_t(R) * 64 * 2 * 4, st));
    {
        LaunchTimer t(c, false, timed, st);
        CU(sf_launch_generate_batch(a.bt, a.soa, a.counts, st));
    }
    const int blocks = int(a.min_blocks) * c->sm_count;
    const uint32_t K = a.soa.shadow_slots;
    for (uint32_t r = 0; r < R; ++r) {
        RoundQueues q;
        wave_round_queues(q, a.lists, N, K, r, a.counts);
        for (uint32_t j = 0; j < Q; ++j) {
            TraceLaunch tl{};
            tl.q = q;
            uint32_t* qc = a.qcounts + (size_t(r) * 64 + j) * 2;
            tl.work_counter = qc;
            tl.resume = j == 0 ? nullptr : wave_resume(a.resume, N, K, j - 1);
            tl.resume_count = j == 0 ? nullptr : qc - 2 + 1;
            tl.next_resume = wave_resume(a.resume, N, K, j);
            tl.next_resume_count = qc + 1;
            tl.quantum = j + 1 == Q ? 0u : a.quantum;
            tl.regen = a.regen;
            LaunchTimer t(c, true, timed, st);
            tl.optics = (a.rich & SF_RICH_OPTICS) ? 1u : 0u;
            // the optics trace kernel runs two blocks of 256 threads per SM
            CU(sf_launch_trace_batch(a.bt, a.soa, tl, c->d_stats, tl.optics ? 2 * c->sm_count : blocks,
                                     int(a.min_blocks), a.any_generic ? 1 : 0, st));
        }
        LaunchTimer t(c, false, timed, st);
        CU(sf_launch_shade_batch(a.bt, a.rich, a.soa, q, a.status, r + 1 == R ? 1 : 0, st));
    }
    {
        LaunchTimer t(c, false, timed, st);
        CU(sf_launch_commit_batch(a.bt, a.soa, st));
    }
    LaunchTimer t(c, false, timed, st);
    CU(sf_launch_advance_batch(a.bt, st));
    return SF_OK;
}

}  // namespace sfh

namespace {

sf_status batch_record_pass(sf_batch* b, bool timed) { return wave_record_pass(b->ctx, b->a, b->ctx->stream, timed); }

sf_status batch_reset(sf_batch* b) {
    sf_context* c = b->ctx;
    CU(cudaMemcpyAsync(b->a.bt.jobs, b->jobs.data(), b->jobs.size() * sizeof(BatchJob), cudaMemcpyHostToDevice,
                       c->stream));
    for (auto& j : b->jobs) CU(sf_launch_film_clear(j.film, c->stream));
    CU(cudaMemsetAsync(b->a.status, 0, 16, c->stream));
    b->status_host = 0;
    return SF_OK;
}

void batch_drop_graph(sf_batch* b) {
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
}

}  // namespace

extern "C" sf_status sf_batch_create(sf_context* c, const sf_batch_job* jobs, uint32_t n, sf_batch** out) {
    if (!c || !jobs || !out) return fail(SF_ERR_INVALID, "null argument");
    *out = nullptr;
    if (n == 0 || n > SF_BATCH_MAX_JOBS) return fail(SF_ERR_INVALID, "a batch holds 1 to 1024 jobs");
    uint64_t paths = 0, pixels = 0, film_bytes = 0;
    uint32_t rounds = 0, max_steps = 0;
    bool generic = false;
    for (uint32_t i = 0; i < n; ++i) {
        if (!jobs[i].graph || jobs[i].graph->ctx != c) return fail(SF_ERR_INVALID, "job graph missing or of another context");
        sf_status st = validate_config(jobs[i].cfg);
        if (st != SF_OK) return st;
        if (const sf_status sc = scene_check(jobs[i].scene); sc != SF_OK) return sc;

        const sf_render_config& cf = jobs[i].cfg;
        uint32_t spd = std::max<uint32_t>(std::min(cf.samples_per_dispatch ? cf.samples_per_dispatch : cf.samples_per_pixel,
                                                   cf.samples_per_pixel), 1);
        paths += uint64_t(cf.width) * cf.height * spd;
        pixels += uint64_t(cf.width) * cf.height;
        // accum | aux | depth, and for fog scenes volume | moments | surface
        film_bytes += ((uint64_t(cf.width) * cf.height * (has_fog(jobs[i].scene) ? 84 : 36) + 255) & ~uint64_t(255));
        rounds = std::max(rounds, rounds_of(cf, jobs[i].scene));
        max_steps = std::max(max_steps, cf.max_steps);
        generic |= jobs[i].graph->prog.form == SF_FORM_GENERIC;
    }
    if (paths > 0x7fffffffull) return fail(SF_ERR_INVALID, "batch too large (2^31 paths)");
    cudaSetDevice(c->device);
    auto* b = new sf_batch();
    b->ctx = c;
    for (uint32_t i = 0; i < n; ++i) b->scenes.push_back(jobs[i].scene);
    const size_t scene_bytes = (n * sizeof(DevScene) + 255) & ~size_t(255);
    size_t extra = 0;
    uint32_t K = 1;  // the most shadow segments one bounce of any job issues
    bool any_fog = false;
    uint32_t rich = 0;
    for (uint32_t i = 0; i < n; ++i) {
        K = std::max(K, shadow_slots_of(jobs[i].scene));
        any_fog |= has_fog(jobs[i].scene);
        rich |= rich_of(jobs[i].scene);
    }
    // a fog job keeps the volume layer split: every path gets a volume row; finish
    // details, textures and optics keep the footprint and medium row
    const size_t pv_bytes = any_fog ? size_t(paths) * 16 : 0;
    const size_t ex_bytes = rich ? size_t(paths) * 16 : 0;
    sf_status st = arena_alloc(c, b->a, uint32_t(paths), n, rounds, K,
                               scene_bytes + pv_bytes + ex_bytes + film_bytes, &extra);
    if (st != SF_OK) { delete b; return st; }
    b->a.max_steps = max_steps;
    b->a.any_generic = generic;
    b->a.bt.n_jobs = n;
    b->a.bt.total_paths = uint32_t(paths);
    b->a.bt.total_pixels = uint32_t(pixels);
    char* base = static_cast<char*>(b->a.mem) + extra;
    DevScene* d_scenes = reinterpret_cast<DevScene*>(base);
    std::vector<DevScene> scenes(n);
    if (any_fog) b->a.soa.pv = reinterpret_cast<float4*>(base + scene_bytes);
    if (rich) b->a.soa.ex = reinterpret_cast<float4*>(base + scene_bytes + pv_bytes);
    b->a.rich = rich;
    char* film = base + scene_bytes + pv_bytes + ex_bytes;
    uint32_t pbeg = 0, xbeg = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const sf_render_config& cf = jobs[i].cfg;
        uint32_t spd = std::max<uint32_t>(std::min(cf.samples_per_dispatch ? cf.samples_per_dispatch : cf.samples_per_pixel,
                                                   cf.samples_per_pixel), 1);
        scene_dev(jobs[i].scene, cf, jobs[i].graph->info, scenes[i]);
        BatchJob j{};
        j.prog = jobs[i].graph->d_prog;
        j.scene = d_scenes + i;
        size_t px = size_t(cf.width) * cf.height;
        // accum | aux (| volume | moments | surface for fog scenes) | depth: every float4
        // plane stays 16-byte aligned for any pixel count
        const bool fog = has_fog(jobs[i].scene);
        j.film.accum = reinterpret_cast<float4*>(film);
        j.film.aux = reinterpret_cast<float4*>(film + px * 16);
        if (fog) {
            j.film.vol = reinterpret_cast<float4*>(film + px * 32);
            j.film.vmom = j.film.vol + px;
            j.film.surf = j.film.vmom + px;
        }
        j.film.depth = reinterpret_cast<float*>(film + px * (fog ? 80 : 32));
        j.film.width = cf.width;
        j.film.height = cf.height;
        film += (px * (fog ? 84 : 36) + 255) & ~size_t(255);
        j.geom = DispatchGeom{0, 0, cf.width, cf.height, 0, spd, uint32_t(px * spd)};
        j.path_begin = pbeg;
        j.pixel_begin = xbeg;
        j.form = jobs[i].graph->prog.form;
        pbeg += uint32_t(px * spd);
        xbeg += uint32_t(px);
        b->jobs.push_back(j);
        b->graphs.push_back(jobs[i].graph);
        graph_retain(jobs[i].graph);
    }
    ctx_retain(c);
    cudaError_t e = cudaMemcpyAsync(d_scenes, scenes.data(), n * sizeof(DevScene), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) st = batch_reset(b);
    if (e == cudaSuccess && st == SF_OK) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess || st != SF_OK) {
        sf_batch_destroy(b);
        return e != cudaSuccess ? cuda_fail(e, "batch upload") : st;
    }
    *out = b;
    return SF_OK;
}

extern "C" sf_status sf_batch_set_launch(sf_batch* b, uint32_t min_blocks, uint32_t quantum, uint32_t regen) {
    if (!b) return fail(SF_ERR_INVALID, "null batch");
    sf_status st = check_launch(min_blocks, quantum, regen, false);
    if (st != SF_OK) return st;
    if (b->a.min_blocks != min_blocks || b->a.quantum != quantum || b->a.regen != regen) batch_drop_graph(b);
    b->a.min_blocks = min_blocks;
    b->a.quantum = quantum;
    b->a.regen = regen;
    return SF_OK;
}

extern "C" sf_status sf_batch_run(sf_batch* b, uint32_t passes, int use_graph) {
    if (!b) return fail(SF_ERR_INVALID, "null batch");
    sf_context* c = b->ctx;
    cudaSetDevice(c->device);
    for (uint32_t i = 0; i < passes; ++i) {
        if (!use_graph) {
            sf_status st = batch_record_pass(b, true);
            if (st != SF_OK) return st;
            continue;
        }
        if (!b->exec) {
            cudaGraph_t g = nullptr;
            CU(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            sf_status st = batch_record_pass(b, false);
            cudaError_t e = cudaStreamEndCapture(c->stream, &g);
            if (st != SF_OK) { if (g) cudaGraphDestroy(g); return st; }
            if (e != cudaSuccess) return cuda_fail(e, "graph capture");
            e = cudaGraphInstantiate(&b->exec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { b->exec = nullptr; return cuda_fail(e, "graph instantiate"); }
        }
        LaunchTimer t(c, false);
        CU(cudaGraphLaunch(b->exec, c->stream));
    }
    return SF_OK;
}

extern "C" sf_status sf_batch_sync(sf_batch* b, uint32_t timeout_ms, uint32_t* status_word) {
    if (!b) return fail(SF_ERR_INVALID, "null batch");
    sf_context* c = b->ctx;
    cudaSetDevice(c->device);
    sf_status st = wait_stream(c->stream, timeout_ms);
    if (st != SF_OK) return st;
    uint32_t w = 0;
    CU(cudaMemcpy(&w, b->a.status, 4, cudaMemcpyDeviceToHost));
    b->status_host |= w;
    if (status_word) *status_word = b->status_host;
    if (b->status_host) return fail(SF_ERR_WAVEFRONT, "wavefront invariant word " + std::to_string(b->status_host));
    return SF_OK;
}

extern "C" sf_status sf_batch_autotune(sf_batch* b, uint32_t* best_mb, uint32_t* best_q, uint32_t* best_regen,
                                      float* best_ms) {
    if (!b) return fail(SF_ERR_INVALID, "null batch");
    sf_context* c = b->ctx;
    cudaSetDevice(c->device);
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    float best = 1e30f;
    uint32_t bm = b->a.min_blocks, bq = b->a.quantum, br = b->a.regen;
    // one timed pass of a candidate shape
    auto time_pass = [&](uint32_t mb, uint32_t q, uint32_t rg, float* ms) -> sf_status {
        b->a.min_blocks = mb;
        b->a.quantum = q;
        b->a.regen = rg;
        cudaEventRecord(e0, c->stream);
        sf_status st = batch_record_pass(b, false);
        cudaEventRecord(e1, c->stream);
        if (st != SF_OK) return st;
        cudaError_t e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
        return e == cudaSuccess ? SF_OK : cuda_fail(e, "autotune");
    };
    // coordinate search: resident blocks x step quantum (0 = none) at regen 1, then the regeneration threshold
    const uint32_t mbs[3] = {2, 3, 4}, qs[4] = {0, 64, 128, 256}, rgs[4] = {1, 4, 8, 16};
    sf_status st = SF_OK;
    for (uint32_t mb : mbs)
        for (uint32_t q : qs) {
            float ms = 0;
            if ((st = time_pass(mb, q, 1, &ms)) != SF_OK) break;
            if (ms < best) { best = ms; bm = mb; bq = q; br = 1; }
        }
    for (uint32_t i = 1; i < 4 && st == SF_OK; ++i) {
        float ms = 0;
        if ((st = time_pass(bm, bq, rgs[i], &ms)) != SF_OK) break;
        if (ms < best) { best = ms; br = rgs[i]; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != SF_OK) return st;
    batch_drop_graph(b);
    b->a.min_blocks = bm;
    b->a.quantum = bq;
    b->a.regen = br;
    st = batch_reset(b);
    if (st != SF_OK) return st;
    CU(cudaStreamSynchronize(c->stream));
    if (best_mb) *best_mb = bm;
    if (best_q) *best_q = bq;
    if (best_regen) *best_regen = br;
    if (best_ms) *best_ms = best;
    return SF_OK;
}

extern "C" sf_status sf_batch_readback(sf_batch* b, uint32_t job, sf_film_planes* out) {
    if (!b || !out) return fail(SF_ERR_INVALID, "null argument");
    if (job >= b->jobs.size()) return fail(SF_ERR_INVALID, "job index out of range");
    sf_context* c = b->ctx;
    cudaSetDevice(c->device);
    CU(film_readback(c, b->jobs[job].film, *out, c->stream));
    return SF_OK;
}

extern "C" sf_status sf_batch_destroy(sf_batch* b) {
    if (!b) return SF_OK;
    sf_context* c = b->ctx;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    batch_drop_graph(b);
    ctx_free(c, b->a.mem, b->a.mem_bytes);
    for (sf_graph* g : b->graphs) sf_graph_destroy(g);
    delete b;
    ctx_release(c);
    return SF_OK;
}


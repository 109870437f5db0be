// Host side of serving (sf_server_* / sf_serve_*): the scheduler thread, its slots,
// the device and pinned-host pools, admission by the HBM budget.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "sf_host_internal.h"

using namespace sfh;

// ------------------------------------------------------------------ serving
// One scheduler thread per server. A slot is a wavefront arena plus two streams (high
// priority for batches holding a preview, low for refinements and 2D tiles) and a
// pinned staging area; it carries one batch at a time. Whenever a slot is free the
// scheduler takes requests from the queue in arrival order into a batch of one class
// (2D tiles, 3D on the per-form kernel, 3D on the generic interpreter), admitting each
// only if the device pool and the host result pool hold its bytes. Every device byte
// of films and tile outputs comes from chunks reserved once, so no request calls
// cudaMalloc or cudaFree, which would serialise the device.
namespace {

using ServeClock = std::chrono::steady_clock;

// First-fit range allocator with coalescing, over offsets of one region.
struct RangeAlloc {
    std::map<size_t, size_t> free_;  // offset -> bytes
    void init(size_t n) {
        free_.clear();
        if (n) free_[0] = n;
    }
    bool take(size_t n, size_t* off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            *off = it->first;
            size_t rest = it->second - n, roff = it->first + n;
            free_.erase(it);
            if (rest) free_[roff] = rest;
            return true;
        }
        return false;
    }
    void give(size_t off, size_t n) {
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

// Device memory of films and tile outputs: 1 GiB chunks (larger for a larger
// request) reserved on demand up to the budget and held until the server ends.
struct DevicePool {
    struct Chunk {
        char* base;
        size_t bytes;
        RangeAlloc ra;
    };
    std::vector<Chunk> chunks;
    uint64_t budget = 0, reserved = 0, used = 0, peak = 0;
    static constexpr size_t kChunk = size_t(1) << 30;

    static size_t round(size_t n) { return (n + 255) & ~size_t(255); }
    // SF_ERR_BUDGET without a message when the budget is full (the request waits).
    sf_status alloc(sf_context* c, size_t n, void** out) {
        n = round(n);
        if (used + n > budget) return SF_ERR_BUDGET;
        for (auto& ch : chunks) {
            size_t off = 0;
            if (ch.ra.take(n, &off)) {
                *out = ch.base + off;
                used += n;
                peak = std::max(peak, used);
                return SF_OK;
            }
        }
        size_t want = std::min<uint64_t>(std::max(kChunk, n), budget - reserved);
        if (want < n) return SF_ERR_BUDGET;
        void* p = nullptr;
        sf_status st = ctx_alloc(c, want, &p);
        if (st != SF_OK) return st;
        chunks.push_back({static_cast<char*>(p), want, {}});
        chunks.back().ra.init(want);
        reserved += want;
        size_t off = 0;
        chunks.back().ra.take(n, &off);
        *out = static_cast<char*>(p) + off;
        used += n;
        peak = std::max(peak, used);
        return SF_OK;
    }
    void release(void* p, size_t n) {
        if (!p) return;
        n = round(n);
        char* q = static_cast<char*>(p);
        for (auto& ch : chunks)
            if (q >= ch.base && q < ch.base + ch.bytes) {
                ch.ra.give(size_t(q - ch.base), n);
                used -= std::min<uint64_t>(used, n);
                return;
            }
    }
    void destroy(sf_context* c) {
        for (auto& ch : chunks) ctx_free(c, ch.base, ch.bytes);
        chunks.clear();
        reserved = used = 0;
    }
};

// A preview's film, kept on the device until the preview is released and no
// refinement still needs it. DevScene | accum | aux | depth.
struct ServeFilm {
    void* mem = nullptr;
    size_t bytes = 0;
    DevScene* scene = nullptr;
    FilmPlanes planes{};
    sf_graph* graph = nullptr;
    uint32_t samples = 0;  // samples once every scheduled pass has finished
    uint32_t max_bounces = 0, max_steps = 0;
    uint32_t rounds = 0;   // wavefront rounds of a pass (rounds_of)
    uint32_t rich = 0;     // SF_RICH_* of the scene: finish details, a texture, optics
    bool busy = false;     // written by a batch in flight
    int refs = 0;          // the preview until released, plus each refinement until it ends
};

enum ServeClass { SC_TILE = 0, SC_FORM = 1, SC_GENERIC = 2 };

struct ServeReq {
    uint64_t ticket = 0;
    uint32_t kind = 0, state = SF_REQ_QUEUED;
    sf_status status = SF_OK;
    int cls = SC_TILE;
    std::string error;
    double t_submit = 0, t_start = 0, t_done = 0;
    uint32_t width = 0, height = 0, samples = 0, sample_start = 0, batch_requests = 0;
    uint64_t work = 0;
    ServeFilm* film = nullptr;  // 3D
    DevScene scene{};           // PREVIEW: uploaded with its first batch
    PlanarDev F{};              // TILE_2D
    CanvasDev K{};
    bool traps = true;          // TILE_2D: SF_TILE_ALL
    void* dmem = nullptr;       // TILE_2D: descriptors and outputs
    size_t dbytes = 0;
    size_t h_off = 0, h_bytes = 0;
};

constexpr uint32_t kServeMaxSlots = 8;
constexpr uint32_t kServeShadowSlots = 3;  // shadow segments per bounce the slot arenas hold
constexpr uint32_t kServeMaxTiles = 64;  // 2D tiles per batch
// A tile's device block starts with PlanarDev (0), CanvasDev (256) and its pixel
// counter (512); the staging area holds the same bytes, counter zero.
constexpr size_t kTileHeader = 768;
static_assert(sizeof(PlanarDev) <= 256 && sizeof(CanvasDev) <= 256, "tile header layout");

struct ServeSlot {
    cudaStream_t hi = nullptr, lo = nullptr, st = nullptr;
    cudaEvent_t done = nullptr;
    WaveArena arena;
    char* stage = nullptr;  // pinned: job table | scenes | tile descriptors | status word
    size_t stage_bytes = 0;
    std::vector<ServeReq*> reqs;
    int cls = SC_TILE;
    bool busy = false;
};

}  // namespace

struct sf_server {
    sf_context* ctx = nullptr;
    sf_server_config cfg{};
    ServeClock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread thread;
    bool stop = false;
    uint64_t next_ticket = 1;
    std::unordered_map<uint64_t, std::unique_ptr<ServeReq>> reqs;
    std::deque<ServeReq*> queue;
    std::vector<ServeSlot> slots;
    DevicePool pool;
    char* host = nullptr;  // pinned result pool
    RangeAlloc host_ra;
    uint64_t host_used = 0;
    sf_server_stats stats{};
};

namespace {

double serve_now(const sf_server* s) {
    return std::chrono::duration<double, std::milli>(ServeClock::now() - s->t0).count();
}

size_t stage_jobs_off(const sf_server*) { return 0; }
size_t stage_scenes_off(const sf_server* s) { return DevicePool::round(size_t(s->cfg.max_jobs) * sizeof(BatchJob)); }
size_t stage_tiles_off(const sf_server* s) {
    return stage_scenes_off(s) + DevicePool::round(size_t(s->cfg.max_jobs) * sizeof(DevScene));
}
size_t stage_status_off(const sf_server* s) { return stage_tiles_off(s) + size_t(kServeMaxTiles) * kTileHeader; }

void film_unref(sf_server* s, ServeFilm* f) {
    if (--f->refs > 0) return;
    s->pool.release(f->mem, f->bytes);
    sf_graph_destroy(f->graph);
    delete f;
}

void finish_req(sf_server* s, ServeReq* r, sf_status st, const std::string& error = std::string()) {
    r->state = st == SF_OK ? SF_REQ_DONE : SF_REQ_FAILED;
    r->status = st;
    r->error = error;
    r->t_done = serve_now(s);
    if (r->kind == SF_REQ_TILE_2D) {
        s->pool.release(r->dmem, r->dbytes);
        r->dmem = nullptr;
    }
    if (r->film) {
        r->film->busy = false;
        if (r->kind == SF_REQ_REFINE) {
            film_unref(s, r->film);
            r->film = nullptr;
        }
    }
    if (st == SF_OK) s->stats.completed++;
    else s->stats.failed++;
}

// Bytes a request needs when admitted: device (films, tile outputs) and host results.
void request_bytes(const ServeReq* r, size_t* dev, size_t* host) {
    size_t px = size_t(r->width) * r->height;
    if (r->kind == SF_REQ_PREVIEW) *dev = DevicePool::round(sizeof(DevScene)) + DevicePool::round(px * 36);
    else if (r->kind == SF_REQ_TILE_2D) *dev = kTileHeader + px * 24;
    else *dev = 0;
    // 3D: accum; 2D: iterations | smooth, or iterations | distance | 4 trap planes
    *host = DevicePool::round(r->kind != SF_REQ_TILE_2D ? px * 16 : r->traps ? px * 24 : px * 8);
}

// Retires the batches whose completion event has fired. Returns true if any did.
bool serve_retire(sf_server* s) {
    bool any = false;
    for (auto& sl : s->slots) {
        if (!sl.busy) continue;
        cudaError_t e = cudaEventQuery(sl.done);
        if (e == cudaErrorNotReady) continue;
        sf_status st = SF_OK;
        std::string msg;
        if (e != cudaSuccess) {
            st = cuda_fail(e, "serving batch");
            msg = last_error();
        } else if (sl.cls != SC_TILE) {
            uint32_t w = 0;
            std::memcpy(&w, sl.stage + stage_status_off(s), 4);
            if (w) {
                st = SF_ERR_WAVEFRONT;
                msg = "wavefront invariant word " + std::to_string(w);
            }
        }
        for (ServeReq* r : sl.reqs) finish_req(s, r, st, msg);
        sl.reqs.clear();
        sl.busy = false;
        any = true;
    }
    if (any) s->cv_done.notify_all();
    return any;
}

sf_status launch_tiles(sf_server* s, ServeSlot& sl) {
    cudaStream_t st = sl.st;
    char* stage = sl.stage + stage_tiles_off(s);
    for (size_t i = 0; i < sl.reqs.size(); ++i) {
        ServeReq* r = sl.reqs[i];
        size_t n = size_t(r->width) * r->height;
        char* d = static_cast<char*>(r->dmem);
        char* h = stage + i * kTileHeader;
        std::memset(h, 0, kTileHeader);
        std::memcpy(h, &r->F, sizeof r->F);
        std::memcpy(h + 256, &r->K, sizeof r->K);
        CU(cudaMemcpyAsync(d, h, kTileHeader, cudaMemcpyHostToDevice, st));
        float* dist = reinterpret_cast<float*>(d + kTileHeader);
        float* traps = dist + n;
        uint32_t* iters = reinterpret_cast<uint32_t*>(traps + 4 * n);
        s->ctx->launches++;
        s->stats.launches++;
        CU(sf_launch_escape2d(reinterpret_cast<PlanarDev*>(d), reinterpret_cast<CanvasDev*>(d + 256), 0, 0, r->width,
                              r->height, 0xffffffffu, dist, traps, iters, s->ctx->d_stats,
                              reinterpret_cast<uint32_t*>(d + 512), r->traps ? 1 : 0,
                              r->F.family == 3 || r->F.family == 4, st));
        char* out = s->host + r->h_off;
        CU(cudaMemcpyAsync(out, iters, n * 4, cudaMemcpyDeviceToHost, st));
        if (r->traps) CU(cudaMemcpyAsync(out + n * 4, dist, n * 4 * 5, cudaMemcpyDeviceToHost, st));  // dist | traps
        else CU(cudaMemcpyAsync(out + n * 4, traps, n * 4, cudaMemcpyDeviceToHost, st));
    }
    return SF_OK;
}

sf_status launch_wave(sf_server* s, ServeSlot& sl) {
    cudaStream_t st = sl.st;
    WaveArena& a = sl.arena;
    BatchJob* hj = reinterpret_cast<BatchJob*>(sl.stage + stage_jobs_off(s));
    DevScene* hs = reinterpret_cast<DevScene*>(sl.stage + stage_scenes_off(s));
    uint32_t paths = 0, pixels = 0, rounds = 0, steps = 0, n_scenes = 0, rich = 0;
    for (size_t i = 0; i < sl.reqs.size(); ++i) {
        ServeReq* r = sl.reqs[i];
        ServeFilm* f = r->film;
        uint32_t px = r->width * r->height;
        BatchJob j{};
        j.prog = f->graph->d_prog;
        j.scene = f->scene;
        j.film = f->planes;
        j.geom = DispatchGeom{0, 0, r->width, r->height, r->sample_start, r->samples, px * r->samples};
        j.path_begin = paths;
        j.pixel_begin = pixels;
        j.form = f->graph->prog.form;
        hj[i] = j;
        paths += px * r->samples;
        pixels += px;
        rounds = std::max(rounds, f->rounds);
        steps = std::max(steps, f->max_steps);
        rich |= f->rich;
        if (r->kind == SF_REQ_PREVIEW) {
            hs[n_scenes] = r->scene;
            CU(cudaMemcpyAsync(f->scene, hs + n_scenes, sizeof(DevScene), cudaMemcpyHostToDevice, st));
            CU(sf_launch_film_clear(f->planes, st));
            s->ctx->launches++;
            s->stats.launches++;
            n_scenes++;
        }
    }
    a.bt.n_jobs = uint32_t(sl.reqs.size());
    a.bt.total_paths = paths;
    a.bt.total_pixels = pixels;
    a.max_steps = steps;
    a.any_generic = sl.cls == SC_GENERIC;
    CU(cudaMemcpyAsync(a.bt.jobs, hj, sl.reqs.size() * sizeof(BatchJob), cudaMemcpyHostToDevice, st));
    CU(cudaMemsetAsync(a.status, 0, 16, st));
    // rounds vary per batch; the arena's queue counters are sized for its largest
    WaveArena pass = a;
    pass.rounds = rounds;
    // scenes with finish details, a texture or optics: the feature-built kernels and the
    // footprint and medium rows (kept by the slot, unused by plain batches)
    pass.rich = rich;
    if (!rich) pass.soa.ex = nullptr;
    uint64_t before = s->ctx->launches;
    sf_status rs = wave_record_pass(s->ctx, pass, st, false);
    s->stats.launches += s->ctx->launches - before;
    if (rs != SF_OK) return rs;
    for (ServeReq* r : sl.reqs)
        CU(cudaMemcpyAsync(s->host + r->h_off, r->film->planes.accum, size_t(r->width) * r->height * 16,
                           cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(sl.stage + stage_status_off(s), a.status, 4, cudaMemcpyDeviceToHost, st));
    return SF_OK;
}

// Forms and launches one batch on a free slot. Returns true if it launched one.
bool serve_admit(sf_server* s, ServeSlot& sl) {
    std::vector<ServeReq*> take;
    int cls = -1;
    uint64_t paths = 0, pixels = 0;
    uint32_t rounds = 0;
    bool blocked = false;
    // films with an earlier request left in the queue: their later requests wait, so
    // each film's passes run in submission order
    std::set<const ServeFilm*> held;
    auto skip = [&](std::deque<ServeReq*>::iterator& it) {
        if ((*it)->film) held.insert((*it)->film);
        ++it;
    };
    for (auto it = s->queue.begin(); it != s->queue.end() && take.size() < s->cfg.max_jobs;) {
        ServeReq* r = *it;
        if (r->kind == SF_REQ_REFINE && (r->film->busy || !r->film->mem || held.count(r->film))) { skip(it); continue; }
        if (cls >= 0 && r->cls != cls) { skip(it); continue; }
        uint64_t px = uint64_t(r->width) * r->height;
        if (r->kind == SF_REQ_TILE_2D) {
            if (take.size() >= kServeMaxTiles || (pixels + px > s->cfg.max_tile_pixels && !take.empty())) break;
        } else {
            uint64_t need = px * r->samples;
            if (paths + need > s->cfg.path_capacity) { skip(it); continue; }
        }
        size_t dev = 0, hb = 0;
        request_bytes(r, &dev, &hb);
        size_t hoff = 0;
        if (!s->host_ra.take(hb, &hoff)) { blocked = true; break; }
        void* dm = nullptr;
        if (dev) {
            sf_status st = s->pool.alloc(s->ctx, dev, &dm);
            if (st != SF_OK) {
                s->host_ra.give(hoff, hb);
                blocked = true;
                break;
            }
        }
        r->h_off = hoff;
        r->h_bytes = hb;
        s->host_used += hb;
        if (r->kind == SF_REQ_TILE_2D) {
            r->dmem = dm;
            r->dbytes = dev;
        } else if (r->kind == SF_REQ_PREVIEW) {
            ServeFilm* f = r->film;
            f->mem = dm;
            f->bytes = dev;
            char* b = static_cast<char*>(dm);
            size_t px2 = size_t(px);
            f->scene = reinterpret_cast<DevScene*>(b);
            char* film = b + DevicePool::round(sizeof(DevScene));
            f->planes.accum = reinterpret_cast<float4*>(film);
            f->planes.aux = reinterpret_cast<float4*>(film + px2 * 16);
            f->planes.depth = reinterpret_cast<float*>(film + px2 * 32);
            f->planes.width = r->width;
            f->planes.height = r->height;
        }
        if (r->kind != SF_REQ_TILE_2D) {
            r->sample_start = r->film->samples;
            r->film->samples += r->samples;
            r->film->busy = true;
            paths += px * r->samples;
            rounds = std::max(rounds, r->film->rounds);
            r->work = px * r->samples;
        } else {
            r->work = px;
        }
        pixels += px;
        cls = r->cls;
        take.push_back(r);
        it = s->queue.erase(it);
    }
    if (blocked) s->stats.admission_waits++;
    if (take.empty()) return false;
    sl.reqs = take;
    sl.cls = cls;
    bool preview = false;
    for (ServeReq* r : take) preview |= r->kind == SF_REQ_PREVIEW;
    sl.st = preview ? sl.hi : sl.lo;
    double now = serve_now(s);
    for (ServeReq* r : take) {
        r->state = SF_REQ_RUNNING;
        r->t_start = now;
        r->batch_requests = uint32_t(take.size());
    }
    sf_status st = cls == SC_TILE ? launch_tiles(s, sl) : launch_wave(s, sl);
    cudaError_t e = st == SF_OK ? cudaEventRecord(sl.done, sl.st) : cudaSuccess;
    if (st == SF_OK && e != cudaSuccess) st = cuda_fail(e, "cudaEventRecord");
    s->stats.batches++;
    s->stats.batched_requests += take.size();
    if (st != SF_OK) {
        // the stream may still run part of the batch: wait for it before failing the requests
        std::string msg = last_error();
        cudaStreamSynchronize(sl.st);
        for (ServeReq* r : take) finish_req(s, r, st, msg);
        sl.reqs.clear();
        s->cv_done.notify_all();
        return true;
    }
    sl.busy = true;
    return true;
}

void serve_loop(sf_server* s) {
    cudaSetDevice(s->ctx->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (!s->stop) {
        bool progress = serve_retire(s);
        bool busy = false;
        bool admitting = true;
        for (auto& sl : s->slots) {
            // a scan that admits nothing would admit nothing for the next free slot either
            if (admitting && !sl.busy && !s->queue.empty()) {
                admitting = serve_admit(s, sl);
                progress |= admitting;
            }
            busy |= sl.busy;
        }
        if (progress) continue;
        if (busy) {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(20));
            lk.lock();
        } else {
            s->cv_work.wait_for(lk, std::chrono::milliseconds(2));
        }
    }
    // drain the batches in flight
    for (auto& sl : s->slots)
        if (sl.busy) {
            lk.unlock();
            cudaEventSynchronize(sl.done);
            lk.lock();
        }
    serve_retire(s);
}

void fill_result(const sf_server* s, const ServeReq* r, sf_result* o) {
    std::memset(o, 0, sizeof *o);
    o->state = r->state;
    o->status = r->status;
    o->kind = r->kind;
    o->width = r->width;
    o->height = r->height;
    o->samples = r->kind == SF_REQ_TILE_2D ? 0 : r->sample_start + r->samples;
    o->batch_requests = r->batch_requests;
    o->work = r->work;
    o->submit_ms = r->t_submit;
    o->start_ms = r->t_start;
    o->done_ms = r->t_done;
    if (r->state != SF_REQ_DONE) return;
    const char* h = s->host + r->h_off;
    size_t n = size_t(r->width) * r->height;
    if (r->kind == SF_REQ_TILE_2D) {
        o->iterations = reinterpret_cast<const uint32_t*>(h);
        if (r->traps) {
            o->distance = reinterpret_cast<const float*>(h + n * 4);
            o->traps = reinterpret_cast<const float*>(h + n * 8);
            o->smooth = o->traps;
        } else {
            o->smooth = reinterpret_cast<const float*>(h + n * 4);
        }
    } else {
        o->accum = reinterpret_cast<const float*>(h);
    }
}

}  // namespace

extern "C" sf_status sf_server_create(sf_context* c, const sf_server_config* cfg, sf_server** out) {
    if (!c || !out) return fail(SF_ERR_INVALID, "null argument");
    *out = nullptr;
    sf_server_config k = cfg ? *cfg : sf_server_config{};
    if (!k.slots) k.slots = 4;
    if (!k.path_capacity) k.path_capacity = 1u << 22;
    if (!k.max_jobs) k.max_jobs = 256;
    if (!k.max_tile_pixels) k.max_tile_pixels = 1u << 25;
    if (!k.host_result_bytes) k.host_result_bytes = uint64_t(1) << 30;
    if (!k.min_blocks) k.min_blocks = 3;
    if (!k.quantum) k.quantum = 128;
    if (!k.regen) k.regen = 4;
    if (!k.hbm_budget) return fail(SF_ERR_INVALID, "hbm_budget must be set");
    if (k.slots > kServeMaxSlots) return fail(SF_ERR_INVALID, "1..8 slots");
    if (k.max_jobs > SF_BATCH_MAX_JOBS) return fail(SF_ERR_INVALID, "a batch holds 1 to 1024 requests");
    if (k.path_capacity > 0x7fffffffu) return fail(SF_ERR_INVALID, "path capacity above 2^31");
    sf_status ls = check_launch(k.min_blocks, k.quantum, k.regen, false);
    if (ls != SF_OK) return ls;
    cudaSetDevice(c->device);
    auto* s = new sf_server();
    s->ctx = c;
    s->cfg = k;
    s->pool.budget = k.hbm_budget;
    ctx_retain(c);
    auto bail = [&](sf_status st) {
        sf_server_destroy(s);
        return st;
    };
    cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(&s->host), k.host_result_bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        s->host = nullptr;
        return bail(cuda_fail(e, "pinned result pool"));
    }
    s->host_ra.init(k.host_result_bytes);
    int lo_prio = 0, hi_prio = 0;
    cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    s->slots.resize(k.slots);
    // bounces <= 32 (validate_config), and the 33 rounds of an optics scene's null events
    const uint32_t max_rounds = 32 + 2 + 33;
    for (auto& sl : s->slots) {
        sl.stage_bytes = stage_status_off(s) + 256;
        e = cudaStreamCreateWithPriority(&sl.hi, cudaStreamNonBlocking, hi_prio);
        if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&sl.lo, cudaStreamNonBlocking, lo_prio);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        if (e == cudaSuccess)
            e = cudaHostAlloc(reinterpret_cast<void**>(&sl.stage), sl.stage_bytes, cudaHostAllocDefault);
        if (e != cudaSuccess) return bail(cuda_fail(e, "server slot"));
        size_t ex_off = 0;
        sf_status st = arena_alloc(c, sl.arena, k.path_capacity, k.max_jobs, max_rounds, kServeShadowSlots,
                                   size_t(k.path_capacity) * 16, &ex_off);
        if (st != SF_OK) return bail(st);
        sl.arena.soa.ex = reinterpret_cast<float4*>(static_cast<char*>(sl.arena.mem) + ex_off);
        sl.arena.min_blocks = k.min_blocks;
        sl.arena.quantum = k.quantum;
        sl.arena.regen = k.regen;
    }
    s->t0 = ServeClock::now();
    s->thread = std::thread(serve_loop, s);
    *out = s;
    return SF_OK;
}

extern "C" sf_status sf_serve_submit(sf_server* s, const sf_request* q, uint64_t* ticket) {
    if (!s || !q || !ticket) return fail(SF_ERR_INVALID, "null argument");
    *ticket = 0;
    auto r = std::make_unique<ServeReq>();
    r->kind = q->kind;
    if (q->kind == SF_REQ_PREVIEW) {
        if (!q->graph || q->graph->ctx != s->ctx) return fail(SF_ERR_INVALID, "preview graph missing or of another context");
        sf_status st = validate_config(q->cfg);
        if (st != SF_OK) return st;
        if (const sf_status sc = scene_check(q->scene); sc != SF_OK) return sc;
        if (has_hdri(q->scene)) return fail(SF_ERR_UNSUPPORTED, "HDRI panoramas are rendered by sessions, not served");
        if (shadow_slots_of(q->scene) > kServeShadowSlots)
            return fail(SF_ERR_UNSUPPORTED, "the server's arenas hold 3 shadow segments per bounce");
        r->width = q->cfg.width;
        r->height = q->cfg.height;
        r->samples = q->cfg.samples_per_pixel;
        scene_dev(q->scene, q->cfg, q->graph->info, r->scene);
        r->cls = q->graph->prog.form == SF_FORM_GENERIC ? SC_GENERIC : SC_FORM;
    } else if (q->kind == SF_REQ_REFINE) {
        if (q->samples == 0) return fail(SF_ERR_INVALID, "a refinement adds at least one sample");
    } else if (q->kind == SF_REQ_TILE_2D) {
        sf_status st = planar_check(&q->planar);
        if (st != SF_OK) return st;
        if (!q->canvas.width || !q->canvas.height) return fail(SF_ERR_INVALID, "empty canvas");
        r->width = q->canvas.width;
        r->height = q->canvas.height;
        planar_dev(q->planar, r->F);
        std::memset(&r->K, 0, sizeof r->K);
        r->K.center[0] = q->canvas.center[0];
        r->K.center[1] = q->canvas.center[1];
        r->K.zoom = q->canvas.zoom;
        r->K.aspect = float(q->canvas.width) / float(q->canvas.height);
        float rad = q->canvas.rotation_deg * (3.14159265358979323846f / 180.0f);
        r->K.rot_sin = sinf(rad);
        r->K.rot_cos = cosf(rad);
        r->K.width = q->canvas.width;
        r->K.height = q->canvas.height;
        r->K.seed = uint32_t(q->canvas.seed) ^ uint32_t(q->canvas.seed >> 32);
        r->cls = SC_TILE;
        if (q->tile_outputs > SF_TILE_COUNTS) return fail(SF_ERR_INVALID, "unknown tile outputs");
        r->traps = q->tile_outputs == SF_TILE_ALL;
        if (uint64_t(r->width) * r->height > s->cfg.max_tile_pixels)
            return fail(SF_ERR_INVALID, "tile larger than the server's max_tile_pixels");
    } else {
        return fail(SF_ERR_INVALID, "unknown request kind");
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return fail(SF_ERR_INVALID, "server stopping");
    if (q->kind == SF_REQ_REFINE) {
        auto it = s->reqs.find(q->parent);
        if (it == s->reqs.end() || it->second->kind != SF_REQ_PREVIEW || !it->second->film)
            return fail(SF_ERR_INVALID, "refinement of an unknown or released preview");
        ServeReq* p = it->second.get();
        if (p->state == SF_REQ_FAILED) return fail(SF_ERR_INVALID, "refinement of a failed preview");
        r->film = p->film;
        r->width = p->width;
        r->height = p->height;
        r->samples = q->samples;
        r->cls = p->cls;
        r->film->refs++;
    }
    size_t dev = 0, hb = 0;
    request_bytes(r.get(), &dev, &hb);
    if (r->kind != SF_REQ_TILE_2D && uint64_t(r->width) * r->height * r->samples > s->cfg.path_capacity) {
        if (r->film) film_unref(s, r->film);
        return fail(SF_ERR_INVALID, "request needs more paths than the server's path_capacity");
    }
    if (dev > s->cfg.hbm_budget || hb > s->cfg.host_result_bytes) {
        if (r->film) film_unref(s, r->film);
        return fail(SF_ERR_BUDGET, "request larger than the server's HBM budget or result pool");
    }
    if (q->kind == SF_REQ_PREVIEW) {
        auto* f = new ServeFilm();
        f->graph = q->graph;
        graph_retain(q->graph);
        f->max_bounces = q->cfg.max_bounces;
        f->max_steps = q->cfg.max_steps;
        f->rounds = rounds_of(q->cfg, q->scene);
        f->rich = rich_of(q->scene);
        f->refs = 1;
        r->film = f;
    }
    r->ticket = s->next_ticket++;
    r->t_submit = serve_now(s);
    *ticket = r->ticket;
    s->queue.push_back(r.get());
    s->reqs.emplace(r->ticket, std::move(r));
    s->stats.submitted++;
    s->cv_work.notify_one();
    return SF_OK;
}

extern "C" sf_status sf_serve_poll(sf_server* s, uint64_t ticket, sf_result* out) {
    if (!s || !out) return fail(SF_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return fail(SF_ERR_INVALID, "unknown ticket");
    fill_result(s, it->second.get(), out);
    return SF_OK;
}

extern "C" sf_status sf_serve_wait(sf_server* s, uint64_t ticket, uint32_t timeout_ms, sf_result* out) {
    if (!s) return fail(SF_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto deadline = ServeClock::now() + std::chrono::milliseconds(timeout_ms);
    for (;;) {
        auto it = s->reqs.find(ticket);
        if (it == s->reqs.end()) return fail(SF_ERR_INVALID, "unknown ticket");
        ServeReq* r = it->second.get();
        if (r->state == SF_REQ_DONE || r->state == SF_REQ_FAILED) {
            if (out) fill_result(s, r, out);
            return r->state == SF_REQ_DONE ? SF_OK : fail(r->status, "request failed: " + r->error);
        }
        if (timeout_ms == 0) s->cv_done.wait(lk);
        else if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && ServeClock::now() >= deadline)
            return fail(SF_ERR_TIMEOUT, "request not finished in time");
    }
}

extern "C" sf_status sf_serve_release(sf_server* s, uint64_t ticket) {
    if (!s) return fail(SF_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return fail(SF_ERR_INVALID, "unknown ticket");
    ServeReq* r = it->second.get();
    if (r->state == SF_REQ_QUEUED || r->state == SF_REQ_RUNNING) return fail(SF_ERR_BUSY, "request in flight");
    if (r->h_bytes) {
        s->host_ra.give(r->h_off, r->h_bytes);
        s->host_used -= r->h_bytes;
    }
    if (r->film) film_unref(s, r->film);
    s->reqs.erase(it);
    s->cv_work.notify_one();  // memory freed: queued requests may now fit
    return SF_OK;
}

extern "C" sf_status sf_server_stats_get(sf_server* s, sf_server_stats* out) {
    if (!s || !out) return fail(SF_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->hbm_used = s->pool.used;
    out->hbm_peak = s->pool.peak;
    out->hbm_reserved = s->pool.reserved;
    out->host_used = s->host_used;
    out->now_ms = serve_now(s);
    return SF_OK;
}

extern "C" sf_status sf_server_destroy(sf_server* s) {
    if (!s) return SF_OK;
    sf_context* c = s->ctx;
    cudaSetDevice(c->device);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->thread.joinable()) s->thread.join();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (ServeReq* r : s->queue) finish_req(s, r, SF_ERR_INVALID, "server stopped");
        s->queue.clear();
        s->cv_done.notify_all();
        for (auto& kv : s->reqs)
            if (kv.second->film) film_unref(s, kv.second->film);
        s->reqs.clear();
    }
    for (auto& sl : s->slots) {
        if (sl.hi) cudaStreamSynchronize(sl.hi);
        if (sl.lo) cudaStreamSynchronize(sl.lo);
        ctx_free(c, sl.arena.mem, sl.arena.mem_bytes);
        if (sl.stage) cudaFreeHost(sl.stage);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.hi) cudaStreamDestroy(sl.hi);
        if (sl.lo) cudaStreamDestroy(sl.lo);
    }
    s->pool.destroy(c);
    if (s->host) cudaFreeHost(s->host);
    delete s;
    ctx_release(c);
    return SF_OK;
}

// Tiled export: the image in host memory, one tile-sized film on the device.
//
// The reference's TiledExport (crates/syfrack-render/src/export.rs:830-900) renders
// bounded GPU tiles and commits each complete tile into a host image from a
// collector, so snapshots never hold half a tile. Here one window session (the
// session code with a film the size of a tile, whose origin moves from tile to
// tile) renders every sample of a tile on the context stream; the tile's planes are
// copied into one of two pinned staging buffers behind an event, and the host
// commits a staged tile while the device renders the next one.
#include <sys/stat.h>

#include <chrono>
#include <cstring>
#include <thread>

#include "sf_host_internal.h"

using namespace sfh;

namespace {

constexpr uint32_t EX_MAGIC = 0x58454653u;  // "SFEX"
constexpr uint32_t EX_VERSION = 3;  // 2: the scene carries its fog; 3: the config its hit epsilon
constexpr int kStages = 2;

struct Stage {
    float* host = nullptr;      // pinned: accum (16 B/px) | depth (4 B/px) | aux (16 B/px)
                                // (| volume | moments | surface, 16 B/px each, for fog scenes)
    cudaEvent_t ready = nullptr;
    int tile = -1;              // tile whose planes are in flight or staged, -1 when free
};

}  // namespace

struct sf_export {
    sf_context* ctx = nullptr;
    sf_session* win = nullptr;  // holds the graph reference
    std::vector<sf_tile> tiles; // done = samples_per_pixel once committed
    std::vector<float> accum, depth, aux;
    std::vector<float> vol;     // fog scenes: volume | moments | surface planes of the image (4 floats/px each)
    Stage stage[kStages];
    int next_stage = 0;
    uint32_t tile_size = 0;
};

namespace {

sf_status wait_event(cudaEvent_t ev, uint32_t timeout_ms) {
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaEventQuery(ev);
        if (e == cudaSuccess) return SF_OK;
        if (e != cudaErrorNotReady) return cuda_fail(e, "export tile copy");
        if (std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(timeout_ms))
            return fail(SF_ERR_TIMEOUT, "export tile copy did not finish");
        std::this_thread::sleep_for(std::chrono::microseconds(100));
    }
}

// The collector: a staged tile's planes into the host image, whole.
sf_status commit_stage(sf_export* e, Stage& s) {
    if (s.tile < 0) return SF_OK;
    sf_status st = wait_event(s.ready, 10000);  // DISPATCH_TIMEOUT, renderer.rs:236
    if (st != SF_OK) return st;
    sf_tile& t = e->tiles[size_t(s.tile)];
    const uint32_t W = e->win->cfg.width;
    const size_t n = size_t(t.w) * t.h;
    const float* acc = s.host;
    const float* dep = s.host + 4 * n;
    const float* aux = s.host + 5 * n;
    const float* vol = s.host + 9 * n;
    const size_t px = e->depth.size();
    for (uint32_t y = 0; y < t.h; ++y) {
        const size_t dst = size_t(t.y + y) * W + t.x, src = size_t(y) * t.w;
        std::memcpy(&e->accum[4 * dst], acc + 4 * src, size_t(t.w) * 16);
        std::memcpy(&e->depth[dst], dep + src, size_t(t.w) * 4);
        std::memcpy(&e->aux[4 * dst], aux + 4 * src, size_t(t.w) * 16);
        if (!e->vol.empty())
            for (size_t k = 0; k < 3; ++k)
                std::memcpy(&e->vol[4 * (k * px + dst)], vol + 4 * (k * n + src), size_t(t.w) * 16);
    }
    t.done = e->win->cfg.samples_per_pixel;
    s.tile = -1;
    return SF_OK;
}

sf_status flush(sf_export* e) {
    for (Stage& s : e->stage) {
        sf_status st = commit_stage(e, s);
        if (st != SF_OK) return st;
    }
    return SF_OK;
}

// Every sample of one tile into the window film, then its planes to a staging buffer.
sf_status render_tile(sf_export* e, int index) {
    Stage& s = e->stage[e->next_stage];
    sf_status st = commit_stage(e, s);  // the stage's previous tile, copied long ago
    if (st != SF_OK) return st;
    sf_session* w = e->win;
    sf_context* c = e->ctx;
    const sf_tile t = e->tiles[size_t(index)];
    w->film.x0 = t.x;
    w->film.y0 = t.y;
    w->film.width = t.w;
    w->film.height = t.h;
    CU(sf_launch_film_clear(w->film, c->stream));
    const uint32_t spp = w->cfg.samples_per_pixel, spd = w->cfg.samples_per_dispatch;
    for (uint32_t done = 0; done < spp;) {
        const uint32_t n = std::min(spd, spp - done);
        sf_tile d = t;
        d.done = done;
        st = sf_session_dispatch(w, d, n);
        if (st != SF_OK) return st;
        done += n;
    }
    const size_t n = size_t(t.w) * t.h;
    CU(cudaMemcpyAsync(s.host, w->film.accum, n * 16, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaMemcpyAsync(s.host + 4 * n, w->film.depth, n * 4, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaMemcpyAsync(s.host + 5 * n, w->film.aux, n * 16, cudaMemcpyDeviceToHost, c->stream));
    if (w->film.vol) {
        CU(cudaMemcpyAsync(s.host + 9 * n, w->film.vol, n * 16, cudaMemcpyDeviceToHost, c->stream));
        CU(cudaMemcpyAsync(s.host + 13 * n, w->film.vmom, n * 16, cudaMemcpyDeviceToHost, c->stream));
        CU(cudaMemcpyAsync(s.host + 17 * n, w->film.surf, n * 16, cudaMemcpyDeviceToHost, c->stream));
    }
    CU(cudaEventRecord(s.ready, c->stream));
    s.tile = index;
    e->next_stage = (e->next_stage + 1) % kStages;
    return SF_OK;
}

bool in_flight(const sf_export* e, int index) {
    for (const Stage& s : e->stage)
        if (s.tile == index) return true;
    return false;
}

sf_status export_alloc(sf_context* c, sf_graph* g, const sf_scene_desc& scene, const sf_render_config& cfg,
                       sf_export** out) {
    sf_status st = validate_config(cfg);
    if (st != SF_OK) return st;
    if (const sf_status sc = scene_check(scene); sc != SF_OK) return sc;
    cudaSetDevice(c->device);
    auto* w = new sf_session();
    w->ctx = c;
    w->graph = g;
    w->scene = scene;
    w->cfg = cfg;
    w->window = true;
    st = session_alloc(w);
    if (st != SF_OK) {
        if (w->mem) ctx_free(c, w->mem, w->mem_bytes);
        delete w;
        return st;
    }
    ctx_retain(c);
    graph_retain(g);
    auto* e = new sf_export();
    e->ctx = c;
    e->win = w;
    e->tile_size = w->tile_size;
    e->tiles = w->tiles;  // TileGrid::new (tiles.rs:4-40), row-major
    for (auto& t : e->tiles) t.done = 0;
    const size_t px = size_t(cfg.width) * cfg.height;
    e->accum.assign(4 * px, 0.0f);
    e->depth.assign(px, -1.0f);
    e->aux.assign(4 * px, 0.0f);
    for (size_t i = 0; i < px; ++i) e->aux[4 * i + 3] = -1.0f;
    const bool fog = w->film.vol != nullptr;
    if (fog) e->vol.assign(12 * px, 0.0f);
    const size_t stage_bytes =
        size_t(std::min(w->tile_size, cfg.width)) * std::min(w->tile_size, cfg.height) * (fog ? 84 : 36);
    for (Stage& s : e->stage) {
        cudaError_t err = cudaHostAlloc(reinterpret_cast<void**>(&s.host), stage_bytes, cudaHostAllocDefault);
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&s.ready, cudaEventDisableTiming);
        if (err != cudaSuccess) {
            sf_export_destroy(e);
            return cuda_fail(err, "export staging");
        }
    }
    *out = e;
    return SF_OK;
}

}  // namespace

extern "C" sf_status sf_export_create(sf_context* c, sf_graph* g, const sf_scene_desc* scene,
                                      const sf_render_config* cfg, sf_export** out) {
    if (!c || !g || !scene || !cfg || !out) return fail(SF_ERR_INVALID, "null argument");
    *out = nullptr;
    return export_alloc(c, g, *scene, *cfg, out);
}

extern "C" sf_status sf_export_step(sf_export* e, uint32_t budget_ms, int* done) {
    if (!e) return fail(SF_ERR_INVALID, "null export");
    cudaSetDevice(e->ctx->device);
    auto t0 = std::chrono::steady_clock::now();
    const uint32_t target = e->win->cfg.samples_per_pixel;
    for (;;) {
        // TileGrid::next_pending (tiles.rs:52-59): the first tile below the target
        int next = -1;
        for (size_t i = 0; i < e->tiles.size(); ++i)
            if (e->tiles[i].done < target && !in_flight(e, int(i))) { next = int(i); break; }
        if (next < 0) break;
        sf_status st = render_tile(e, next);
        if (st != SF_OK) return st;
        double el = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (!budget_ms || el >= budget_ms) break;
    }
    sf_status st = flush(e);
    if (st != SF_OK) return st;
    CU(cudaMemcpy(&e->win->status_host, e->win->status, 4, cudaMemcpyDeviceToHost));
    if (e->win->status_host) return fail(SF_ERR_WAVEFRONT, "wavefront invariant failed during export");
    bool complete = true;
    for (auto& t : e->tiles)
        if (t.done < target) complete = false;
    if (done) *done = complete ? 1 : 0;
    return SF_OK;
}

extern "C" sf_status sf_export_progress(sf_export* e, sf_progress* out) {
    if (!e || !out) return fail(SF_ERR_INVALID, "null argument");
    std::memset(out, 0, sizeof *out);
    out->tiles = uint32_t(e->tiles.size());
    out->dispatches = e->win->dispatches;
    out->target = e->win->cfg.samples_per_pixel;
    uint32_t mn = 0xffffffffu, mx = 0;
    for (auto& t : e->tiles) {
        mn = std::min(mn, t.done);
        mx = std::max(mx, t.done);
        out->pixel_samples_done += uint64_t(t.w) * t.h * t.done;
    }
    out->samples_min = e->tiles.empty() ? 0 : mn;
    out->samples_max = mx;
    out->pixel_samples_total = uint64_t(e->win->cfg.width) * e->win->cfg.height * e->win->cfg.samples_per_pixel;
    out->status_word = e->win->status_host;
    return SF_OK;
}

extern "C" sf_status sf_export_readback(sf_export* e, sf_film_planes* out) {
    if (!e || !out) return fail(SF_ERR_INVALID, "null argument");
    cudaSetDevice(e->ctx->device);
    sf_status st = flush(e);
    if (st != SF_OK) return st;
    const size_t px = e->depth.size();
    if (out->accum) std::memcpy(out->accum, e->accum.data(), px * 16);
    if (out->depth) std::memcpy(out->depth, e->depth.data(), px * 4);
    if (out->aux) std::memcpy(out->aux, e->aux.data(), px * 16);
    const bool split = !e->vol.empty();
    if (split) {  // the volume layer split of a fog scene
        if (out->volume) std::memcpy(out->volume, e->vol.data(), px * 16);
        if (out->moments) std::memcpy(out->moments, e->vol.data() + 4 * px, px * 16);
        if (out->surface) std::memcpy(out->surface, e->vol.data() + 8 * px, px * 16);
    }
    // without fog the volume contribution is zero and surface = radiance
    for (size_t i = 0; i < px; ++i) {
        const float n = e->accum[4 * i + 3];
        if (!split)
            for (float* p : {out->volume, out->moments})
                if (p) { p[4 * i] = p[4 * i + 1] = p[4 * i + 2] = 0.0f; p[4 * i + 3] = n; }
        if (out->color) {  // RenderOutput.color: accum.rgb / max(count, 1), alpha 1
            const float d = std::max(n, 1.0f);
            for (int k = 0; k < 3; ++k) out->color[4 * i + k] = e->accum[4 * i + k] / d;
            out->color[4 * i + 3] = 1.0f;
        }
    }
    if (out->surface && !split) std::memcpy(out->surface, e->accum.data(), px * 16);
    return SF_OK;
}

extern "C" sf_status sf_export_save(sf_export* e, const char* dir) {
    if (!e || !dir || !*dir) return fail(SF_ERR_INVALID, "null argument");
    if (has_hdri(e->win->scene)) return fail(SF_ERR_UNSUPPORTED, "scenes with an HDRI panorama are not checkpointed");
    if (e->win->scene.texture.graph)  // the texture's graph is a caller object, like a panorama
        return fail(SF_ERR_UNSUPPORTED, "textured scenes are not checkpointed");
    cudaSetDevice(e->ctx->device);
    sf_status st = flush(e);
    if (st != SF_OK) return st;
    const size_t px = e->depth.size();
    Writer image;
    image.put_bytes(e->accum.data(), px * 16);
    image.put_bytes(e->depth.data(), px * 4);
    image.put_bytes(e->aux.data(), px * 16);
    if (!e->vol.empty()) image.put_bytes(e->vol.data(), px * 48);
    const sf_graph* g = e->win->graph;
    Writer w;
    w.put(EX_MAGIC);
    w.put(EX_VERSION);
    w.put_str(producer_of(e->ctx));
    w.put(e->win->cfg);
    w.put(e->win->scene);
    w.put_str(g->topology);
    w.put(uint32_t(g->host.nodes.size()));
    w.put_bytes(g->host.nodes.data(), g->host.nodes.size() * sizeof(sf_node));
    w.put(fnv1a(g->host.placements.data(), g->host.placements.size() * sizeof(sf_placement)));
    w.put(e->tile_size);
    w.put(uint32_t(e->tiles.size()));
    for (auto& t : e->tiles) w.put(t);
    w.put(uint64_t(image.buf.size()));
    w.put(fnv1a(image.buf.data(), image.buf.size()));
    w.put(fnv1a(w.buf.data(), w.buf.size()));
    return install_checkpoint(dir, {{"export.bin", &image.buf}, {"state.bin", &w.buf}});
}

extern "C" sf_status sf_export_resume(sf_context* c, sf_graph* g, const char* dir, sf_export** out) {
    if (!c || !g || !dir || !out) return fail(SF_ERR_INVALID, "null argument");
    *out = nullptr;
    std::string d(dir);
    std::vector<uint8_t> state, image;
    if (!read_file(d + "/state.bin", state) || !read_file(d + "/export.bin", image))
        return fail(SF_ERR_IO, "cannot read export checkpoint in " + d);
    if (state.size() < 16) return fail(SF_ERR_CHECKPOINT, "export state truncated");
    uint64_t stored;
    std::memcpy(&stored, state.data() + state.size() - 8, 8);
    if (fnv1a(state.data(), state.size() - 8) != stored) return fail(SF_ERR_CHECKPOINT, "export state checksum mismatch");
    Reader r{state};
    if (r.get<uint32_t>() != EX_MAGIC || r.get<uint32_t>() != EX_VERSION)
        return fail(SF_ERR_CHECKPOINT, "not an export checkpoint of this version");
    const std::string producer = r.get_str();
    if (producer != producer_of(c)) return fail(SF_ERR_CHECKPOINT, "export from another producer: " + producer);
    const sf_render_config cfg = r.get<sf_render_config>();
    const sf_scene_desc scene = r.get<sf_scene_desc>();
    const std::string topo = r.get_str();
    const uint32_t nn = r.get<uint32_t>();
    if (!r.ok || nn > 4096) return fail(SF_ERR_CHECKPOINT, "export state truncated");
    std::vector<sf_node> nodes(nn);
    r.get_bytes(nodes.data(), nn * sizeof(sf_node));
    const uint64_t placements_hash = r.get<uint64_t>();
    const uint32_t tile_size = r.get<uint32_t>();
    const uint32_t nt = r.get<uint32_t>();
    if (!r.ok || nt > (1u << 24)) return fail(SF_ERR_CHECKPOINT, "export state truncated");
    std::vector<sf_tile> tiles(nt);
    for (auto& t : tiles) t = r.get<sf_tile>();
    const uint64_t image_bytes = r.get<uint64_t>(), image_hash = r.get<uint64_t>();
    if (!r.ok) return fail(SF_ERR_CHECKPOINT, "export state truncated");
    if (image_bytes != image.size() || fnv1a(image.data(), image.size()) != image_hash)
        return fail(SF_ERR_CHECKPOINT, "export.bin checksum mismatch");
    if (topo != g->topology || nn != g->host.nodes.size() ||
        std::memcmp(nodes.data(), g->host.nodes.data(), nn * sizeof(sf_node)) != 0 ||
        placements_hash != fnv1a(g->host.placements.data(), g->host.placements.size() * sizeof(sf_placement)))
        return fail(SF_ERR_CHECKPOINT, "export was made with another graph");
    const size_t px = size_t(cfg.width) * cfg.height;
    if (image.size() != px * (has_fog(scene) ? 84 : 36)) return fail(SF_ERR_CHECKPOINT, "export image size mismatch");
    sf_export* e = nullptr;
    sf_status st = export_alloc(c, g, scene, cfg, &e);
    if (st != SF_OK) return st;
    bool same = e->tile_size == tile_size && e->tiles.size() == tiles.size();
    for (size_t i = 0; same && i < tiles.size(); ++i) {
        const sf_tile& a = tiles[i];
        const sf_tile& b = e->tiles[i];
        same = a.x == b.x && a.y == b.y && a.w == b.w && a.h == b.h &&
               (a.done == 0 || a.done == cfg.samples_per_pixel);
    }
    if (!same) {
        sf_export_destroy(e);
        return fail(SF_ERR_CHECKPOINT, "export tile layout mismatch");
    }
    e->tiles = tiles;
    std::memcpy(e->accum.data(), image.data(), px * 16);
    std::memcpy(e->depth.data(), image.data() + px * 16, px * 4);
    std::memcpy(e->aux.data(), image.data() + px * 20, px * 16);
    if (!e->vol.empty()) std::memcpy(e->vol.data(), image.data() + px * 36, px * 48);
    *out = e;
    return SF_OK;
}

extern "C" sf_status sf_export_device_bytes(sf_export* e, uint64_t* out) {
    if (!e || !out) return fail(SF_ERR_INVALID, "null argument");
    *out = e->win->mem_bytes;
    return SF_OK;
}

extern "C" sf_status sf_export_destroy(sf_export* e) {
    if (!e) return SF_OK;
    cudaSetDevice(e->ctx->device);
    cudaStreamSynchronize(e->ctx->stream);
    for (Stage& s : e->stage) {
        if (s.host) cudaFreeHost(s.host);
        if (s.ready) cudaEventDestroy(s.ready);
    }
    sf_session_destroy(e->win);
    delete e;
    return SF_OK;
}

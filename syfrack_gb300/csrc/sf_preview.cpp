// The interactive preview session: the reference's ControlSession
// (crates/syfrack-render/src/control/mod.rs:172-530) on this library's fixed kernels.
//
// Nothing is compiled per graph: the graph is a device program (or a specialised
// form) read by the same kernel, so a graph or scene edit uploads data and restarts
// the machine. tick() polls the previous quantum's event and submits at most one
// quantum; it never waits for the device. The machine runs on its own
// highest-priority stream, so a preview quantum overtakes queued renders.
#include <chrono>
#include <cstring>
#include <thread>

#include "sf_host_internal.h"

using namespace sfh;

struct sf_preview {
    sf_context* ctx = nullptr;
    sf_graph* graph = nullptr;
    sf_scene_desc scene{};
    uint32_t width = 0, height = 0, quantum = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    void* mem = nullptr;
    size_t mem_bytes = 0;
    DevScene* d_scene = nullptr;
    PreviewState st{};
    PreviewOut out{};
    uint32_t* d_status = nullptr;
    uint32_t* h_status = nullptr;  // pinned: status of the last quantum
    bool pending = false, initialize = true;
    uint32_t remaining = 0, dispatches = 0;
    std::string failure;
};

namespace {

sf_status upload_scene(sf_preview* p) {
    sf_render_config cfg{};
    cfg.width = p->width;
    cfg.height = p->height;
    cfg.samples_per_pixel = 1;
    cfg.max_bounces = 0;
    cfg.max_steps = 1;
    cfg.pixel_tolerance = 1.0f;  // the control engine's fixed tolerance (control/mod.rs:241)
    DevScene S;
    scene_dev(p->scene, cfg, p->graph->info, S);
    CU(cudaMemcpyAsync(p->d_scene, &S, sizeof S, cudaMemcpyHostToDevice, p->stream));
    return SF_OK;
}

// ControlSession::set_scene's restart: new values, every pixel starts over.
sf_status restart(sf_preview* p) {
    if (p->pending) {  // the quantum in flight belongs to the old image
        CU(cudaStreamSynchronize(p->stream));
        p->pending = false;
    }
    sf_status st = upload_scene(p);
    if (st != SF_OK) return st;
    p->initialize = true;
    p->remaining = p->width * p->height;
    p->dispatches = 0;
    p->failure.clear();
    return SF_OK;
}

}  // namespace

extern "C" sf_status sf_preview_create(sf_context* c, sf_graph* g, const sf_scene_desc* scene, uint32_t width,
                                       uint32_t height, uint32_t quantum, sf_preview** out) {
    if (!c || !g || !scene || !out) return fail(SF_ERR_INVALID, "null argument");
    *out = nullptr;
    if (!width || !height || uint64_t(width) * height > (1u << 26)) return fail(SF_ERR_INVALID, "preview size");
    if (quantum == 0) quantum = 128;  // QUANTUM, control/mod.rs:18
    if (const sf_status sc = scene_check(*scene); sc != SF_OK) return sc;
    cudaSetDevice(c->device);
    auto* p = new sf_preview();
    p->ctx = c;
    p->graph = g;
    p->scene = *scene;
    p->width = width;
    p->height = height;
    p->quantum = quantum;
    auto undo = [&](sf_status s) {
        if (p->mem) ctx_free(c, p->mem, p->mem_bytes);
        if (p->h_status) cudaFreeHost(p->h_status);
        if (p->done) cudaEventDestroy(p->done);
        if (p->stream) cudaStreamDestroy(p->stream);
        delete p;
        return s;
    };
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    cudaError_t e = cudaStreamCreateWithPriority(&p->stream, cudaStreamNonBlocking, hi);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&p->h_status), 16, cudaHostAllocDefault);
    if (e != cudaSuccess) return undo(cuda_fail(e, "preview stream"));
    const size_t n = size_t(width) * height;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
    const size_t o_scene = take(sizeof(DevScene)), o_march = take(n * 16), o_grad = take(n * 16),
                 o_tags = take(n * 8), o_acc = take(n * 16), o_depth = take(n * 4), o_aux = take(n * 16),
                 o_status = take(16);
    p->mem_bytes = off;
    sf_status st = ctx_alloc(c, off, &p->mem);
    if (st != SF_OK) return undo(st);
    char* base = static_cast<char*>(p->mem);
    p->d_scene = reinterpret_cast<DevScene*>(base + o_scene);
    p->st.march = reinterpret_cast<float4*>(base + o_march);
    p->st.grad = reinterpret_cast<float4*>(base + o_grad);
    p->st.tags = reinterpret_cast<uint2*>(base + o_tags);
    p->out.accum = reinterpret_cast<float4*>(base + o_acc);
    p->out.depth = reinterpret_cast<float*>(base + o_depth);
    p->out.aux = reinterpret_cast<float4*>(base + o_aux);
    p->d_status = reinterpret_cast<uint32_t*>(base + o_status);
    st = restart(p);
    if (st != SF_OK) return undo(st);
    ctx_retain(c);
    graph_retain(g);
    *out = p;
    return SF_OK;
}

extern "C" sf_status sf_preview_set(sf_preview* p, sf_graph* g, const sf_scene_desc* scene) {
    if (!p) return fail(SF_ERR_INVALID, "null preview");
    cudaSetDevice(p->ctx->device);
    if (scene) {
        if (const sf_status sc = scene_check(*scene); sc != SF_OK) return sc;
        p->scene = *scene;
    }
    if (g && g != p->graph) {
        if (g->ctx != p->ctx) return fail(SF_ERR_INVALID, "graph of another context");
        if (p->pending) {
            CU(cudaStreamSynchronize(p->stream));
            p->pending = false;
        }
        graph_retain(g);
        sf_graph_destroy(p->graph);  // drops this preview's reference
        p->graph = g;
    }
    return restart(p);
}

extern "C" sf_status sf_preview_tick(sf_preview* p, int* complete) {
    if (!p) return fail(SF_ERR_INVALID, "null preview");
    if (!p->failure.empty()) return fail(SF_ERR_GRAPH, p->failure);
    cudaSetDevice(p->ctx->device);
    if (complete) *complete = 0;
    if (p->pending) {
        cudaError_t e = cudaEventQuery(p->done);
        if (e == cudaErrorNotReady) return SF_OK;  // never wait
        if (e != cudaSuccess) return cuda_fail(e, "preview quantum");
        p->pending = false;
        p->dispatches++;
        p->remaining = p->h_status[0];
        if (p->h_status[2]) {
            p->failure = "preview graph produced a non-finite distance";
            return fail(SF_ERR_GRAPH, p->failure);
        }
    }
    if (p->remaining == 0) {
        if (complete) *complete = 1;
        return SF_OK;
    }
    CU(cudaMemsetAsync(p->d_status, 0, 16, p->stream));
    {
        LaunchTimer t(p->ctx, false, true, p->stream);
        CU(sf_launch_preview(p->graph->d_prog, p->d_scene, p->width * p->height, p->st, p->out, p->quantum,
                             p->initialize ? 1u : 0u, p->d_status, p->stream));
    }
    p->initialize = false;
    CU(cudaMemcpyAsync(p->h_status, p->d_status, 16, cudaMemcpyDeviceToHost, p->stream));
    CU(cudaEventRecord(p->done, p->stream));
    p->pending = true;
    return SF_OK;
}

extern "C" sf_status sf_preview_wait(sf_preview* p, uint32_t timeout_ms) {
    if (!p) return fail(SF_ERR_INVALID, "null preview");
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        int complete = 0;
        sf_status st = sf_preview_tick(p, &complete);
        if (st != SF_OK) return st;
        if (complete) return SF_OK;
        if (std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(timeout_ms))
            return fail(SF_ERR_TIMEOUT, "preview did not complete");
        std::this_thread::sleep_for(std::chrono::microseconds(100));
    }
}

extern "C" sf_status sf_preview_progress(sf_preview* p, uint32_t* completed_pixels, uint32_t* dispatches) {
    if (!p) return fail(SF_ERR_INVALID, "null preview");
    if (completed_pixels) *completed_pixels = p->width * p->height - p->remaining;
    if (dispatches) *dispatches = p->dispatches;
    return SF_OK;
}

extern "C" sf_status sf_preview_readback(sf_preview* p, sf_film_planes* out) {
    if (!p || !out) return fail(SF_ERR_INVALID, "null argument");
    cudaSetDevice(p->ctx->device);
    FilmPlanes f{};
    f.accum = p->out.accum;
    f.depth = p->out.depth;
    f.aux = p->out.aux;
    f.width = p->width;
    f.height = p->height;
    CU(film_readback(p->ctx, f, *out, p->stream));
    return SF_OK;
}

extern "C" sf_status sf_preview_pick(sf_preview* p, float u, float v, float* depth, float* aux) {
    if (!p || !depth) return fail(SF_ERR_INVALID, "null argument");
    cudaSetDevice(p->ctx->device);
    const uint64_t x = uint64_t(std::min(std::max(u, 0.0f), 0.9999f) * float(p->width));
    const uint64_t y = uint64_t(std::min(std::max(v, 0.0f), 0.9999f) * float(p->height));
    const uint64_t i = y * p->width + x;
    float a[4] = {0.f, 0.f, 0.f, -1.f};
    CU(cudaMemcpyAsync(depth, p->out.depth + i, 4, cudaMemcpyDeviceToHost, p->stream));
    CU(cudaMemcpyAsync(a, p->out.aux + i, 16, cudaMemcpyDeviceToHost, p->stream));
    CU(cudaStreamSynchronize(p->stream));
    if (aux) std::memcpy(aux, a, 16);
    return SF_OK;
}

extern "C" sf_status sf_preview_destroy(sf_preview* p) {
    if (!p) return SF_OK;
    sf_context* c = p->ctx;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(p->stream);
    ctx_free(c, p->mem, p->mem_bytes);
    cudaFreeHost(p->h_status);
    cudaEventDestroy(p->done);
    cudaStreamDestroy(p->stream);
    sf_graph* g = p->graph;
    delete p;
    sf_graph_destroy(g);
    ctx_release(c);
    return SF_OK;
}

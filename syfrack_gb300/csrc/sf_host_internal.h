// Internal interface of the host runtime shared by its translation units
// (sf_host.cpp: graphs, contexts, sessions, checkpoints, escape time; sf_batch_host.cpp:
// batched wavefronts; sf_serve.cpp: the serving scheduler; sf_export.cpp: tiled
// exports). Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/syfrack_gpu.h"
#include "sf_kernels.cuh"
#include "sf_program.h"

namespace sfh {

// Error reporting: the calling thread's message for sf_last_error.
sf_status fail(sf_status s, const std::string& msg);
sf_status cuda_fail(cudaError_t e, const char* what);
const std::string& last_error();
#define CU(expr)                                                   \
    do {                                                           \
        cudaError_t _e = (expr);                                   \
        if (_e != cudaSuccess) return sfh::cuda_fail(_e, #expr);   \
    } while (0)

// The graph as the host holds it after validation.
struct HostGraph {
    std::vector<sf_node> nodes;
    std::vector<sf_link> links;
    std::vector<uint32_t> body;
    std::vector<sf_placement> placements;
    float safety = 1.f, hint = 1.f;

    const sf_node* node(uint32_t id) const {
        for (auto& n : nodes)
            if (n.id == id) return &n;
        return nullptr;
    }
    bool input_of(uint32_t to, uint32_t port, uint32_t* from) const {
        for (auto& l : links)
            if (l.to_node == to && l.to_port == port) { *from = l.from_node; return true; }
        return false;
    }
    std::vector<uint32_t> body_of(const sf_node& n) const {
        std::vector<uint32_t> b;
        if (n.kind == SF_NODE_ITERATE)
            for (uint32_t i = 0; i < n.body_len; ++i) b.push_back(body[n.body_offset + i]);
        return b;
    }
};

}  // namespace sfh

// ------------------------------------------------------------------ context
struct sf_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint64_t budget = 0, used = 0;
    std::string device_name;
    int cc_major = 0, cc_minor = 0, sm_count = 0;
    bool profiling = false;
    bool lane_stats = false;  // the trace kernel's per-call lane statistics (a slower instantiation)
    struct Timed { cudaEvent_t a, b; bool trace; };
    std::vector<Timed> timed;
    std::vector<cudaEvent_t> spare;
    double kernel_ms = 0, trace_ms = 0;
    std::atomic<uint64_t> launches{0}, trace_launches{0};
    unsigned long long* d_stats = nullptr;  // SF_STAT_COUNT counters
    uint32_t* d_work = nullptr;             // scratch work counters
    // Graphs and sessions hold a reference, so handles may be destroyed in any order.
    int refs = 1;
    std::mutex mu;
    std::mutex alloc_mu;  // budget accounting (a server thread allocates too)
    // pinned staging of readbacks and the primary-ray scratch, grown on demand and
    // reused by every call (stage_mu guards both)
    void* stage = nullptr;
    size_t stage_bytes = 0;
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    // arenas of destroyed sessions (idle: their stream was synchronised), kept for the
    // next session of the same size; counted in `used`, released first when an
    // admission needs the room (alloc_mu guards them)
    std::vector<std::pair<void*, size_t>> cached;
    std::mutex stage_mu;
};

struct sf_graph {
    sf_context* ctx = nullptr;
    int refs = 1;  // sessions hold a reference
    sfh::HostGraph host;
    DeProgram prog;
    DeProgram* d_prog = nullptr;
    float* d_inst = nullptr;  // Instances blocks (DeProgram.inst_data)
    size_t inst_bytes = 0;
    sf_graph_info info;
    std::string topology;
};

namespace sfh {

// Device memory under the context's HBM admission budget.
// Device memory within the context's budget; `trim` lets the cached scratch of
// primary and escape-time calls be released first (callers holding stage_mu pass false).
sf_status ctx_alloc(sf_context* c, size_t bytes, void** p, bool trim = true);
void ctx_free(sf_context* c, void* p, size_t bytes);
// Frees an idle block into the context's cache of session arenas (at most four).
void ctx_free_cached(sf_context* c, void* p, size_t bytes);
void ctx_retain(sf_context* c);
void ctx_release(sf_context* c);
void graph_retain(sf_graph* g);
cudaEvent_t get_event(sf_context* c);
void collect_timing(sf_context* c);
sf_status wait_stream(cudaStream_t st, uint32_t timeout_ms);

// Scoped CUDA-event timing of one launch on the context stream.
struct LaunchTimer {
    sf_context* c;
    cudaEvent_t a = nullptr;
    bool trace;
    cudaStream_t st;
    LaunchTimer(sf_context* ctx, bool is_trace, bool timed = true, cudaStream_t stream = nullptr)
        : c(ctx), trace(is_trace), st(stream ? stream : ctx->stream) {
        c->launches++;
        if (is_trace) c->trace_launches++;
        if (c->profiling && timed) {
            a = get_event(c);
            cudaEventRecord(a, st);
        }
    }
    ~LaunchTimer() {
        if (a) {
            cudaEvent_t b = get_event(c);
            cudaEventRecord(b, st);
            c->timed.push_back({a, b, trace});
        }
    }
};

float sqrt_threshold(float b);
void scene_dev(const sf_scene_desc& d, const sf_render_config& c, const sf_graph_info& gi, DevScene& S);
sf_status validate_config(const sf_render_config& c);
// Scene limits and the light kinds and colouring the device path supports: at most
// max_lights lights, and (unless the integrator traces shadow segments as it issues
// them) at most 8 shadow segments per bounce.
sf_status scene_check(const sf_scene_desc& d, uint32_t max_lights = SF_MAX_LIGHTS, bool inline_shadows = false);
uint32_t shadow_slots_of(const sf_scene_desc& d);
// The scene's lights: light_list when set, else the inline array.
inline const sf_area_light* scene_lights(const sf_scene_desc& d) { return d.light_list ? d.light_list : d.lights; }
inline uint32_t scene_light_count(const sf_scene_desc& d) {
    return d.light_list ? d.light_list_count : std::min<uint32_t>(d.light_count, SF_MAX_LIGHTS);
}
// Lights SF_SHARED_LIGHTS.. of the scene, packed for the device light table.
void scene_lights_dev(const sf_scene_desc& d, std::vector<DevLight>& more);
// Panorama tables (sf_environment.cpp) and an HDRI light's device fields.
sf_status environment_tables(const float* rgb, uint32_t width, uint32_t height, std::vector<float>& texels,
                             uint32_t& ow, uint32_t& oh, bool& uniform);
void environment_dev(const sf_environment* e, DevLight& o);
bool has_hdri(const sf_scene_desc& d);
sf_status check_launch(uint32_t min_blocks, uint32_t quantum, uint32_t regen, bool small_blocks);
void planar_dev(const sf_planar_desc& f, PlanarDev& o);
sf_status planar_check(const sf_planar_desc* f);
cudaError_t film_readback(sf_context* c, const FilmPlanes& f, const sf_film_planes& out, cudaStream_t st);
// Fog scenes keep the film's volume layer split (volume, moments and surface planes).
inline bool has_fog(const sf_scene_desc& d) { return d.fog.density > 0.0f; }
// DevScene.rich of a scene: finish details, a texture, optics (SF_RICH_* bits).
inline uint32_t rich_of(const sf_scene_desc& d) {
    uint32_t r = 0;
    const uint32_t nf = d.finish_count < SF_MAX_FINISHES ? d.finish_count : SF_MAX_FINISHES;
    for (uint32_t i = 0; i < nf; ++i)
        if (d.details[i].pattern) r |= SF_RICH_DETAIL | (d.details[i].pattern >= 10 ? SF_RICH_ROUGH_DIFFUSE : 0u);
    for (uint32_t i = 0; i <= nf; ++i)
        if (d.optics[i].enabled) r |= SF_RICH_OPTICS;
    if (d.texture.graph) r |= SF_RICH_TEXTURE;
    return r;
}
// Wavefront rounds of a dispatch: every bounce, one round to resolve the last shadow
// segments and, with optics, the 32 coverage null events a path may take without a
// bounce (the reference sizes its wavefront the same way, session.rs:397-405).
inline uint32_t rounds_of(const sf_render_config& c, const sf_scene_desc& d) {
    return c.max_bounces + 2 + ((rich_of(d) & SF_RICH_OPTICS) ? 33u : 0u);
}

// Wavefront path state for N paths with K shadow slots (a bounce issues at most K
// shadow segments): eight path planes, K sets of shadow planes and visibility words,
// march rows for the continuation (row = path) and each shadow (row = N + k*N + path),
// round lists (active, continuation, K*N shadow rows) in two parities, and two
// resume lists of (1 + K) * N items.
inline size_t wave_soa_bytes(size_t N, uint32_t K) { return N * 16 * 8 + size_t(K) * N * (16 * 3 + 4); }
inline size_t wave_march_bytes(size_t N, uint32_t K) { return (1 + size_t(K)) * N * (16 + 16 + 4); }
inline size_t wave_lists_bytes(size_t N, uint32_t K) { return 2 * (2 + size_t(K)) * N * 4; }
inline size_t wave_resume_bytes(size_t N, uint32_t K) { return 2 * (1 + size_t(K)) * N * 4; }
inline void wave_bind(PathSoA& soa, void* soa_mem, void* march_mem, uint32_t N, uint32_t K) {
    float4* p = static_cast<float4*>(soa_mem);
    soa.o = p; p += N;
    soa.d = p; p += N;
    soa.tp = p; p += N;
    soa.L = p; p += N;
    soa.pn = p; p += N;
    soa.hit = reinterpret_cast<uint4*>(p); p += N;
    soa.hit_tr = p; p += N;
    soa.hit_n = p; p += N;
    soa.sh_o = p; p += size_t(K) * N;
    soa.sh_d = p; p += size_t(K) * N;
    soa.sh_c = p; p += size_t(K) * N;
    soa.vis = reinterpret_cast<uint32_t*>(p);
    float4* m = static_cast<float4*>(march_mem);
    const size_t rows = (1 + size_t(K)) * N;
    soa.m0 = m;
    soa.m1 = m + rows;
    soa.m2 = reinterpret_cast<uint32_t*>(m + 2 * rows);
    soa.capacity = N;
    soa.shadow_slots = K;
}
inline void wave_round_queues(RoundQueues& q, uint32_t* lists, size_t N, uint32_t K, uint32_t r, uint32_t* counts) {
    const size_t stride = (2 + size_t(K)) * N;
    uint32_t* cur = lists + (r & 1) * stride;
    uint32_t* nxt = lists + ((r & 1) ^ 1) * stride;
    q.active = r == 0 ? nullptr : cur;
    q.cont = r == 0 ? nullptr : cur + N;
    q.shadow = cur + 2 * N;
    q.counts = counts + 4 * r;
    q.next_active = nxt;
    q.next_cont = nxt + N;
    q.next_shadow = nxt + 2 * N;
    q.next_counts = counts + 4 * (r + 1);
    q.work_counter = counts + 4 * r + 3;
}
inline uint32_t* wave_resume(uint32_t* resume, size_t N, uint32_t K, uint32_t parity) {
    return resume + size_t(parity & 1) * (1 + size_t(K)) * N;
}

// Device storage of one batched wavefront: the job table, path state and queues.
struct WaveArena {
    BatchTable bt{};
    PathSoA soa{};
    uint32_t capacity = 0, rounds = 0, max_steps = 0, max_jobs = 0;
    uint32_t* lists = nullptr;
    uint32_t* resume = nullptr;
    uint32_t* counts = nullptr;
    uint32_t* qcounts = nullptr;
    uint32_t* status = nullptr;
    void* mem = nullptr;
    size_t mem_bytes = 0;
    bool any_generic = false;
    uint32_t rich = 0;  // SF_RICH_* of any job: the shading and trace kernels' features
    uint32_t min_blocks = 3, quantum = 128, regen = 4;
};

sf_status arena_alloc(sf_context* c, WaveArena& a, uint32_t capacity, uint32_t max_jobs, uint32_t rounds,
                      uint32_t shadow_slots, size_t extra_bytes, size_t* extra_offset);
sf_status wave_record_pass(sf_context* c, const WaveArena& a, cudaStream_t st, bool timed);

}  // namespace sfh

// A render session (RenderSession, session.rs:165): scene constants, film and path state.
struct sf_session {
    sf_context* ctx = nullptr;
    sf_graph* graph = nullptr;
    sf_scene_desc scene;
    std::vector<sf_area_light> light_store;  // the session's copy of scene.light_list
    uint32_t light_smem = 0;                  // dynamic shared bytes of its lights past SF_SHARED_LIGHTS
    sf_render_config cfg;
    DevScene* d_scene = nullptr;
    FilmPlanes film{};
    PathSoA soa{};
    uint32_t capacity = 0;
    uint32_t* lists = nullptr;     // 2 x {active, cont, shadow} x capacity
    uint32_t* resume = nullptr;    // 2 x 2*capacity segments cut at a step quantum
    uint32_t* qcounts = nullptr;   // per round and launch: {work counter, resumed count}
    uint32_t* counts = nullptr;    // per round: {active, cont, shadow, work}
    uint32_t* status = nullptr;
    void* mem = nullptr;
    size_t mem_bytes = 0;
    std::vector<sf_tile> tiles;
    uint32_t tile_size = 0, dispatches = 0;
    uint32_t min_blocks = 7, quantum = 0, regen = 4;  // 7 blocks of 128 threads per SM
    uint32_t status_host = 0;
    double ms_per_path = 0.0;  // measured device cost of a path, for step() pacing
    bool window = false;       // tiled export: a tile-sized film whose origin the export sets
    uint32_t shadow_slots = 1; // shadow segments a bounce may issue (1 + suns + skies)
};

namespace sfh {

sf_status session_alloc(sf_session* s);
void tile_grid(sf_session* s);

// Checkpoint files: plain binary records, FNV-1a checksums, a producer identity,
// and a sibling directory swapped into place (session.rs:33-45, :1194-1346).
uint64_t fnv1a(const void* data, size_t n, uint64_t h = 0xcbf29ce484222325ull);
std::string producer_of(const sf_context* c);
bool write_file(const std::string& path, const std::vector<uint8_t>& data);
bool read_file(const std::string& path, std::vector<uint8_t>& data);
void remove_tree(const std::string& dir);
sf_status install_checkpoint(const std::string& final_dir,
                             const std::vector<std::pair<std::string, const std::vector<uint8_t>*>>& files);
struct Writer {
    std::vector<uint8_t> buf;
    template <class T> void put(const T& v) {
        const uint8_t* p = reinterpret_cast<const uint8_t*>(&v);
        buf.insert(buf.end(), p, p + sizeof(T));
    }
    void put_bytes(const void* p, size_t n) {
        const uint8_t* q = static_cast<const uint8_t*>(p);
        buf.insert(buf.end(), q, q + n);
    }
    void put_str(const std::string& s) { put(uint32_t(s.size())); put_bytes(s.data(), s.size()); }
};
struct Reader {
    const std::vector<uint8_t>& buf;
    size_t pos = 0;
    bool ok = true;
    template <class T> T get() {
        T v{};
        if (pos + sizeof(T) > buf.size()) { ok = false; return v; }
        std::memcpy(&v, buf.data() + pos, sizeof(T));
        pos += sizeof(T);
        return v;
    }
    void get_bytes(void* p, size_t n) {
        if (pos + n > buf.size()) { ok = false; return; }
        std::memcpy(p, buf.data() + pos, n);
        pos += n;
    }
    std::string get_str() {
        uint32_t n = get<uint32_t>();
        if (!ok || pos + n > buf.size()) { ok = false; return ""; }
        std::string s(reinterpret_cast<const char*>(buf.data() + pos), n);
        pos += n;
        return s;
    }
};

}  // namespace sfh

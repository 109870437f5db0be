// Launch parameter blocks and host-callable launchers of sf_kernels.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "sf_program.h"

// Path flags kept in the path state.
enum { SF_PF_CONT = 1u, SF_PF_SHADOW = 2u, SF_PF_FROM_BSDF = 4u, SF_PF_FROM_VOLUME = 8u };
// PathSoA.ex.z bits above the medium slot.
enum { SF_EX_SOLID = 1u << 8, SF_EX_INIT = 1u << 9 };
#define SF_PF_SHADOW_SHIFT 8  // bits 8..15 of the flags: which shadow slots hold a segment
// Hit record flags.
enum { SF_HF_HIT = 1u, SF_HF_EXHAUSTED = 2u };
// Wavefront invariant word (wavefront.wgsl:183/:220/:236 bits 1, 2, 4).
enum { SF_WF_QUEUE_OVERFLOW = 1u, SF_WF_COMPACT_OVERFLOW = 2u, SF_WF_ALIVE_AT_COMMIT = 4u, SF_WF_SHADOW_OVERFLOW = 8u };

// Statistics accumulated by the trace kernels (64-bit device counters).
// WARP_DE_CALLS counts warp-level DE invocations; ITER_SLOTS sums, per invocation,
// the warp's largest iteration count times its active lanes (SIMT efficiency:
// DE_EVALS / (32 * WARP_DE_CALLS) and DE_ITERS / ITER_SLOTS).
enum { SF_STAT_DE_EVALS = 0, SF_STAT_DE_ITERS, SF_STAT_SEGMENTS, SF_STAT_STEPS, SF_STAT_SHADOW_SEGMENTS,
       SF_STAT_WARP_DE_CALLS, SF_STAT_ITER_SLOTS, SF_STAT_WARP_CYCLES, SF_STAT_TAIL_CYCLES, SF_STAT_COUNT = 10 };

// Structure-of-arrays path storage for one dispatch of `capacity` paths.
struct PathSoA {
    float4* o;       // ray origin, w = prev_pdf
    float4* d;       // ray direction, w = prev_area_total
    float4* tp;      // throughput, w = bits(rng)
    float4* L;       // radiance, w = bits(bounce | flags << 16)
    float4* pn;      // prev normal, w unused
    float4* sh_o;    // shadow origin, w = t_end
    float4* sh_d;    // shadow direction
    float4* sh_c;    // radiance carried by the shadow segment if clear
    uint4* hit;      // (bits(t), steps, light_index, flags)
    float4* hit_tr;  // normalised traps
    float4* hit_n;   // normal, w = bits(iterations | material << 16)
    uint32_t* vis;   // shadow visibility (1 = clear)
    float4* Ls;      // per-path final radiance (committed in ascending sample order)
    // resumable march state of a segment cut at the step quantum: continuation rows
    // [0, capacity), shadow rows capacity + [0, K * capacity)
    float4* m0;      // t, omega, prev_radius, step_len
    float4* m1;      // t_end, cand_t, cand_err, bits(steps)
    uint32_t* m2;    // light index ahead of the segment
    // fog scenes only (null otherwise): primary volume xyz, w = bits(volume tags of the
    // pending shadow slots | the camera segment scattered << 8); the sample's volume
    // part once the path ends
    float4* pv;
    // scenes with finish details, a texture or optics only (null otherwise): x = the
    // transported texture width, y = its spread, z = bits(medium slot | inside a solid
    // medium << 8 | initial medium pending << 9), w = bits(coverage null events taken)
    float4* ex;
    uint32_t capacity;
    uint32_t shadow_slots;  // K: sh_o/sh_d/sh_c/vis have K * capacity rows (row = k * capacity + path)
};

// Queues of one round: active paths, continuation rays, shadow rays (ids),
// with their counts in `counts[0..2]`; next round's lists are written by shade.
struct RoundQueues {
    const uint32_t* active;   // null: identity (round 0)
    const uint32_t* cont;     // null: identity (round 0)
    const uint32_t* shadow;
    const uint32_t* counts;   // [active, cont, shadow]
    uint32_t* next_active;
    uint32_t* next_cont;
    uint32_t* next_shadow;
    uint32_t* next_counts;    // [active, cont, shadow]
    uint32_t* work_counter;   // trace kernel fetch counter (zeroed per round)
};

// One launch of the persistent trace kernel: the round's fresh segments
// (continuations then shadows) or the segments resumed after a step quantum.
// Item encoding: continuation lists hold paths, shadow lists shadow rows
// (k * capacity + path); resume lists hold path or shadow row | (shadow ? 1u << 31 : 0).
struct TraceLaunch {
    RoundQueues q;
    const uint32_t* resume;       // null on the first launch of a round
    const uint32_t* resume_count;
    uint32_t* next_resume;        // segments cut at this launch's quantum
    uint32_t* next_resume_count;
    uint32_t* work_counter;
    uint32_t quantum;             // march steps per segment per launch (0 = unbounded)
    uint32_t regen;               // idle lanes a warp waits for before it takes new segments (1..32)
    uint32_t lane_stats;          // 1: count warp-level DE calls and iteration slots (diagnostic kernel)
    uint32_t optics;              // 1: the scene has dielectric materials (the optics trace kernel)
};

struct FilmPlanes {
    float4* accum;  // sum of (L, 1) per sample
    float* depth;   // first-hit distance, -1 for a miss (sample 0)
    float4* aux;    // first-hit normal and steps (sample 0)
    // the volume layer split of fog scenes (null otherwise): sums of (volume, 1), their
    // Welford moments, sums of (radiance - volume, 1)
    float4* vol;
    float4* vmom;
    float4* surf;
    uint32_t width, height;
    uint32_t x0, y0;  // image pixel of the planes' first element (a window film; 0, 0 for the image)
};
__device__ __forceinline__ size_t film_index(const FilmPlanes& f, uint32_t px, uint32_t py) {
    return (size_t)(py - f.y0) * f.width + (px - f.x0);
}

struct DispatchGeom {
    uint32_t tile_x, tile_y, tile_w, tile_h;
    uint32_t sample_start, samples;
    uint32_t paths;  // tile_w * tile_h * samples
    uint32_t light_smem;  // dynamic shared bytes: the scene's lights past SF_SHARED_LIGHTS
};

// stripe_k: the stripe count as an integer (|k| <= 64), else SF_STRIPES_GENERAL;
// bail_t: the largest float whose correctly rounded square root is <= bailout.
#define SF_STRIPES_GENERAL 0x7fffffff
struct PlanarDev {
    uint32_t family, power, iterations;
    int32_t stripe_k;
    float julia[2], center[2];
    float zoom, inversion, relaxation, memory, bailout, trap_radius, stripes;
    float angle_cos, angle_sin, twist_cos, twist_sin;
    float bail_t;
};

struct CanvasDev {
    float center[2], zoom, aspect, rot_cos, rot_sin;
    uint32_t width, height, seed;
};

// One job of a batched wavefront: its graph, scene, film and tile, and where its
// paths and pixels start in the batch's shared index spaces. Lives in device memory
// (the graph replay advances sample_start there).
struct BatchJob {
    const DeProgram* prog;
    const DevScene* scene;
    FilmPlanes film;
    DispatchGeom geom;
    uint32_t path_begin;
    uint32_t pixel_begin;
    uint32_t form;
    uint32_t pad;
};
#define SF_BATCH_MAX_JOBS 1024
struct BatchTable {
    BatchJob* jobs;
    uint32_t n_jobs;
    uint32_t total_paths;
    uint32_t total_pixels;
    uint32_t pad;
};

// ---- launchers (return cudaError_t of the launch) ----
cudaError_t sf_launch_de_probe(const DeProgram* prog, const float* x, const float* y, const float* z, size_t n,
                               float* dist, float* traps, uint32_t* iters, uint32_t* mats, cudaStream_t st);
cudaError_t sf_launch_primary(const DeProgram* prog, const DevScene* scene, uint32_t width, uint32_t height,
                              uint32_t max_steps, int rule, float eps, float t_far, int normal_mode, float* t_out,
                              uint32_t* steps_out, float* normal_out, uint32_t* work_counter,
                              unsigned long long* stats, int persistent, cudaStream_t st);
cudaError_t sf_launch_generate(const DevScene* scene, PathSoA soa, DispatchGeom g, uint32_t* counts, cudaStream_t st);
// Persistent trace kernel, one instantiation per form (sf_trace_<form>.cu).
cudaError_t sf_launch_trace(uint32_t form, const DeProgram* prog, const DevScene* scene, PathSoA soa, TraceLaunch tl,
                            unsigned long long* stats, int blocks, int min_blocks, uint32_t light_smem, cudaStream_t st);
cudaError_t sf_launch_trace_bulb(const DeProgram*, const DevScene*, PathSoA, TraceLaunch, unsigned long long*, int, int, uint32_t,
                                 cudaStream_t);
cudaError_t sf_launch_trace_box(const DeProgram*, const DevScene*, PathSoA, TraceLaunch, unsigned long long*, int, int, uint32_t,
                                cudaStream_t);
cudaError_t sf_launch_trace_menger(const DeProgram*, const DevScene*, PathSoA, TraceLaunch, unsigned long long*, int,
                                   int, uint32_t, cudaStream_t);
cudaError_t sf_launch_trace_any(const DeProgram*, const DevScene*, PathSoA, TraceLaunch, unsigned long long*, int, int, uint32_t,
                                cudaStream_t);
// Batched wavefront (sf_batch.cu): all jobs' paths in one set of launches.
cudaError_t sf_launch_generate_batch(BatchTable bt, PathSoA soa, uint32_t* counts, cudaStream_t st);
cudaError_t sf_launch_trace_batch(BatchTable bt, PathSoA soa, TraceLaunch tl, unsigned long long* stats, int blocks,
                                  int min_blocks, int any_generic, cudaStream_t st);
cudaError_t sf_launch_shade_batch(BatchTable bt, uint32_t rich, PathSoA soa, RoundQueues q, uint32_t* status, int final_round,
                                  cudaStream_t st);
cudaError_t sf_launch_commit_batch(BatchTable bt, PathSoA soa, cudaStream_t st);
cudaError_t sf_launch_advance_batch(BatchTable bt, cudaStream_t st);
cudaError_t sf_launch_shade(const DevScene* scene, uint32_t rich, PathSoA soa, RoundQueues q, DispatchGeom g, FilmPlanes film,
                            uint32_t* status, int final_round, cudaStream_t st);
cudaError_t sf_launch_commit(PathSoA soa, DispatchGeom g, FilmPlanes film, cudaStream_t st);

// The preview machine's per-pixel state and outputs (one row per pixel).
struct PreviewState {
    float4* march;  // t, omega, previous radius, step length
    float4* grad;   // tap gradient xyz, tap offset
    uint2* tags;    // state (0 march, 2..5 taps, 6 done, 8 error), march steps
};
struct PreviewOut {
    float4* accum;  // preview colour, 1
    float* depth;   // hit distance, -1 until hit (and on a miss)
    float4* aux;    // normal, march steps (-1 until hit)
};
// One quantum (at most `quantum` DE evaluations per pixel); init starts every pixel
// over. status[0] += pixels still open, status[2] += pixels that met an error.
cudaError_t sf_launch_preview(const DeProgram* prog, const DevScene* scene, uint32_t pixels, PreviewState st,
                              PreviewOut out, uint32_t quantum, uint32_t init, uint32_t* status, cudaStream_t s);
cudaError_t sf_launch_film_clear(FilmPlanes film, cudaStream_t st);
cudaError_t sf_launch_megakernel(const DeProgram* prog, const DevScene* scene, uint32_t rich, PathSoA soa, DispatchGeom g,
                                 FilmPlanes film, unsigned long long* stats, cudaStream_t st);
cudaError_t sf_launch_planar(const PlanarDev* f, const float* x, const float* y, size_t n, float* dist, float* traps,
                             uint32_t* iters, cudaStream_t st);
// with_traps = 0 writes only dist, traps[0 .. n) (smooth time) and iters. *work is
// the tile's pixel counter and must be 0 when the launch starts; root != 0 for the
// Newton and Nova families (planar family 3 and 4).
cudaError_t sf_launch_escape2d(const PlanarDev* f, const CanvasDev* canvas, uint32_t tile_x, uint32_t tile_y,
                               uint32_t tile_w, uint32_t tile_h, uint32_t sample, float* dist, float* traps,
                               uint32_t* iters, unsigned long long* stats, uint32_t* work, int with_traps, int root,
                               cudaStream_t st);
// orbit_f[n] = float(Z_n), orbit_lo[n] = float(Z_n - orbit_f[n]), n < *orbit_len <= max_iter + 1.
cudaError_t sf_launch_ref_orbit(double cx, double cy, uint32_t max_iter, double bailout, float2* orbit_lo,
                                float2* orbit_f, uint32_t* orbit_len, cudaStream_t st);
// The same orbit in two launches: the serial FP64 recurrence into z (max_iter + 4
// entries), then its parallel split into the hi/lo arrays.
cudaError_t sf_launch_ref_orbit_split(double cx, double cy, uint32_t max_iter, double bailout, double2* z,
                                      float2* orbit_lo, float2* orbit_f, uint32_t* orbit_len, cudaStream_t st);
// *work is the pixel counter of the launch and must be 0 when it starts. c_lo: the
// centre's part below the orbit's c_ref, added to every pixel's offset.
cudaError_t sf_launch_perturb(const float2* orbit_lo, const float2* orbit_f, const uint32_t* orbit_len, uint32_t width,
                              uint32_t height, float pitch, float2 c_lo, uint32_t max_iter, float bailout,
                              uint32_t* iters, float* smooth, unsigned long long* stats, uint32_t* work,
                              cudaStream_t st);
cudaError_t sf_launch_direct_f64(double cx, double cy, double lox, double loy, uint32_t width, uint32_t height,
                                 double pitch, uint32_t max_iter, double bailout, uint32_t* iters, float* smooth,
                                 cudaStream_t st);
int sf_device_sm_count();
cudaError_t sf_launch_ffma_peak(float* out, uint32_t iters, int blocks, cudaStream_t st);

// Batched wavefront over many jobs (scenes, graphs, tile sizes, sample counts) in
// one set of launches: every stage indexes one shared path space and finds each
// path's job by binary search over the jobs' first paths. The job table is device
// memory, so a captured CUDA graph can be replayed with advancing sample indices.
#include "sf_stages.cuh"
#include "sf_trace_kernel.cuh"

static __device__ __forceinline__ void stage_begins(uint32_t* begins, const BatchTable& bt, bool pixels) {
    for (uint32_t i = threadIdx.x; i < bt.n_jobs; i += blockDim.x)
        begins[i] = pixels ? bt.jobs[i].pixel_begin : bt.jobs[i].path_begin;
    __syncthreads();
}

__global__ void __launch_bounds__(256) k_generate_batch(BatchTable bt, PathSoA soa, uint32_t* counts) {
    __shared__ uint32_t begins[SF_BATCH_MAX_JOBS];
    stage_begins(begins, bt, false);
    uint32_t path = blockIdx.x * blockDim.x + threadIdx.x;
    if (path == 0) {
        counts[0] = bt.total_paths;
        counts[1] = bt.total_paths;
        counts[2] = 0;
    }
    if (path >= bt.total_paths) return;
    const BatchJob& job = bt.jobs[find_job(begins, bt.n_jobs, path)];
    generate_path(*job.scene, soa, job.geom, path - job.path_begin, path);
}

// FEAT: the surface features the kernel is built with (SF_FEAT_*; 0 when no job has any).
template <int FEAT>
__global__ void __launch_bounds__(256) k_shade_batch(BatchTable bt, PathSoA soa, RoundQueues q, uint32_t* status,
                                                     int final_round) {
    __shared__ uint32_t begins[SF_BATCH_MAX_JOBS];
    stage_begins(begins, bt, false);
    const uint32_t n = q.counts[0];
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        uint32_t path = q.active ? q.active[j] : j;
        const BatchJob& job = bt.jobs[find_job(begins, bt.n_jobs, path)];
        uint32_t nf = shade_path<FEAT>(*job.scene, soa, job.geom, job.film, path - job.path_begin, path, status,
                                       final_round);
        if (!final_round) enqueue_next(q, soa, nf, path);
    }
}

__global__ void __launch_bounds__(256) k_commit_batch(BatchTable bt, PathSoA soa) {
    __shared__ uint32_t begins[SF_BATCH_MAX_JOBS];
    stage_begins(begins, bt, true);
    uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= bt.total_pixels) return;
    const BatchJob& job = bt.jobs[find_job(begins, bt.n_jobs, pix)];
    commit_pixel(soa, job.geom, job.film, pix - job.pixel_begin, job.path_begin);
}

// After a pass: every job's next pass starts at the following samples.
__global__ void k_advance_batch(BatchTable bt) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < bt.n_jobs) bt.jobs[i].geom.sample_start += bt.jobs[i].geom.samples;
}

static unsigned blocks_for(size_t n) { return (unsigned)((n + 255) / 256 > 0 ? (n + 255) / 256 : 1); }

cudaError_t sf_launch_generate_batch(BatchTable bt, PathSoA soa, uint32_t* counts, cudaStream_t st) {
    k_generate_batch<<<blocks_for(bt.total_paths), 256, 0, st>>>(bt, soa, counts);
    return cudaGetLastError();
}
cudaError_t sf_launch_shade_batch(BatchTable bt, uint32_t rich, PathSoA soa, RoundQueues q, uint32_t* status,
                                  int final_round, cudaStream_t st) {
    unsigned cap = (unsigned)sf_device_sm_count() * 16u;
    unsigned b = blocks_for(bt.total_paths);
    b = b < cap ? b : cap;
    if (rich & SF_RICH_TEXTURE) k_shade_batch<3><<<b, 256, 0, st>>>(bt, soa, q, status, final_round);
    else if (rich) k_shade_batch<1><<<b, 256, 0, st>>>(bt, soa, q, status, final_round);
    else k_shade_batch<0><<<b, 256, 0, st>>>(bt, soa, q, status, final_round);
    return cudaGetLastError();
}
cudaError_t sf_launch_commit_batch(BatchTable bt, PathSoA soa, cudaStream_t st) {
    k_commit_batch<<<blocks_for(bt.total_pixels), 256, 0, st>>>(bt, soa);
    return cudaGetLastError();
}
cudaError_t sf_launch_advance_batch(BatchTable bt, cudaStream_t st) {
    k_advance_batch<<<blocks_for(bt.n_jobs), 256, 0, st>>>(bt);
    return cudaGetLastError();
}

template <int FORM>
static cudaError_t launch_trace_batch_form(BatchTable bt, PathSoA soa, TraceLaunch tl, unsigned long long* stats,
                                           int blocks, int min_blocks, cudaStream_t st) {
    if (tl.optics) {  // a job with dielectric materials: the optics instantiation, 2 blocks per SM
        k_trace<FORM, 2, true, false, true><<<blocks, 256, 0, st>>>(nullptr, nullptr, soa, tl, stats, bt);
        return cudaGetLastError();
    }
    switch (min_blocks) {
    case 3: k_trace<FORM, 3, true><<<blocks, 256, 0, st>>>(nullptr, nullptr, soa, tl, stats, bt); break;
    case 4: k_trace<FORM, 4, true><<<blocks, 256, 0, st>>>(nullptr, nullptr, soa, tl, stats, bt); break;
    default: k_trace<FORM, 2, true><<<blocks, 256, 0, st>>>(nullptr, nullptr, soa, tl, stats, bt); break;
    }
    return cudaGetLastError();
}

cudaError_t sf_launch_trace_batch(BatchTable bt, PathSoA soa, TraceLaunch tl, unsigned long long* stats, int blocks,
                                  int min_blocks, int any_generic, cudaStream_t st) {
    if (min_blocks < 2 || min_blocks > 4) min_blocks = 2;
    if (blocks <= 0) blocks = sf_device_sm_count() * min_blocks;
    if (any_generic) return launch_trace_batch_form<SF_FORM_ANY>(bt, soa, tl, stats, blocks, min_blocks, st);
    return launch_trace_batch_form<SF_FORM_MIXED>(bt, soa, tl, stats, blocks, min_blocks, st);
}

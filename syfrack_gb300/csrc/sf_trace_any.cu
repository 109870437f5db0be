// Persistent trace kernel instantiated for the any form (see sf_trace_kernel.cuh).
#include "sf_trace_kernel.cuh"

cudaError_t sf_launch_trace_any(const DeProgram* prog, const DevScene* scene, PathSoA soa, TraceLaunch tl,
                               unsigned long long* stats, int blocks, int min_blocks, uint32_t light_smem, cudaStream_t st) {
    return launch_trace_form<SF_FORM_ANY>(prog, scene, soa, tl, stats, blocks, min_blocks, light_smem, st);
}

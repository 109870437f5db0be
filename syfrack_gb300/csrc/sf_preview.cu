// The interactive preview machine (the reference's control engine,
// crates/syfrack-render/src/control/mod.rs and shaders/control.wgsl:54-135, 266-303):
// one primary ray per pixel centre, marched on the exact field in resumable quanta
// of DE evaluations, four tetrahedral taps at the hit, and a fixed preview shading.
// A ray is never abandoned at a step budget: it ends at a hit or past the scene
// extent; quanta only bound a launch.
#include <cuda_runtime.h>

#include "sf_kernels.cuh"
#include "sf_trace.cuh"
#include "sf_warp.cuh"

enum { PV_MARCH = 0, PV_TAP0 = 2, PV_DONE = 6, PV_ERROR = 8 };

__global__ void __launch_bounds__(256) k_preview(const DeProgram* __restrict__ prog_g,
                                                 const DevScene* __restrict__ scene_g, PreviewState st,
                                                 PreviewOut out, uint32_t quantum, uint32_t init, uint32_t* status) {
    __shared__ DeProgram P;
    __shared__ DevScene S;
    stage_program(P, prog_g);
    stage_pod(S, scene_g);
    __syncthreads();
    const uint32_t n = S.width * S.height;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 m;   // t, omega, previous radius, step length
    float4 g;   // gradient of the taps, tap offset
    uint2 tag;  // state, march steps
    if (init) {
        m = make_float4(0.0f, 1.2f, 0.0f, 0.0f);
        g = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        tag = make_uint2(PV_MARCH, 0u);
        out.accum[i] = make_float4(0.025f, 0.03f, 0.04f, 1.0f);
        out.depth[i] = -1.0f;
        out.aux[i] = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    } else {
        m = st.march[i];
        g = st.grad[i];
        tag = st.tags[i];
    }
    bool open = tag.x < PV_DONE;
    if (open) {
        const float3 org = ld3(S.origin);
        const uint32_t px = i % S.width, py = i / S.width;
        const float ndcx = ((float(px) + 0.5f) / float(S.width)) * 2.0f - 1.0f;
        const float ndcy = ((float(py) + 0.5f) / float(S.height)) * 2.0f - 1.0f;
        const float3 rd = normalize3(ld3(S.forward) + ld3(S.right) * (ndcx * S.tan_half) +
                                     ld3(S.up) * (-ndcy * S.tan_half / S.aspect));
        const float accept = S.pixel_cone * S.pixel_tolerance;
        const float end = S.extent;
        for (uint32_t q = 0; q < quantum && tag.x < PV_DONE; ++q) {
            float3 p = org + rd * m.x;
            if (tag.x >= PV_TAP0) p = p + tetra_offset(tag.x - PV_TAP0) * g.w;
            const float d = de_raw_exact_search(P, p).d;
            if (!(fabsf(d) <= 3.4028235e38f)) {  // an undefined distance is an evaluation error
                tag.x = PV_ERROR;
                atomicAdd(&status[2], 1u);
                break;
            }
            if (tag.x >= PV_TAP0) {
                g = make_float4(g.x + tetra_offset(tag.x - PV_TAP0).x * d, g.y + tetra_offset(tag.x - PV_TAP0).y * d,
                                g.z + tetra_offset(tag.x - PV_TAP0).z * d, g.w);
                if (tag.x < PV_TAP0 + 3) { tag.x++; continue; }
                const float3 nn = safe_normalize3(mk3(g.x, g.y, g.z));
                const float light = 0.20f + 0.80f * fmaxf(dot3(nn, normalize3(mk3(0.4f, 0.7f, 0.6f))), 0.0f);
                out.accum[i] = make_float4(0.68f * light, 0.70f * light, 0.73f * light, 1.0f);
                out.depth[i] = m.x;
                out.aux[i] = make_float4(nn.x, nn.y, nn.z, float(tag.y));
                tag.x = PV_DONE;
                break;
            }
            // the relaxed march of march_segment, without a step budget
            const float radius = fabsf(d) * S.step_scale;
            const float t = m.x;
            const bool failed = m.y > 1.0f && radius + m.z < m.w * 1.0001f;
            if (failed) { m.w -= m.y * m.w; m.y = 1.0f; }
            else m.w = radius * m.y;
            m.z = radius;
            const float err = radius * rcp_approx(fmaxf(t, 1e-6f));
            if (!failed && err < accept) {  // hit: the taps follow at this t
                g = make_float4(0.0f, 0.0f, 0.0f, fmaxf(t * S.pixel_cone * 0.5f, 1e-4f) * S.pixel_tolerance);
                tag.x = PV_TAP0;
                continue;
            }
            bool miss = false;
            if (!failed && t + m.w >= end) {
                if (radius >= end - t) miss = true;
                else { m.y = 1.0f; m.w = radius; }
            }
            if (!miss) {
                m.x += m.w;
                miss = m.x >= end;
            }
            if (miss) {
                out.accum[i] = make_float4(0.025f, 0.035f, 0.05f, 1.0f);
                tag.x = PV_DONE;
                break;
            }
            tag.y = min(tag.y, 0xfffffffeu) + 1u;
        }
        st.march[i] = m;
        st.grad[i] = g;
        st.tags[i] = tag;
        open = tag.x < PV_DONE;
    }
    // pixels still open after this quantum (one atomic per converged group of lanes)
    const uint32_t am = __activemask();
    const uint32_t ballot = __ballot_sync(am, open);
    if (lane_id() == (uint32_t)(__ffs(am) - 1) && ballot) atomicAdd(&status[0], __popc(ballot));
}

cudaError_t sf_launch_preview(const DeProgram* prog, const DevScene* scene, uint32_t pixels, PreviewState st,
                              PreviewOut out, uint32_t quantum, uint32_t init, uint32_t* status, cudaStream_t s) {
    if (!pixels) return cudaSuccess;
    k_preview<<<(pixels + 255) / 256, 256, 0, s>>>(prog, scene, st, out, quantum, init, status);
    return cudaGetLastError();
}

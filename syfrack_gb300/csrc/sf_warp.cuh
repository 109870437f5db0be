// Warp-level helpers shared by the kernels of the DE path.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "sf_program.h"

#define FULL_MASK 0xffffffffu

static __device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
static __device__ __forceinline__ uint32_t lanemask_lt() { return (1u << lane_id()) - 1u; }

// Warp-aggregated fetch of one work item per requesting lane: one atomic per warp.
static __device__ __forceinline__ uint32_t warp_fetch(uint32_t* counter, bool want) {
    uint32_t m = __ballot_sync(FULL_MASK, want);
    uint32_t base = 0;
    if (m) {
        uint32_t leader = __ffs(m) - 1;
        if (lane_id() == leader) base = atomicAdd(counter, __popc(m));
        base = __shfl_sync(FULL_MASK, base, leader);
    }
    return base + __popc(m & lanemask_lt());
}

// Warp-aggregated append under an arbitrary active mask (grid-stride tails).
static __device__ __forceinline__ void warp_append(uint32_t* counter, uint32_t* list, bool pred, uint32_t value) {
    uint32_t active = __activemask();
    uint32_t m = __ballot_sync(active, pred);
    if (!m) return;
    uint32_t leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane_id() == leader) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(active, base, leader);
    if (pred) list[base + __popc(m & lanemask_lt())] = value;
}

// Sum of a per-lane counter into a 64-bit device counter (one atomic per warp).
static __device__ __forceinline__ void warp_stat(unsigned long long* dst, unsigned long long v) {
    uint32_t active = __activemask();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(active, v, o);
    if (lane_id() == (uint32_t)(__ffs(active) - 1) && v) atomicAdd(dst, v);
}

// Stage the lowered graph (header + used ops) and scene constants in shared memory.
static __device__ void stage_program(DeProgram& dst, const DeProgram* src) {
    const uint32_t n_ops = src->n_ops;
    const size_t header = offsetof(DeProgram, ops);
    const size_t bytes = header + size_t(n_ops) * sizeof(DeOp);
    const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
    uint32_t* d = reinterpret_cast<uint32_t*>(&dst);
    for (size_t i = threadIdx.x; i < bytes / 4; i += blockDim.x) d[i] = __ldg(s + i);
    // the union leaf table after the ops
    constexpr size_t tail = offsetof(DeProgram, union_leaves) / 4, end = sizeof(DeProgram) / 4;
    for (size_t i = tail + threadIdx.x; i < end; i += blockDim.x) d[i] = __ldg(s + i);
}
template <class T> static __device__ void stage_pod(T& dst, const T* src) {
    const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
    uint32_t* d = reinterpret_cast<uint32_t*>(&dst);
    for (size_t i = threadIdx.x; i < sizeof(T) / 4; i += blockDim.x) d[i] = __ldg(s + i);
}


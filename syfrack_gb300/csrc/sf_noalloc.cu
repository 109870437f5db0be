// Deep zoom without any device allocation (sf_deep_zoom_noalloc).
//
// Some callers cannot let a library call cudaMalloc: hosts that reserve the whole
// device memory for their own pool at start-up (an embedding renderer or engine that
// hands out every byte itself), and latency-critical threads where cudaMalloc's
// implicit device-wide synchronisation is not acceptable. For them this entry point
// takes the caller's device output buffers and keeps its scratch -- the reference
// orbit as binary32 hi/lo pairs, its length and the statistics counters -- in one
// file-scope device array, held by every GPU that loads the library until exit.
#include <cuda_runtime.h>

#include <cstddef>
#include <mutex>
#include <string>

#include "../../include/syfrack_gpu.h"
#include "sf_kernels.cuh"

sf_status sf_report_error(sf_status status, const std::string& message);

namespace {

constexpr uint32_t kMaxIter = 65536;  // largest max_iter the scratch holds
constexpr int kMaxDevices = 64;

struct NoAllocScratch {
    float2 orbit_lo[kMaxIter + 4];  // the orbit and two entries past its end
    float2 orbit_f[kMaxIter + 4];
    uint32_t orbit_len;
    uint32_t work;  // pixel counter of the perturbation launch
    unsigned long long stats[SF_STAT_COUNT];
};

// 1 MB per device. In host code this name is only a stand-in for the symbol:
// kernels receive the address cudaGetSymbolAddress returns for the current device.
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

std::mutex g_mu;
NoAllocScratch* g_addr[kMaxDevices] = {};

// Device address of the scratch for the current device, looked up once per device.
sf_status scratch_address(NoAllocScratch** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return sf_report_error(SF_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return sf_report_error(SF_ERR_INVALID, "device index above 63");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return sf_report_error(SF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_addr[dev] = static_cast<NoAllocScratch*>(p);
    }
    *out = g_addr[dev];
    return SF_OK;
}

}  // namespace

extern "C" sf_status sf_deep_zoom_noalloc(const sf_deep_zoom_desc* d, uint32_t* iterations, float* smooth,
                                          void* stream) {
    if (!d || !iterations || !smooth) return sf_report_error(SF_ERR_INVALID, "null argument");
    if (!d->width || !d->height || !d->max_iter) return sf_report_error(SF_ERR_INVALID, "empty deep-zoom request");
    if (uint64_t(d->width) * d->height > (1ull << 31))
        return sf_report_error(SF_ERR_INVALID, "deep-zoom frames hold at most 2^31 pixels");
    if (d->max_iter > kMaxIter)
        return sf_report_error(SF_ERR_INVALID, "max_iter " + std::to_string(d->max_iter) +
                                                   " exceeds the allocation-free limit of 65536 iterations");
    if (!(d->bailout >= 2.0f)) return sf_report_error(SF_ERR_INVALID, "bailout must be at least 2");
    if (d->orbit_mode != SF_ORBIT_DEVICE)
        return sf_report_error(SF_ERR_INVALID, "the allocation-free deep zoom computes its orbit on the device");
    NoAllocScratch* sc = nullptr;
    sf_status s = scratch_address(&sc);
    if (s != SF_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the pixel counter and the statistics start at zero (they are adjacent); the orbit
    // and its length are written before they are read
    static_assert(offsetof(NoAllocScratch, stats) == offsetof(NoAllocScratch, work) + 4, "work | stats layout");
    cudaError_t e = cudaMemsetAsync(&sc->work, 0, 4 + sizeof(sc->stats), st);
    // the orbit of c_ref = centre hi; the centre's lo part joins every pixel's offset
    const double cx = d->center_hi[0], cy = d->center_hi[1];
    const float2 c_lo = make_float2(float(d->center_lo[0]), float(d->center_lo[1]));
    double pitch = d->width_units / double(d->width);
    if (e == cudaSuccess) e = sf_launch_ref_orbit(cx, cy, d->max_iter, d->bailout, sc->orbit_lo, sc->orbit_f,
                                                  &sc->orbit_len, st);
    if (e == cudaSuccess)
        e = sf_launch_perturb(sc->orbit_lo, sc->orbit_f, &sc->orbit_len, d->width, d->height, float(pitch), c_lo,
                              d->max_iter, d->bailout, iterations, smooth, sc->stats, &sc->work, st);
    if (e != cudaSuccess) return sf_report_error(SF_ERR_CUDA, std::string("sf_deep_zoom_noalloc: ") + cudaGetErrorString(e));
    return SF_OK;
}

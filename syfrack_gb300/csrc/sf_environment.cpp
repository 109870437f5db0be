// Panoramas for HDRI lights: EnvironmentMap::from_rgb
// (crates/syfrack-render/src/environment.rs:271-366) on the host, texels on the device.
//
// The source image is averaged over each output cell in solid angle (a small bright
// source keeps its energy when the map shrinks to 2048x1024), then each texel gets
// the cumulative share of luminance x solid angle of the importance distribution,
// computed over the texel's bilinear halo (weights 1/8, 3/4, 1/8 per axis) so that a
// nominally black neighbour of a bright source keeps some probability. A map whose
// texels are all equal is sampled uniformly.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "sf_host_internal.h"

using namespace sfh;

struct sf_environment {
    sf_context* ctx = nullptr;
    float4* texels = nullptr;
    size_t bytes = 0;
    uint32_t width = 0, height = 0;
    bool uniform = false;
};

namespace {

constexpr uint32_t kMaxWidth = 2048, kMaxHeight = 1024;  // environment.rs:17-18
constexpr uint64_t kMaxInputPixels = 8192ull * 4096ull;    // environment.rs:20
constexpr double kPi = 3.14159265358979323846;

// Solid angle of a texel row (environment.rs:387-395), stable near the poles.
double cell_area(uint32_t w, uint32_t h, uint32_t row) {
    const double top = kPi * double(row) / double(h), bottom = kPi * double(row + 1) / double(h);
    return 2.0 * kPi / double(w) * 2.0 * std::sin((top + bottom) * 0.5) * std::sin((bottom - top) * 0.5);
}

}  // namespace

namespace sfh {

sf_status environment_tables(const float* rgb, uint32_t width, uint32_t height, std::vector<float>& texels,
                             uint32_t& ow, uint32_t& oh, bool& uniform) {
    if (!rgb || width == 0 || height == 0 || uint64_t(width) * height > kMaxInputPixels)
        return fail(SF_ERR_INVALID, "invalid panorama dimensions (1x1 to 8192x4096)");
    const size_t n = size_t(width) * height * 3;
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(rgb[i])) return fail(SF_ERR_INVALID, "panorama contains non-finite radiance");
    const double scale = std::max({double(width) / kMaxWidth, double(height) / kMaxHeight, 1.0});
    ow = uint32_t(std::max(std::floor(double(width) / scale), 1.0));
    oh = uint32_t(std::max(std::floor(double(height) / scale), 1.0));
    texels.assign(size_t(ow) * oh * 4, 0.0f);
    for (uint32_t oy = 0; oy < oh; ++oy) {
        const double top = double(oy) * height / oh, bottom = double(oy + 1) * height / oh;
        for (uint32_t ox = 0; ox < ow; ++ox) {
            const double left = double(ox) * width / ow, right = double(ox + 1) * width / ow;
            double sum[3] = {0, 0, 0}, total = 0;
            const uint32_t iy1 = std::min<uint32_t>(uint32_t(std::ceil(bottom)), height);
            const uint32_t ix1 = std::min<uint32_t>(uint32_t(std::ceil(right)), width);
            for (uint32_t iy = uint32_t(std::floor(top)); iy < iy1; ++iy) {
                const double y0 = std::max(top, double(iy)) / height, y1 = std::min(bottom, double(iy + 1)) / height;
                const double latitude = std::cos(kPi * y0) - std::cos(kPi * y1);
                for (uint32_t ix = uint32_t(std::floor(left)); ix < ix1; ++ix) {
                    const double weight = latitude * (std::min(right, double(ix + 1)) - std::max(left, double(ix)));
                    const float* px = rgb + (size_t(iy) * width + ix) * 3;
                    for (int c = 0; c < 3; ++c) sum[c] += double(std::max(px[c], 0.0f)) * weight;
                    total += weight;
                }
            }
            float* t = &texels[(size_t(oy) * ow + ox) * 4];
            for (int c = 0; c < 3; ++c) t[c] = float(sum[c] / total);
        }
    }
    uniform = true;
    for (size_t i = 1; i < size_t(ow) * oh && uniform; ++i)
        for (int c = 0; c < 3; ++c)
            if (texels[i * 4 + c] != texels[c]) { uniform = false; break; }
    if (uniform) {
        texels[(size_t(ow) * oh - 1) * 4 + 3] = 1.0f;
        return SF_OK;
    }
    auto lum = [&](uint32_t row, uint32_t col) {
        const float* t = &texels[(size_t(row) * ow + col) * 4];
        return double(t[0]) * 0.2126 + double(t[1]) * 0.7152 + double(t[2]) * 0.0722;
    };
    const double halo[3][2] = {{-1, 0.125}, {0, 0.75}, {1, 0.125}};
    std::vector<double> weights(size_t(ow) * oh);
    double total = 0;
    for (uint32_t y = 0; y < oh; ++y)
        for (uint32_t x = 0; x < ow; ++x) {
            double w = 0;
            for (auto& hy : halo) {
                const int r = std::min(std::max(int(y) + int(hy[0]), 0), int(oh) - 1);
                for (auto& hx : halo) {
                    const int cc = ((int(x) + int(hx[0])) % int(ow) + int(ow)) % int(ow);
                    w += lum(uint32_t(r), uint32_t(cc)) * hx[1] * hy[1];
                }
            }
            weights[size_t(y) * ow + x] = w * cell_area(ow, oh, y);
        }
    for (double w : weights) total += w;
    double cumulative = 0;
    for (size_t i = 0; i < weights.size(); ++i) {
        cumulative += total > 0 ? weights[i] / total : cell_area(ow, oh, uint32_t(i / ow)) / (4.0 * kPi);
        texels[i * 4 + 3] = float(std::min(cumulative, 1.0));
    }
    texels[(weights.size() - 1) * 4 + 3] = 1.0f;
    return SF_OK;
}

}  // namespace sfh

extern "C" sf_status sf_environment_build(const float* rgb, uint32_t width, uint32_t height, float* texels,
                                          uint32_t* out_width, uint32_t* out_height, int* uniform) {
    std::vector<float> t;
    uint32_t ow = 0, oh = 0;
    bool u = false;
    sf_status s = environment_tables(rgb, width, height, t, ow, oh, u);
    if (s != SF_OK) return s;
    if (out_width) *out_width = ow;
    if (out_height) *out_height = oh;
    if (uniform) *uniform = u ? 1 : 0;
    if (texels) std::memcpy(texels, t.data(), t.size() * sizeof(float));
    return SF_OK;
}

extern "C" sf_status sf_environment_create(sf_context* c, const float* rgb, uint32_t width, uint32_t height,
                                           sf_environment** out) {
    if (!c || !out) return fail(SF_ERR_INVALID, "null argument");
    *out = nullptr;
    std::vector<float> t;
    uint32_t ow = 0, oh = 0;
    bool u = false;
    sf_status s = environment_tables(rgb, width, height, t, ow, oh, u);
    if (s != SF_OK) return s;
    cudaSetDevice(c->device);
    auto* e = new sf_environment();
    e->ctx = c;
    e->width = ow;
    e->height = oh;
    e->uniform = u;
    e->bytes = t.size() * sizeof(float);
    void* p = nullptr;
    s = ctx_alloc(c, e->bytes, &p);
    if (s != SF_OK) { delete e; return s; }
    e->texels = static_cast<float4*>(p);
    cudaError_t err = cudaMemcpy(e->texels, t.data(), e->bytes, cudaMemcpyHostToDevice);
    if (err != cudaSuccess) {
        ctx_free(c, e->texels, e->bytes);
        delete e;
        return cuda_fail(err, "panorama upload");
    }
    ctx_retain(c);
    *out = e;
    return SF_OK;
}

extern "C" sf_status sf_environment_destroy(sf_environment* e) {
    if (!e) return SF_OK;
    sf_context* c = e->ctx;
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();  // no launch may still read the texels
    ctx_free(c, e->texels, e->bytes);
    delete e;
    ctx_release(c);
    return SF_OK;
}

namespace sfh {
void environment_dev(const sf_environment* e, DevLight& o) {
    o.texels = reinterpret_cast<uint64_t>(e->texels);
    o.tw = e->width;
    o.th = e->height;
    o.a[2] = e->uniform ? 1.0f : 0.0f;
}
}  // namespace sfh

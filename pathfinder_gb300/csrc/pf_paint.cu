// pf_paint.cu — host side of gradient paints: the 256-texel colour ramp of
// each gradient and the per-gradient record the composite evaluates.
//
// The ramp is the reference's gradient tile (renderer/src/paint.rs:855-863):
// texel x holds Gradient::sample((x + 0.5) / 256) (content/src/gradient.rs:
// 188-211), with the stops ordered as Gradient::add keeps them (:158-164) and
// ColorU/ColorF conversions as in color/src/lib.rs:70-73, 163-171.
#include "pf_kernels.cuh"
#include "../../include/pathfinder_cuda.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace pf {

namespace {

// _mm_cvtps_epi32: round to nearest even; 0x80000000 when out of range.
int32_t cvt_rne_f(float x) {
    if (!(x >= -2147483648.0f && x < 2147483648.0f)) return INT32_MIN;
    return (int32_t)std::nearbyint(x);
}

uint32_t pack(const float c[4]) {
    uint32_t v = 0;
    for (int k = 0; k < 4; k++) v |= (uint32_t)(uint8_t)cvt_rne_f(c[k] * 255.0f) << (8 * k);  // `as u8` wraps
    return v;
}

}  // namespace

uint32_t gradient_sample(const std::vector<PFCUDAColorStop>& stops, float t) {
    if (stops.empty()) return 0;  // transparent black
    t = std::fmin(1.0f, std::fmax(0.0f, t));
    const size_t last = stops.size() - 1;
    // first stop with offset >= t that is not at offset 0
    size_t upper = std::partition_point(stops.begin(), stops.end(), [&](const PFCUDAColorStop& s) {
                       return s.offset < t || s.offset == 0.0f;
                   }) - stops.begin();
    upper = std::min(upper, last);
    const size_t lower = upper > 0 ? upper - 1 : upper;
    const PFCUDAColorStop &lo = stops[lower], &hi = stops[upper];
    const float denom = hi.offset - lo.offset;
    if (denom == 0.0f)
        return (uint32_t)lo.color.r | ((uint32_t)lo.color.g << 8) | ((uint32_t)lo.color.b << 16) |
               ((uint32_t)lo.color.a << 24);
    const float ratio = std::fmin((t - lo.offset) / denom, 1.0f);
    const float inv = 1.0f / 255.0f;
    const float a[4] = {lo.color.r * inv, lo.color.g * inv, lo.color.b * inv, lo.color.a * inv};
    const float b[4] = {hi.color.r * inv, hi.color.g * inv, hi.color.b * inv, hi.color.a * inv};
    float c[4];
    for (int k = 0; k < 4; k++) c[k] = a[k] + (b[k] - a[k]) * ratio;
    return pack(c);
}

int32_t build_gradient(const PFCUDAGradient& g, OverlayDev* out, std::vector<uint32_t>& texels, bool* opaque) {
    if (g.kind != PF_GRADIENT_LINEAR && g.kind != PF_GRADIENT_RADIAL) return PF_CUDA_ERR_INVALID;
    if (g.wrap != PF_GRADIENT_WRAP_CLAMP && g.wrap != PF_GRADIENT_WRAP_REPEAT) return PF_CUDA_ERR_INVALID;
    if (g.stop_count && !g.stops) return PF_CUDA_ERR_INVALID;
    if (texels.size() + 256 >= 0x80000000ull) return PF_CUDA_ERR_INVALID;
    std::vector<PFCUDAColorStop> stops(g.stops, g.stops + g.stop_count);
    std::stable_sort(stops.begin(), stops.end(),
                     [](const PFCUDAColorStop& a, const PFCUDAColorStop& b) { return a.offset < b.offset; });
    const uint32_t base = (uint32_t)texels.size();
    texels.resize(texels.size() + 256);
    for (int x = 0; x < 256; x++) texels[base + x] = gradient_sample(stops, ((float)x + 0.5f) / 256.0f);
    // Gradient::is_opaque (content/src/gradient.rs:215-217): every stop opaque
    // (so a gradient without stops counts as opaque, as there)
    *opaque = true;
    for (const PFCUDAColorStop& s : stops) *opaque = *opaque && s.color.a == 255;

    OverlayDev d{};
    d.kind = g.kind;
    d.wrap = g.wrap;
    d.texel_offset = base;
    d.page_w = 256;
    d.page_h = 1;
    if (g.kind == PF_GRADIENT_LINEAR) {
        // project the gradient line onto u in [0, 1] (renderer/src/paint.rs:603-612):
        // m0 = dp / |dp|^2, m13 = m0.x * -from.x + m0.y * -from.y
        const float dx = g.to.x - g.from.x, dy = g.to.y - g.from.y;
        const float l2 = dx * dx + dy * dy;
        if (l2 > 0.0f) {
            d.g[0] = dx / l2;
            d.g[1] = dy / l2;
            d.g[2] = d.g[0] * -g.from.x + d.g[1] * -g.from.y;
        }  // a degenerate line samples u = 0 (the reference divides by zero there)
    } else {
        // scene -> gradient space: Transform2F::inverse of the gradient's
        // transform (geometry/src/transform2d.rs:60-72, 294-298; paint.rs:613-616)
        const PFTransform2F& t = g.transform;
        const float det = t.m00 * t.m11 - t.m01 * t.m10;
        if (det == 0.0f) return PF_CUDA_ERR_INVALID;
        const float inv = 1.0f / det;
        const float a = inv * t.m11, b = inv * -t.m01, c = inv * -t.m10, e = inv * t.m00;
        d.g[0] = a; d.g[1] = b; d.g[3] = c; d.g[4] = e;
        d.g[2] = -(a * t.vector.x + b * t.vector.y);
        d.g[5] = -(c * t.vector.x + e * t.vector.y);
        // filter parameters as the RGBA16F metadata texture holds them
        // (renderer/src/gpu/renderer.rs:728-737, :975-980)
        d.from_x = round_f16(g.from.x);
        d.from_y = round_f16(g.from.y);
        d.vec_x = round_f16(g.to.x - g.from.x);
        d.vec_y = round_f16(g.to.y - g.from.y);
        d.r0 = round_f16(g.radius0);
        d.r1 = round_f16(g.radius1);
    }
    *out = d;
    return PF_CUDA_OK;
}

// An image pattern (content/src/pattern.rs) on its own texture page, placed
// as renderer/src/paint.rs:498-560 places it: a transparent border texel on
// each axis that does not repeat, the image inside it, page UV =
// scale(1 / page size) * inverse(pattern transform) (:617-623, with
// Transform2F::inverse and products as geometry/src/transform2d.rs:60-72,
// 115-129, 294-310 compute them); filter parameters as
// compute_filter_params writes them (renderer/src/gpu/renderer.rs:988-1040),
// rounded to binary16.
int32_t build_pattern(const PFCUDAPattern& p, OverlayDev* out, std::vector<uint32_t>& texels, bool* opaque) {
    if (!p.pixels || p.width == 0 || p.height == 0 || p.width > 16384 || p.height > 16384) return PF_CUDA_ERR_INVALID;
    if (p.flags & ~(uint32_t)(PF_PATTERN_REPEAT_X | PF_PATTERN_REPEAT_Y | PF_PATTERN_NO_SMOOTHING))
        return PF_CUDA_ERR_INVALID;
    if (p.filter < PF_PATTERN_FILTER_NONE || p.filter > PF_PATTERN_FILTER_COLOR_MATRIX) return PF_CUDA_ERR_INVALID;
    const bool blur = p.filter == PF_PATTERN_FILTER_BLUR_X || p.filter == PF_PATTERN_FILTER_BLUR_Y;
    if (blur && !(p.blur_sigma > 0.0f && p.blur_sigma <= 256.0f)) return PF_CUDA_ERR_INVALID;
    const uint32_t bx = (p.flags & PF_PATTERN_REPEAT_X) ? 0u : 1u, by = (p.flags & PF_PATTERN_REPEAT_Y) ? 0u : 1u;
    const uint32_t pw = p.width + 2 * bx, ph = p.height + 2 * by;
    if (texels.size() + (uint64_t)pw * ph >= 0x80000000ull) return PF_CUDA_ERR_INVALID;
    const PFTransform2F& t = p.transform;
    const float det = t.m00 * t.m11 - t.m01 * t.m10;
    if (det == 0.0f) return PF_CUDA_ERR_INVALID;

    const uint32_t base = (uint32_t)texels.size();
    texels.resize(texels.size() + (size_t)pw * ph, 0u);  // the border stays transparent black
    *opaque = true;  // Image::is_opaque (content/src/pattern.rs:208-212): every texel opaque
    for (uint32_t y = 0; y < p.height; y++)
        for (uint32_t x = 0; x < p.width; x++) {
            const PFColorU c = p.pixels[(size_t)y * p.width + x];
            texels[base + (size_t)(y + by) * pw + (x + bx)] =
                (uint32_t)c.r | ((uint32_t)c.g << 8) | ((uint32_t)c.b << 16) | ((uint32_t)c.a << 24);
            *opaque = *opaque && c.a == 255;
        }

    OverlayDev d{};
    d.kind = kOverlayPattern;
    d.texel_offset = base;
    d.page_w = pw;
    d.page_h = ph;
    d.flags = p.flags;
    d.filter = p.filter;
    // inverse of the pattern transform: (1/det) * adjugate, vector -(M^-1 v)
    const float r = 1.0f / det;
    const float a = r * t.m11, b = r * -t.m01, c = r * -t.m10, e = r * t.m00;
    const float vx = -(a * t.vector.x + b * t.vector.y), vy = -(c * t.vector.x + e * t.vector.y);
    // scale(1 / page size) * inverse, with the zero terms of the 2x2 products
    const float sx = 1.0f / (float)pw, sy = 1.0f / (float)ph;
    d.g[0] = sx * a + 0.0f * c;
    d.g[1] = sx * b + 0.0f * e;
    d.g[3] = 0.0f * a + sy * c;
    d.g[4] = 0.0f * b + sy * e;
    d.g[2] = (sx * vx + 0.0f * vy) + 0.0f;
    d.g[5] = (0.0f * vx + sy * vy) + 0.0f;
    if (blur) {
        const float sigma_inv = 1.0f / p.blur_sigma;
        const float gx = 0.3989422804014327f * sigma_inv;  // 1 / sqrt(2 pi)
        const float gy = std::exp(-0.5f * sigma_inv * sigma_inv);
        const float gz = gy * gy;
        const float support = std::ceil(1.5f * p.blur_sigma) * 2.0f;
        d.blur[0] = p.filter == PF_PATTERN_FILTER_BLUR_X ? 1.0f : 0.0f;
        d.blur[1] = p.filter == PF_PATTERN_FILTER_BLUR_Y ? 1.0f : 0.0f;
        d.blur[2] = round_f16(support);
        d.blur[3] = round_f16(gx);
        d.blur[4] = round_f16(gy);
        d.blur[5] = round_f16(gz);
    } else if (p.filter == PF_PATTERN_FILTER_COLOR_MATRIX) {
        for (int k = 0; k < 20; k++) d.matrix[k] = round_f16(p.color_matrix[k]);
    }
    *out = d;
    return PF_CUDA_OK;
}

}  // namespace pf

namespace {
std::vector<PFCUDAColorStop> ordered_stops(const PFCUDAGradient& g) {
    std::vector<PFCUDAColorStop> stops(g.stops, g.stops + g.stop_count);
    std::stable_sort(stops.begin(), stops.end(),
                     [](const PFCUDAColorStop& a, const PFCUDAColorStop& b) { return a.offset < b.offset; });
    return stops;
}
PFColorU to_color(uint32_t v) {
    return PFColorU{(uint8_t)(v & 0xffu), (uint8_t)((v >> 8) & 0xffu), (uint8_t)((v >> 16) & 0xffu),
                    (uint8_t)(v >> 24)};
}
}  // namespace

extern "C" int32_t PFCUDAGradientSample(const PFCUDAGradient* gradient, float t, PFColorU* out) {
    if (!gradient || !out || (gradient->stop_count && !gradient->stops)) return PF_CUDA_ERR_INVALID;
    *out = to_color(pf::gradient_sample(ordered_stops(*gradient), t));
    return PF_CUDA_OK;
}

extern "C" int32_t PFCUDAGradientRamp(const PFCUDAGradient* gradient, PFColorU* out_256) {
    if (!gradient || !out_256 || (gradient->stop_count && !gradient->stops)) return PF_CUDA_ERR_INVALID;
    const std::vector<PFCUDAColorStop> stops = ordered_stops(*gradient);
    for (int x = 0; x < 256; x++) out_256[x] = to_color(pf::gradient_sample(stops, ((float)x + 0.5f) / 256.0f));
    return PF_CUDA_OK;
}

// pf_oracle.cpp — TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// A CPU restatement of Pathfinder's CPU tiling path (the D3D9 level's scene
// builder) plus an FP64 evaluation of its coverage formula, mask resolve and
// SrcOver composite.  It is the parity oracle for the CUDA renderer and, in its
// FP32 multi-threaded form, the timed CPU baseline.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
//
// Parity pins: the reference has no tests for the tiler or the fill shaders,
// so the tiler arithmetic is pinned only by hand-derived known-answer cases
// (tests/test_oracle_kat.py) and the coverage formula by the reference's own
// area LUT (resources/textures/area-lut.png, checked in tests/golden/).  The
// Rust original cannot be compiled here (no cargo/rustc).
//
// Arithmetic follows the reference's SSE4.1 lane semantics
// (simd/src/x86/mod.rs): separate IEEE single-precision adds/multiplies/divides
// (build with -ffp-contract=off), _mm_min_ps/_mm_max_ps operand order,
// _mm_floor_ps, and _mm_cvtps_epi32 (round to nearest even; 0x80000000 when
// out of range).
//
// Alpha tile IDs: the reference allocates them with a global fetch_add whose
// order depends on the Rayon schedule (renderer/src/gpu_data.rs:449-454).  Here
// they are numbered canonically: global tile order (clip paths, then draw
// paths; each path row-major over its tile rect), counting only tiles that
// received a fill.  The CUDA level numbers them the same way.

#include "../include/pathfinder_cuda.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// SSE lane semantics (simd/src/x86/mod.rs)
// ---------------------------------------------------------------------------
inline float sse_min(float a, float b) { return a < b ? a : b; }  // _mm_min_ps :247-249
inline float sse_max(float a, float b) { return a > b ? a : b; }  // _mm_max_ps :252-254
inline float sse_clamp(float x, float lo, float hi) {             // clamp :257-259
    return sse_min(sse_max(x, lo), hi);
}
inline int32_t sse_cvt(float x) {                                 // to_i32x4 :318-320
    if (!(x >= -2147483648.0f && x < 2147483648.0f)) return INT32_MIN;
    return (int32_t)std::nearbyint(x);  // default rounding mode: nearest even
}
// Rust f32::min (IEEE minNum).
inline float rust_fmin(float a, float b) { return std::fmin(a, b); }

const float kNegInf = -INFINITY;

struct RectF { float minx, miny, maxx, maxy; };
struct RectI {
    int32_t minx, miny, maxx, maxy;
    int32_t width() const { return maxx - minx; }
    int32_t height() const { return maxy - miny; }
    // RectI::contains_point, geometry/src/rect.rs:399-407
    bool contains(int32_t x, int32_t y) const {
        return minx <= x && miny <= y && x <= maxx - 1 && y <= maxy - 1;
    }
};

// LineSegment2F lanes (from.x, from.y, to.x, to.y).
struct Line { float fx, fy, tx, ty; };

// Segment with baseline + ctrl (content/src/segment.rs:22-35).
enum Kind { kLine = 1, kQuad = 2, kCubic = 3 };
struct Segment { Line base; Line ctrl; int kind; };

const uint32_t kInvalid = 0xffffffffu;

// ---------------------------------------------------------------------------
// Scene access
// ---------------------------------------------------------------------------
struct Contour { const PFVector2F* pts; const uint8_t* flags; uint32_t n; };

struct PathInput {
    std::vector<Contour> contours;
    int fill_rule;
    bool is_clip;
    int32_t clip_path;   // draw paths only
    PFColorU paint;
    uint32_t path_index; // within clip paths or draw paths
    uint8_t blend = 0;   // draw paths: PF_BLEND_MODE_*
    uint32_t gradient = 0;  // draw paths: gradient index + 1, 0 = solid paint
    bool occludes = false;  // BuiltDrawPath::occludes (renderer/src/builder.rs:80-94)
};

// ---------------------------------------------------------------------------
// Paint effects: gradients (content/src/gradient.rs, renderer/src/paint.rs)
// ---------------------------------------------------------------------------
// Round to the nearest binary16 value, ties to even (the f16::from_f32 of the
// reference's RGBA16F metadata texture, renderer/src/gpu/renderer.rs:702-763).
float o_round_f16(float x) {
    if (std::isnan(x)) return x;
    double ax = std::fabs((double)x);
    if (ax >= 65520.0) return x > 0 ? INFINITY : -INFINITY;
    double q = std::ldexp(1.0, -24);  // subnormal quantum
    if (ax >= std::ldexp(1.0, -14)) q = std::ldexp(1.0, std::ilogb(ax) - 10);
    return (float)(std::nearbyint((double)x / q) * q);
}

// Gradient::add (content/src/gradient.rs:158-164): each stop goes after every
// stop whose offset is <= its own.
std::vector<PFCUDAColorStop> o_ordered_stops(const PFCUDAGradient& g) {
    std::vector<PFCUDAColorStop> out;
    for (uint32_t i = 0; i < g.stop_count; i++) {
        size_t k = 0;
        while (k < out.size() && out[k].offset <= g.stops[i].offset) k++;
        out.insert(out.begin() + (long)k, g.stops[i]);
    }
    return out;
}

// Gradient::sample (content/src/gradient.rs:188-211) in single precision, with
// ColorU::to_f32, ColorF::lerp and ColorF::to_u8 (color/src/lib.rs:70-73,
// 163-171; to_i32x4 rounds to nearest even).
PFColorU o_gradient_sample(const std::vector<PFCUDAColorStop>& stops, float t) {
    if (stops.empty()) return PFColorU{0, 0, 0, 0};
    t = std::fmin(1.0f, std::fmax(0.0f, t));
    size_t lo = 0, hi = stops.size();  // first stop not (offset < t || offset == 0)
    while (lo < hi) {
        size_t mid = (lo + hi) / 2;
        if (stops[mid].offset < t || stops[mid].offset == 0.0f) lo = mid + 1;
        else hi = mid;
    }
    size_t upper = std::min(lo, stops.size() - 1);
    size_t lower = upper > 0 ? upper - 1 : upper;
    const PFCUDAColorStop &a = stops[lower], &b = stops[upper];
    float denom = b.offset - a.offset;
    if (denom == 0.0f) return a.color;
    float ratio = std::fmin((t - a.offset) / denom, 1.0f);
    const float k = 1.0f / 255.0f;
    float ca[4] = {a.color.r * k, a.color.g * k, a.color.b * k, a.color.a * k};
    float cb[4] = {b.color.r * k, b.color.g * k, b.color.b * k, b.color.a * k};
    uint8_t o[4];
    for (int c = 0; c < 4; c++) o[c] = (uint8_t)sse_cvt((ca[c] + (cb[c] - ca[c]) * ratio) * 255.0f);
    return PFColorU{o[0], o[1], o[2], o[3]};
}

// A paint overlay: a gradient (kind PF_GRADIENT_*) or an image pattern (kind 2).
struct OGrad {
    int32_t kind = 0, wrap = 0;
    float g[6] = {0, 0, 0, 0, 0, 0};  // scene -> colour texture coordinate (row-major 2x3)
    float fx = 0, fy = 0, vx = 0, vy = 0, r0 = 0, r1 = 0;  // radial, rounded to binary16
    PFColorU ramp[256];
    bool opaque = true;
    // patterns: the texture page (image inside a transparent border on axes that do not repeat)
    std::vector<PFColorU> page;
    int32_t pw = 0, ph = 0;
    uint32_t flags = 0;
    int32_t filter = 0;
    float blur[6] = {0, 0, 0, 0, 0, 0};  // offset x, y, support, Gaussian x, y, z (binary16)
    float matrix[20] = {};               // colour matrix columns (binary16)
};
const int32_t kOPattern = 2;

// The gradient's colour ramp (renderer/src/paint.rs:855-863) and texture
// transform (:603-616): linear, the projection onto the gradient line; radial,
// Transform2F::inverse of its transform (geometry/src/transform2d.rs:60-72,
// 294-298).  A degenerate linear gradient samples u = 0 here (the reference
// divides by zero); a singular radial transform is rejected.
bool o_build_gradient(const PFCUDAGradient& in, OGrad& g) {
    if (in.kind != PF_GRADIENT_LINEAR && in.kind != PF_GRADIENT_RADIAL) return false;
    if (in.wrap != PF_GRADIENT_WRAP_CLAMP && in.wrap != PF_GRADIENT_WRAP_REPEAT) return false;
    if (in.stop_count && !in.stops) return false;
    g.kind = in.kind;
    g.wrap = in.wrap;
    std::vector<PFCUDAColorStop> stops = o_ordered_stops(in);
    for (int x = 0; x < 256; x++) g.ramp[x] = o_gradient_sample(stops, ((float)x + 0.5f) / 256.0f);
    g.opaque = true;  // Gradient::is_opaque (content/src/gradient.rs:215-217)
    for (const PFCUDAColorStop& st : stops) g.opaque = g.opaque && st.color.a == 255;
    if (in.kind == PF_GRADIENT_LINEAR) {
        float dx = in.to.x - in.from.x, dy = in.to.y - in.from.y;
        float l2 = dx * dx + dy * dy;  // LineSegment2F::square_length
        if (l2 > 0.0f) {
            float m0x = dx / l2, m0y = dy / l2;
            g.g[0] = m0x;
            g.g[1] = m0y;
            g.g[2] = m0x * -in.from.x + m0y * -in.from.y;
        }
    } else {
        const PFTransform2F& t = in.transform;
        float det = t.m00 * t.m11 - t.m01 * t.m10;
        if (det == 0.0f) return false;
        float r = 1.0f / det;
        float a = r * t.m11, b = r * -t.m01, c = r * -t.m10, d = r * t.m00;
        g.g[0] = a; g.g[1] = b; g.g[2] = -(a * t.vector.x + b * t.vector.y);
        g.g[3] = c; g.g[4] = d; g.g[5] = -(c * t.vector.x + d * t.vector.y);
        g.fx = o_round_f16(in.from.x);
        g.fy = o_round_f16(in.from.y);
        g.vx = o_round_f16(in.to.x - in.from.x);
        g.vy = o_round_f16(in.to.y - in.from.y);
        g.r0 = o_round_f16(in.radius0);
        g.r1 = o_round_f16(in.radius1);
    }
    return true;
}

// An image pattern on its own texture page (renderer/src/paint.rs:498-560):
// one transparent texel of border on each axis that does not repeat; page UV
// = scale(1 / page size) * inverse(pattern transform) (:617-623) in single
// precision with the reference's product order (geometry/src/transform2d.rs:
// 60-72, 115-129, 294-310); filter parameters as compute_filter_params writes
// them (renderer/src/gpu/renderer.rs:988-1040), rounded to binary16.
bool o_build_pattern(const PFCUDAPattern& in, OGrad& g) {
    if (!in.pixels || in.width == 0 || in.height == 0 || in.width > 16384 || in.height > 16384) return false;
    if (in.flags & ~7u) return false;
    if (in.filter < 0 || in.filter > PF_PATTERN_FILTER_COLOR_MATRIX) return false;
    const bool blur = in.filter == PF_PATTERN_FILTER_BLUR_X || in.filter == PF_PATTERN_FILTER_BLUR_Y;
    if (blur && !(in.blur_sigma > 0.0f && in.blur_sigma <= 256.0f)) return false;
    const PFTransform2F& t = in.transform;
    float det = t.m00 * t.m11 - t.m01 * t.m10;
    if (det == 0.0f) return false;
    g.kind = kOPattern;
    g.flags = in.flags;
    g.filter = in.filter;
    const int bx = (in.flags & PF_PATTERN_REPEAT_X) ? 0 : 1, by = (in.flags & PF_PATTERN_REPEAT_Y) ? 0 : 1;
    g.pw = (int)in.width + 2 * bx;
    g.ph = (int)in.height + 2 * by;
    g.page.assign((size_t)g.pw * g.ph, PFColorU{0, 0, 0, 0});
    g.opaque = true;  // Image::is_opaque (content/src/pattern.rs:208-212)
    for (uint32_t y = 0; y < in.height; y++)
        for (uint32_t x = 0; x < in.width; x++) {
            PFColorU c = in.pixels[(size_t)y * in.width + x];
            g.page[(size_t)(y + by) * g.pw + (x + bx)] = c;
            g.opaque = g.opaque && c.a == 255;
        }
    float r = 1.0f / det;
    float a = r * t.m11, b = r * -t.m01, c = r * -t.m10, d = r * t.m00;
    float ivx = -(a * t.vector.x + b * t.vector.y), ivy = -(c * t.vector.x + d * t.vector.y);
    float sx = 1.0f / (float)g.pw, sy = 1.0f / (float)g.ph;
    // [sx 0; 0 sy] * [a b; c d] with the zero products kept, as F32x4 lanes compute it
    g.g[0] = sx * a + 0.0f * c;
    g.g[1] = sx * b + 0.0f * d;
    g.g[3] = 0.0f * a + sy * c;
    g.g[4] = 0.0f * b + sy * d;
    g.g[2] = (sx * ivx + 0.0f * ivy) + 0.0f;
    g.g[5] = (0.0f * ivx + sy * ivy) + 0.0f;
    if (blur) {
        float sigma_inv = 1.0f / in.blur_sigma;
        float gx = 0.3989422804014327f * sigma_inv, gy = std::exp(-0.5f * sigma_inv * sigma_inv), gz = gy * gy;
        float support = std::ceil(1.5f * in.blur_sigma) * 2.0f;
        g.blur[0] = in.filter == PF_PATTERN_FILTER_BLUR_X ? 1.0f : 0.0f;
        g.blur[1] = in.filter == PF_PATTERN_FILTER_BLUR_Y ? 1.0f : 0.0f;
        g.blur[2] = o_round_f16(support);
        g.blur[3] = o_round_f16(gx);
        g.blur[4] = o_round_f16(gy);
        g.blur[5] = o_round_f16(gz);
    } else if (in.filter == PF_PATTERN_FILTER_COLOR_MATRIX) {
        for (int k = 0; k < 20; k++) g.matrix[k] = o_round_f16(in.color_matrix[k]);
    }
    return true;
}

// Outline bounds (content/src/outline.rs:180-193 push_contour, :1086-1092
// union_rect): union of every point, control points included.
bool outline_bounds(const std::vector<Contour>& cs, RectF* out) {
    bool any = false;
    RectF r{0, 0, 0, 0};
    for (const Contour& c : cs) {
        if (c.n == 0) continue;
        RectF cb{c.pts[0].x, c.pts[0].y, c.pts[0].x, c.pts[0].y};
        for (uint32_t i = 1; i < c.n; i++) {
            cb.minx = sse_min(cb.minx, c.pts[i].x); cb.miny = sse_min(cb.miny, c.pts[i].y);
            cb.maxx = sse_max(cb.maxx, c.pts[i].x); cb.maxy = sse_max(cb.maxy, c.pts[i].y);
        }
        if (!any) r = cb;
        else {
            r.minx = sse_min(r.minx, cb.minx); r.miny = sse_min(r.miny, cb.miny);
            r.maxx = sse_max(r.maxx, cb.maxx); r.maxy = sse_max(r.maxy, cb.maxy);
        }
        any = true;
    }
    *out = r;
    return any;
}

// RectF::intersects / intersection (geometry/src/rect.rs:116-139).
bool rect_intersection(RectF a, RectF b, RectF* out) {
    bool ok = a.minx < b.maxx && a.miny < b.maxy && b.minx < a.maxx && b.miny < a.maxy;
    if (!ok) return false;
    *out = RectF{sse_max(a.minx, b.minx), sse_max(a.miny, b.miny),
                 sse_min(a.maxx, b.maxx), sse_min(a.maxy, b.maxy)};
    return true;
}

// tiles::round_rect_out_to_tile_bounds (renderer/src/tiles.rs:64-66).
RectI round_rect_out_to_tile_bounds(RectF r) {
    const float s = 1.0f / 16.0f;
    RectF q{r.minx * s, r.miny * s, r.maxx * s, r.maxy * s};
    return RectI{sse_cvt(std::floor(q.minx)), sse_cvt(std::floor(q.miny)),
                 sse_cvt(std::ceil(q.maxx)), sse_cvt(std::ceil(q.maxy))};
}

// ---------------------------------------------------------------------------
// Per-path build state (BuiltPath + ObjectBuilder, renderer/src/builder.rs)
// ---------------------------------------------------------------------------
struct OFill { uint16_t fx, fy, tx, ty; int32_t tile_x, tile_y; uint32_t local_tile; };
struct OTile {
    int16_t tile_x, tile_y;
    uint32_t alpha_tile_id;   // provisional: kInvalid or 0 (has fill); canonical later
    int8_t backdrop;
    uint8_t ctrl;
    uint16_t color;
};
struct OClip { uint32_t dest_tile_id; int32_t dest_backdrop; uint32_t src_tile_id; int32_t src_backdrop; };

struct BuiltPath {
    RectI tile_rect{0, 0, 0, 0};
    std::vector<int32_t> backdrops;
    std::vector<OTile> tiles;
    std::vector<OClip> clips;     // draw paths with a clip path
    std::vector<OFill> fills;     // emission order
    uint64_t line_count = 0;
    bool limit_hit = false;
};

struct Ctx {
    RectF view_box;
    BuiltPath* bp;
    uint64_t dda_limit;
    bool d3d11 = false;  // the D3D11 level's binning: no view-box clip, truncating fills
};

// ObjectBuilder::add_fill (renderer/src/builder.rs:509-553).
void add_fill(Ctx& ctx, Line seg, int32_t tx, int32_t ty) {
    BuiltPath& bp = *ctx.bp;
    if (!bp.tile_rect.contains(tx, ty)) return;
    const float ulx = (float)tx * 16.0f, uly = (float)ty * 16.0f;
    float s0 = (seg.fx - ulx) * 256.0f, s1 = (seg.fy - uly) * 256.0f;
    float s2 = (seg.tx - ulx) * 256.0f, s3 = (seg.ty - uly) * 256.0f;
    const float lo = 0.0f, hi = (float)(16 * 256 - 1);
    int32_t i0 = sse_cvt(sse_clamp(s0, lo, hi)), i1 = sse_cvt(sse_clamp(s1, lo, hi));
    int32_t i2 = sse_cvt(sse_clamp(s2, lo, hi)), i3 = sse_cvt(sse_clamp(s3, lo, hi));
    if (i0 == i2) return;
    uint32_t local = (uint32_t)((tx - bp.tile_rect.minx) + bp.tile_rect.width() * (ty - bp.tile_rect.miny));
    bp.tiles[local].alpha_tile_id = 0;  // get_or_allocate_alpha_tile_index :555-576
    bp.fills.push_back(OFill{(uint16_t)i0, (uint16_t)i1, (uint16_t)i2, (uint16_t)i3, tx, ty, local});
}

// addFill of the D3D11 level (shaders/d3d11/bin.cs.glsl:100-125): tile-rect
// cull, 8.8 conversion by truncation without a clamp to 4095 (a negative
// value, undefined in GLSL, converts to 0), cull when from.x == to.x.
void add_fill_d3d11(Ctx& ctx, Line seg, int32_t tx, int32_t ty) {
    BuiltPath& bp = *ctx.bp;
    if (!bp.tile_rect.contains(tx, ty)) return;
    const float ulx = (float)tx * 16.0f, uly = (float)ty * 16.0f;
    auto q = [](float v) { return (uint32_t)std::min(std::max(v, 0.0f), 65535.0f); };
    uint32_t i0 = q((seg.fx - ulx) * 256.0f), i1 = q((seg.fy - uly) * 256.0f);
    uint32_t i2 = q((seg.tx - ulx) * 256.0f), i3 = q((seg.ty - uly) * 256.0f);
    if (i0 == i2) return;
    uint32_t local = (uint32_t)((tx - bp.tile_rect.minx) + bp.tile_rect.width() * (ty - bp.tile_rect.miny));
    bp.tiles[local].alpha_tile_id = 0;
    bp.fills.push_back(OFill{(uint16_t)i0, (uint16_t)i1, (uint16_t)i2, (uint16_t)i3, tx, ty, local});
}

// ObjectBuilder::adjust_alpha_tile_backdrop (renderer/src/builder.rs:595-616).
void adjust_backdrop(Ctx& ctx, int32_t tx, int32_t ty, int8_t delta) {
    BuiltPath& bp = *ctx.bp;
    int32_t ox = tx - bp.tile_rect.minx, oy = ty - bp.tile_rect.miny;
    if (ox < 0 || ox >= bp.tile_rect.width() || oy >= bp.tile_rect.height()) return;
    if (oy < 0) { bp.backdrops[ox] += delta; return; }
    uint32_t idx = (uint32_t)(oy * bp.tile_rect.width() + ox);
    bp.tiles[idx].backdrop = (int8_t)(uint8_t)((uint8_t)bp.tiles[idx].backdrop + (uint8_t)delta);
}

// clip::clip_line_segment_to_rect (content/src/clip.rs:494-560), Cohen-Sutherland.
inline uint32_t outcode(float x, float y, RectF r) {
    uint32_t o = 0;
    if (x < r.minx) o |= 1;  // LEFT
    if (y < r.miny) o |= 4;  // TOP
    if (x > r.maxx) o |= 2;  // RIGHT
    if (y > r.maxy) o |= 8;  // BOTTOM
    return o;
}
inline float lerpf(float a, float b, float t) { return a + (b - a) * t; }  // geometry/src/util.rs:25-27

bool clip_line_segment_to_rect(Line& s, RectF r) {
    uint32_t of = outcode(s.fx, s.fy, r), ot = outcode(s.tx, s.ty, r);
    for (int iter = 0; iter < 64; iter++) {
        if (of == 0 && ot == 0) return true;
        if ((of & ot) != 0) return false;
        bool clip_from = of > ot;
        uint32_t oc = clip_from ? of : ot;
        float px, py;
        if (clip_from) { px = s.fx; py = s.fy; } else { px = s.tx; py = s.ty; }
        if (oc & 1) {
            px = r.minx; py = lerpf(s.fy, s.ty, (r.minx - s.fx) / (s.tx - s.fx));
        } else if (oc & 2) {
            px = r.maxx; py = lerpf(s.fy, s.ty, (r.maxx - s.fx) / (s.tx - s.fx));
        } else if (oc & 4) {
            px = lerpf(s.fx, s.tx, (r.miny - s.fy) / (s.ty - s.fy)); py = r.miny;
        } else if (oc & 8) {
            px = lerpf(s.fx, s.tx, (r.maxy - s.fy) / (s.ty - s.fy)); py = r.maxy;
        }
        if (clip_from) { s.fx = px; s.fy = py; of = outcode(px, py, r); }
        else { s.tx = px; s.ty = py; ot = outcode(px, py, r); }
    }
    return false;  // unreachable for finite input
}

// process_line_segment (renderer/src/tiler.rs:191-308).
void process_line_segment(Ctx& ctx, Line seg) {
    ctx.bp->line_count++;
    RectF clip_box{ctx.view_box.minx, kNegInf, ctx.view_box.maxx, ctx.view_box.maxy};
    if (!ctx.d3d11 && !clip_line_segment_to_rect(seg, clip_box)) return;
    auto fill = [&](Line l, int32_t tx, int32_t ty) {
        if (ctx.d3d11) add_fill_d3d11(ctx, l, tx, ty);
        else add_fill(ctx, l, tx, ty);
    };

    const float r = 1.0f / 16.0f;
    int32_t ftx = sse_cvt(std::floor(seg.fx * r)), fty = sse_cvt(std::floor(seg.fy * r));
    int32_t ttx = sse_cvt(std::floor(seg.tx * r)), tty = sse_cvt(std::floor(seg.ty * r));
    float vx = seg.tx - seg.fx, vy = seg.ty - seg.fy;
    bool negx = vx < 0.0f, negy = vy < 0.0f;
    int32_t stepx = negx ? -1 : 1, stepy = negy ? -1 : 1;
    float fcx = (float)(ftx + (negx ? 0 : 1)) * 16.0f;
    float fcy = (float)(fty + (negy ? 0 : 1)) * 16.0f;
    float tmx = (fcx - seg.fx) / vx, tmy = (fcy - seg.fy) / vy;
    float tdx = std::fabs(16.0f / vx), tdy = std::fabs(16.0f / vy);

    float cx = seg.fx, cy = seg.fy;
    int32_t tcx = ftx, tcy = fty;
    enum { kNone = 0, kX = 1, kY = 2 };
    int last = kNone;
    for (uint64_t it = 0;; it++) {
        if (it >= ctx.dda_limit) { ctx.bp->limit_hit = true; return; }
        int dir;
        if (tmx < tmy) dir = kX;
        else if (tmx > tmy) dir = kY;
        else dir = stepx > 0 ? kX : kY;
        float next_t = rust_fmin(dir == kX ? tmx : tmy, 1.0f);
        if (tcx == ttx && tcy == tty) dir = kNone;

        float npx = seg.fx + vx * next_t, npy = seg.fy + vy * next_t;
        fill(Line{cx, cy, npx, npy}, tcx, tcy);

        if (stepy < 0 && dir == kY) {
            fill(Line{npx, npy, (float)tcx * 16.0f, (float)tcy * 16.0f}, tcx, tcy);
        } else if (stepy > 0 && last == kY) {
            fill(Line{(float)tcx * 16.0f, (float)tcy * 16.0f, cx, cy}, tcx, tcy);
        }

        if (stepx < 0 && last == kX) adjust_backdrop(ctx, tcx, tcy, 1);
        else if (stepx > 0 && dir == kX) adjust_backdrop(ctx, tcx, tcy, -1);

        if (dir == kNone) break;
        if (dir == kX) {
            if (tcx == ttx) break;
            tmx = tmx + tdx; tmy = tmy + 0.0f;
            tcx += stepx;
        } else {
            if (tcy == tty) break;
            tmx = tmx + 0.0f; tmy = tmy + tdy;
            tcy += stepy;
        }
        cx = npx; cy = npy;
        last = dir;
    }
}

// Segment::to_cubic (content/src/segment.rs:171-182).
Segment to_cubic(const Segment& s) {
    if (s.kind == kCubic) return s;
    Segment c = s;
    float p12x = s.ctrl.fx + s.ctrl.fx, p12y = s.ctrl.fy + s.ctrl.fy;
    const float third = 1.0f / 3.0f;
    c.ctrl = Line{(s.base.fx + p12x) * third, (s.base.fy + p12y) * third,
                  (p12x + s.base.tx) * third, (p12y + s.base.ty) * third};
    c.kind = kCubic;
    return c;
}

// CubicSegment::is_flat (content/src/segment.rs:292-300), tolerance 0.25.
bool is_flat(const Segment& s) {
    float u0 = 3.0f * s.ctrl.fx, u1 = 3.0f * s.ctrl.fy, u2 = 3.0f * s.ctrl.tx, u3 = 3.0f * s.ctrl.ty;
    u0 = u0 - s.base.fx; u1 = u1 - s.base.fy; u2 = u2 - s.base.tx; u3 = u3 - s.base.ty;
    u0 = u0 - s.base.fx; u1 = u1 - s.base.fy; u2 = u2 - s.base.tx; u3 = u3 - s.base.ty;
    u0 = u0 - s.base.tx; u1 = u1 - s.base.ty; u2 = u2 - s.base.fx; u3 = u3 - s.base.fy;
    u0 = u0 * u0; u1 = u1 * u1; u2 = u2 * u2; u3 = u3 * u3;
    float m0 = sse_max(u0, u2), m1 = sse_max(u1, u3);
    const float tol = 0.25f;
    return m0 + m1 <= 16.0f * tol * tol;
}

// CubicSegment::split at t = 0.5 (content/src/segment.rs:307-359).
void split_half(const Segment& s, Segment* a, Segment* b) {
    const float t = 0.5f;
    float p0x = s.base.fx, p0y = s.base.fy, p3x = s.base.tx, p3y = s.base.ty;
    float p1x = s.ctrl.fx, p1y = s.ctrl.fy, p2x = s.ctrl.tx, p2y = s.ctrl.ty;
    float p01x = p0x + t * (p1x - p0x), p01y = p0y + t * (p1y - p0y);
    float p12x = p1x + t * (p2x - p1x), p12y = p1y + t * (p2y - p1y);
    float p23x = p2x + t * (p3x - p2x), p23y = p2y + t * (p3y - p2y);
    float p012x = p01x + t * (p12x - p01x), p012y = p01y + t * (p12y - p01y);
    float p123x = p12x + t * (p23x - p12x), p123y = p12y + t * (p23y - p12y);
    float p0123x = p012x + t * (p123x - p012x), p0123y = p012y + t * (p123y - p012y);
    a->base = Line{p0x, p0y, p0123x, p0123y}; a->ctrl = Line{p01x, p01y, p012x, p012y}; a->kind = kCubic;
    b->base = Line{p0123x, p0123y, p3x, p3y}; b->ctrl = Line{p123x, p123y, p23x, p23y}; b->kind = kCubic;
}

// process_segment (renderer/src/tiler.rs:166-184), recursive as in the reference,
// with the CUDA tiler's bound of 2^20 lines per input segment (depth first; the
// walk stops there and flags the limit).  Returns false once stopped.
const uint32_t kMaxSegmentLines = 1u << 20;
bool process_segment(Ctx& ctx, const Segment& s, int depth, uint32_t* emitted) {
    if (s.kind == kQuad) return process_segment(ctx, to_cubic(s), depth, emitted);
    if (s.kind == kLine || is_flat(s) || depth >= 32) {
        if (depth >= 32 && s.kind == kCubic && !is_flat(s)) ctx.bp->limit_hit = true;
        process_line_segment(ctx, s.base);
        if (++*emitted >= kMaxSegmentLines) { ctx.bp->limit_hit = true; return false; }
        return true;
    }
    Segment a, b;
    split_half(s, &a, &b);
    if (!process_segment(ctx, a, depth + 1, emitted)) return false;
    return process_segment(ctx, b, depth + 1, emitted);
}

// A segment with a non-finite coordinate gives no fills (as on the GPU).
bool segment_finite(const Segment& s) {
    auto f = [](float v) { return std::isfinite(v); };
    if (!f(s.base.fx) || !f(s.base.fy) || !f(s.base.tx) || !f(s.base.ty)) return false;
    if (s.kind == kQuad) return f(s.ctrl.fx) && f(s.ctrl.fy);
    if (s.kind == kCubic) return f(s.ctrl.fx) && f(s.ctrl.fy) && f(s.ctrl.tx) && f(s.ctrl.ty);
    return true;
}

// Uniform dicing of the D3D11 level (shaders/d3d11/dice.cs.glsl:133-217): a
// curve into n pieces of equal parameter length, n from Sederberg's error
// bound for tolerance 0.25; a line into pieces of at most 16 px; piece ends
// rounded to 1/256 px (the packed microline, :83-97).  The FP32 op order is the
// CUDA level's definition of this mode (dice_seg / dice_count / dice_point).
void dice_segment(Ctx& ctx, const Segment& s) {
    const bool curve = s.kind != kLine;
    float p0x = s.base.fx, p0y = s.base.fy, p3x = s.base.tx, p3y = s.base.ty;
    float c0x = p0x, c0y = p0y, c1x = p3x, c1y = p3y;
    if (s.kind == kQuad) {
        const float third = 1.0f / 3.0f;
        const float qx2 = s.ctrl.fx + s.ctrl.fx, qy2 = s.ctrl.fy + s.ctrl.fy;
        c0x = (p0x + qx2) * third; c0y = (p0y + qy2) * third;
        c1x = (p3x + qx2) * third; c1y = (p3y + qy2) * third;
    } else if (s.kind == kCubic) {
        c0x = s.ctrl.fx; c0y = s.ctrl.fy; c1x = s.ctrl.tx; c1y = s.ctrl.ty;
    }
    float n;
    if (curve) {
        auto dd = [](float a, float b, float c) { return std::fabs((c - 2.0f * b) + a); };
        const float bx = 6.0f * std::max(dd(p0x, c0x, c1x), dd(c0x, c1x, p3x));
        const float by = 6.0f * std::max(dd(p0y, c0y, c1y), dd(c0y, c1y, p3y));
        const float len = std::sqrt(bx * bx + by * by);
        n = std::sqrt(len / (8.0f * 0.25f));
    } else {
        const float dx = p3x - p0x, dy = p3y - p0y;
        n = std::sqrt(dx * dx + dy * dy) / 16.0f;
    }
    const uint32_t kMax = 1u << 16;
    uint32_t pieces;
    if (!(n <= (float)kMax)) {
        ctx.bp->limit_hit = true;
        pieces = n > (float)kMax ? kMax : 1u;
    } else {
        pieces = std::max<uint32_t>((uint32_t)std::ceil(n), 1u);
    }
    auto lerp = [](float a, float b, float t) { return a + (b - a) * t; };
    auto q = [](float v) {
        return std::nearbyint(std::min(std::max(v, -32768.0f), 32767.0f) * 256.0f) * (1.0f / 256.0f);
    };
    float ax = q(p0x), ay = q(p0y);
    for (uint32_t k = 1; k <= pieces; k++) {
        const float t = (float)k / (float)pieces;
        float x, y;
        if (curve) {
            const float ux = lerp(p0x, c0x, t), uy = lerp(p0y, c0y, t);
            const float vx = lerp(c0x, c1x, t), vy = lerp(c0y, c1y, t);
            const float wx = lerp(c1x, p3x, t), wy = lerp(c1y, p3y, t);
            const float uvx = lerp(ux, vx, t), uvy = lerp(uy, vy, t);
            const float vwx = lerp(vx, wx, t), vwy = lerp(vy, wy, t);
            x = lerp(uvx, vwx, t);
            y = lerp(uvy, vwy, t);
        } else {
            x = lerp(p0x, p3x, t);
            y = lerp(p0y, p3y, t);
        }
        const float bx = q(x), by = q(y);
        process_line_segment(ctx, Line{ax, ay, bx, by});
        ax = bx; ay = by;
    }
}

// ContourIter::next (content/src/outline.rs:1024-1065) on a closed contour.
template <typename F>
void for_each_segment(const Contour& c, F&& f) {
    auto is_end = [&](uint32_t i) {
        return (c.flags[i] & (PF_POINT_FLAG_CONTROL_POINT_0 | PF_POINT_FLAG_CONTROL_POINT_1)) == 0;
    };
    uint32_t index = 1;
    const uint32_t len = c.n;
    if (len == 0) return;
    for (;;) {
        if (index == len + 1) return;
        uint32_t i0 = index - 1;
        PFVector2F p0 = c.pts[i0];
        if (index == len) {
            PFVector2F p1 = c.pts[0];
            index++;
            f(Segment{Line{p0.x, p0.y, p1.x, p1.y}, Line{0, 0, 0, 0}, kLine});
            continue;
        }
        uint32_t i1 = index++;
        PFVector2F p1 = c.pts[i1];
        if (is_end(i1)) { f(Segment{Line{p0.x, p0.y, p1.x, p1.y}, Line{0, 0, 0, 0}, kLine}); continue; }
        uint32_t i2 = index++;
        PFVector2F p2 = c.pts[i2];
        if (is_end(i2)) { f(Segment{Line{p0.x, p0.y, p2.x, p2.y}, Line{p1.x, p1.y, 0, 0}, kQuad}); continue; }
        uint32_t i3 = index++;
        PFVector2F p3 = c.pts[i3];
        f(Segment{Line{p0.x, p0.y, p3.x, p3.y}, Line{p1.x, p1.y, p2.x, p2.y}, kCubic});
    }
}

struct Frame {
    RectF view_box;
    uint32_t clip_count = 0, draw_count = 0;
    std::vector<PathInput> paths;             // clip paths then draw paths
    std::vector<std::vector<PFVector2F>> transformed;  // per path, when a transform applies
    std::vector<BuiltPath> built;
    std::vector<uint64_t> tile_offset;        // per path, global tile index of its first tile
    std::vector<uint64_t> fill_offset;        // per path, global emission index of its first fill
    std::vector<uint32_t> alpha_owner;        // alpha id -> global tile index owning the fills
    RectI screen{0, 0, 0, 0};
    std::vector<int32_t> zbuf;
    std::vector<OGrad> grads;                 // the scene's overlays: gradients, then patterns
    float inv[6] = {1, 0, 0, 0, 1, 0};        // frame pixel -> scene (inverse build transform)
    bool limit_hit = false;
    bool d3d11 = false;  // the D3D11 level's dicing and binning
};

// Tiler::new + generate_tiles (renderer/src/tiler.rs:40-91) up to generate_fills.
void build_fills(Frame& fr, uint32_t p, uint64_t dda_limit) {
    const PathInput& in = fr.paths[p];
    BuiltPath& bp = fr.built[p];
    RectF ob;
    RectF bounds{0, 0, 0, 0};
    if (outline_bounds(in.contours, &ob)) {
        RectF isect;
        if (rect_intersection(ob, fr.view_box, &isect)) bounds = isect;
    }
    // A destructive blend mode tiles the whole view box (renderer/src/builder.rs:430-434,
    // BlendMode::is_destructive, content/src/effects.rs:233-262).
    const uint8_t m = in.blend;
    if (!in.is_clip && (m == PF_BLEND_MODE_CLEAR || m == PF_BLEND_MODE_COPY || m == PF_BLEND_MODE_SRC_IN ||
                        m == PF_BLEND_MODE_SRC_OUT || m == PF_BLEND_MODE_DEST_IN || m == PF_BLEND_MODE_DEST_ATOP))
        bounds = fr.view_box;
    bp.tile_rect = round_rect_out_to_tile_bounds(bounds);
    int32_t w = bp.tile_rect.width(), h = bp.tile_rect.height();
    if (w < 0) w = 0;
    if (h < 0) h = 0;
    bp.backdrops.assign((size_t)w, 0);
    bp.tiles.resize((size_t)w * (size_t)h);
    uint8_t ctrl = in.is_clip ? 0 : (in.fill_rule == PF_FILL_RULE_EVEN_ODD ? 0x2 : 0x1);
    uint16_t color = in.is_clip ? 0 : (uint16_t)(in.path_index & 0xffff);
    for (int32_t y = 0; y < h; y++)
        for (int32_t x = 0; x < w; x++) {
            OTile& t = bp.tiles[(size_t)y * w + x];
            t.tile_x = (int16_t)(bp.tile_rect.minx + x);
            t.tile_y = (int16_t)(bp.tile_rect.miny + y);
            t.alpha_tile_id = kInvalid;
            t.backdrop = 0;
            t.ctrl = ctrl;
            t.color = color;
        }
    if (!in.is_clip && in.clip_path >= 0)
        bp.clips.assign(bp.tiles.size(), OClip{kInvalid, 0, kInvalid, 0});
    Ctx ctx{fr.view_box, &bp, dda_limit, fr.d3d11};
    for (const Contour& c : in.contours)
        for_each_segment(c, [&](const Segment& s) {
            if (!segment_finite(s)) { bp.limit_hit = true; return; }
            uint32_t emitted = 0;
            if (fr.d3d11) dice_segment(ctx, s);
            else process_segment(ctx, s, 0, &emitted);
        });
}

// The tile of path q at (tx, ty), or NULL outside its tile rect.
const OTile* tile_at(const Frame& fr, int32_t q, int32_t tx, int32_t ty) {
    const BuiltPath& cb = fr.built[(uint32_t)q];
    if (!cb.tile_rect.contains(tx, ty)) return nullptr;
    return &cb.tiles[(size_t)(ty - cb.tile_rect.miny) * cb.tile_rect.width() + (size_t)(tx - cb.tile_rect.minx)];
}

// Tiler::prepare_tiles (renderer/src/tiler.rs:93-163).  Draw paths whose
// clip path is itself clipped (the D3D11 level's clip levels,
// renderer/src/builder.rs:1124-1220; the CPU tiler has no such case) keep
// their tiles, flagged as behind a clip chain, unless a level of the chain has
// no tile or an empty one there.
void prepare_tiles(Frame& fr, uint32_t p) {
    const PathInput& in = fr.paths[p];
    BuiltPath& bp = fr.built[p];
    const BuiltPath* clip = nullptr;
    bool chain = false;
    if (!in.is_clip && in.clip_path >= 0) {
        clip = &fr.built[(uint32_t)in.clip_path];
        chain = fr.paths[(uint32_t)in.clip_path].clip_path >= 0;
    }
    int32_t w = bp.tile_rect.width();
    for (size_t i = 0; i < bp.tiles.size(); i++) {
        OTile& t = bp.tiles[i];
        size_t column = i % (size_t)w;
        int32_t delta = t.backdrop;
        uint32_t draw_alpha = t.alpha_tile_id;
        int8_t draw_backdrop = (int8_t)(uint8_t)(uint32_t)bp.backdrops[column];
        if (chain) {
            t.ctrl |= 0x4;
            bool culled = false;
            int32_t q = in.clip_path;
            for (uint32_t it = 0; q >= 0 && it <= fr.clip_count; it++) {
                const OTile* ct = tile_at(fr, q, t.tile_x, t.tile_y);
                if (!ct || (ct->alpha_tile_id == kInvalid && ct->backdrop == 0)) { culled = true; break; }
                q = fr.paths[(uint32_t)q].clip_path;
            }
            if (culled) { draw_alpha = kInvalid; draw_backdrop = 0; }
        } else if (clip) {
            int32_t cx = t.tile_x, cy = t.tile_y;
            if (clip->tile_rect.contains(cx, cy)) {
                const OTile& ct = clip->tiles[(size_t)(cy - clip->tile_rect.miny) * clip->tile_rect.width() +
                                              (size_t)(cx - clip->tile_rect.minx)];
                if (ct.alpha_tile_id != kInvalid && draw_alpha != kInvalid) {
                    OClip& oc = bp.clips[i];
                    oc.dest_tile_id = t.alpha_tile_id;
                    oc.dest_backdrop = draw_backdrop;
                    oc.src_tile_id = ct.alpha_tile_id;
                    oc.src_backdrop = ct.backdrop;
                    draw_backdrop = 0;
                } else if (ct.alpha_tile_id != kInvalid && draw_alpha == kInvalid && draw_backdrop != 0) {
                    draw_alpha = ct.alpha_tile_id;
                    draw_backdrop = ct.backdrop;
                } else if (ct.alpha_tile_id == kInvalid && ct.backdrop == 0) {
                    draw_alpha = kInvalid;
                    draw_backdrop = 0;
                }
            } else {
                draw_alpha = kInvalid;
                draw_backdrop = 0;
            }
        }
        t.alpha_tile_id = draw_alpha;
        t.backdrop = draw_backdrop;
        bp.backdrops[column] += delta;
    }
}

template <typename F>
void parallel_for(uint32_t n, int threads, F&& f) {
    if (threads <= 1 || n < 2) { for (uint32_t i = 0; i < n; i++) f(i); return; }
    std::atomic<uint32_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++)
        pool.emplace_back([&]() {
            for (;;) {
                uint32_t i = next.fetch_add(1);
                if (i >= n) break;
                f(i);
            }
        });
    for (auto& th : pool) th.join();
}

// Resolve of sampleMask (shaders/tile_fragment.inc.glsl:539-556).
template <typename T>
T resolve(T c, bool even_odd) {
    if (!even_odd) c = std::fabs(c);
    else {
        T m = c - (T)2 * std::floor(c / (T)2);  // GLSL mod(c, 2)
        c = (T)1 - std::fabs((T)1 - m);
    }
    return std::min((T)1, c);
}

// A solid tile occludes what lies beneath it only if it resolves to full
// coverage: for the nonzero rule that is any nonzero backdrop (the reference's
// test, renderer/src/builder.rs:1013-1029); for even-odd an odd backdrop.
bool solid_tile_occludes(int8_t backdrop, bool even_odd) {
    if (backdrop == 0) return false;
    if (even_odd) return (backdrop & 1) != 0;
    return true;
}

void build_frame(Frame& fr, int threads, uint64_t dda_limit) {
    uint32_t n = (uint32_t)fr.paths.size();
    fr.built.assign(n, BuiltPath());
    // Clip paths are built before draw paths (renderer/src/builder.rs:224-259).
    parallel_for(fr.clip_count, threads, [&](uint32_t i) { build_fills(fr, i, dda_limit); });
    parallel_for(fr.draw_count, threads,
                 [&](uint32_t i) { build_fills(fr, fr.clip_count + i, dda_limit); });
    // Canonical alpha tile IDs and global offsets.
    fr.tile_offset.assign(n + 1, 0);
    fr.fill_offset.assign(n + 1, 0);
    fr.alpha_owner.clear();
    uint32_t next_alpha = 0;
    for (uint32_t p = 0; p < n; p++) {
        BuiltPath& bp = fr.built[p];
        fr.tile_offset[p + 1] = fr.tile_offset[p] + bp.tiles.size();
        fr.fill_offset[p + 1] = fr.fill_offset[p] + bp.fills.size();
        for (size_t i = 0; i < bp.tiles.size(); i++)
            if (bp.tiles[i].alpha_tile_id != kInvalid) {
                bp.tiles[i].alpha_tile_id = next_alpha++;
                fr.alpha_owner.push_back((uint32_t)(fr.tile_offset[p] + i));
            }
        if (bp.limit_hit) fr.limit_hit = true;
    }
    parallel_for(fr.clip_count, threads, [&](uint32_t i) { prepare_tiles(fr, i); });
    parallel_for(fr.draw_count, threads, [&](uint32_t i) { prepare_tiles(fr, fr.clip_count + i); });
    // Z-buffer over the view box's tiles (renderer/src/builder.rs:1013-1029):
    // per screen tile, the largest draw-path index of an opaque path whose tile
    // there is solid (BuiltDrawPath::new, :80-94: opaque paint and a blend mode
    // that occludes the backdrop).
    fr.screen = round_rect_out_to_tile_bounds(fr.view_box);
    int32_t sw = std::max(0, fr.screen.width()), sh = std::max(0, fr.screen.height());
    fr.zbuf.assign((size_t)sw * (size_t)sh, 0);
    for (uint32_t d = 0; d < fr.draw_count; d++) {
        const PathInput& in = fr.paths[fr.clip_count + d];
        if (!in.occludes) continue;
        const BuiltPath& bp = fr.built[fr.clip_count + d];
        bool eo = in.fill_rule == PF_FILL_RULE_EVEN_ODD;
        for (const OTile& t : bp.tiles) {
            if (t.alpha_tile_id != kInvalid) continue;
            if (t.ctrl & 0x4) continue;  // behind a clip chain: may be partly covered
            if (!solid_tile_occludes(t.backdrop, eo)) continue;
            if (!fr.screen.contains(t.tile_x, t.tile_y)) continue;
            int32_t& z = fr.zbuf[(size_t)(t.tile_y - fr.screen.miny) * sw + (t.tile_x - fr.screen.minx)];
            z = std::max(z, (int32_t)d);
        }
    }
}

// ---------------------------------------------------------------------------
// Coverage: utils/area-lut/src/main.rs:29-65 (exact area) composed as
// computeCoverage (shaders/fill_area.inc.glsl:11-27) over the D3D9 fill quad
// (shaders/d3d9/fill.vs.glsl:37-73).
// ---------------------------------------------------------------------------
template <typename T>
T area_exact(T y, T dydx) {
    const T xl = (T)-0.5, xr = (T)0.5;
    const T p0x = xl, p0y = dydx * xl + y;
    const T p1x = xr, p1y = dydx * xr + y;
    auto solve_x = [&](T yy) {  // solve_line_y(p0, p1, yy).x
        T m = (p1y - p0y) / (p1x - p0x);
        return p0x - (p0y - yy) / m;
    };
    auto tri = [](T ax, T ay, T bx, T by) { return (T)0.5 * (bx - ax) * (ay - by); };
    auto rect = [](T ax, T ay, T bx, T by) { return (bx - ax) * (ay - by); };
    const T p3x = p1x, p3y = (T)-0.5;
    const T p7x = p1x, p7y = (T)0.5;
    if (p0y > (T)0.5) {
        if (p1y < (T)-0.5) {
            T p2x = solve_x((T)-0.5), p4x = solve_x((T)0.5);
            return tri(p0x, p0y, p1x, p1y) - tri(p2x, (T)-0.5, p1x, p1y) - rect(p0x, p0y, p7x, p7y) +
                   tri(p0x, p0y, p4x, (T)0.5);
        } else if (p1y < (T)0.5) {
            T p4x = solve_x((T)0.5);
            return tri(p0x, p0y, p1x, p1y) - rect(p0x, p0y, p7x, p7y) + tri(p0x, p0y, p4x, (T)0.5);
        }
        return (T)0;
    } else if (p0y > (T)-0.5) {
        if (p1y < (T)-0.5) {
            T p2x = solve_x((T)-0.5);
            return tri(p0x, p0y, p1x, p1y) - tri(p2x, (T)-0.5, p1x, p1y) - rect(p0x, p0y, p7x, p7y);
        }
        return tri(p0x, p0y, p1x, p1y) - rect(p0x, p0y, p7x, p7y);
    }
    return -rect(p0x, p0y, p7x, p7y) + rect(p0x, p0y, p3x, p3y);
}

// computeCoverage for one pixel; from/to relative to the pixel centre.
template <typename T>
T pixel_coverage(T fx, T fy, T tx, T ty) {
    bool lt = fx < tx;
    T lx = lt ? fx : tx, ly = lt ? fy : ty, rx = lt ? tx : fx, ry = lt ? ty : fy;
    T wx = std::min(std::max(fx, (T)-0.5), (T)0.5), wy = std::min(std::max(tx, (T)-0.5), (T)0.5);
    T dX = wx - wy;
    if (dX == (T)0) return (T)0;
    T offset = (wx + (wy - wx) * (T)0.5) - lx;
    T t = offset / (rx - lx);
    T y = ly + (ry - ly) * t;
    T d = (ry - ly) / (rx - lx);
    return area_exact<T>(y, -std::fabs(d * dX)) * dX;
}

template <typename T>
void accumulate_fill(const OFill& f, T* mask /*256*/) {
    T fx = (T)f.fx / (T)256, fy = (T)f.fy / (T)256, tx = (T)f.tx / (T)256, ty = (T)f.ty / (T)256;
    int x0 = (int)std::floor(std::min(fx, tx)), x1 = (int)std::ceil(std::max(fx, tx));
    int y0 = (int)std::floor(std::floor(std::min(fy, ty)) * (T)0.25) * 4;
    x0 = std::max(x0, 0); x1 = std::min(x1, 16);
    for (int py = std::max(y0, 0); py < 16; py++)
        for (int px = x0; px < x1; px++) {
            T cx = (T)px + (T)0.5, cy = (T)py + (T)0.5;
            mask[py * 16 + px] += pixel_coverage<T>(fx - cx, fy - cy, tx - cx, ty - cy);
        }
}

// Per alpha tile: sum of its fills (the mask texture contents before backdrop).
template <typename T>
void compute_raw_masks(const Frame& fr, std::vector<T>& masks, int threads) {
    size_t A = fr.alpha_owner.size();
    masks.assign(A * 256, (T)0);
    // Fills are attributed through the owning tile's canonical id, recorded
    // before prepare_tiles may repoint a draw tile at a clip mask.
    std::vector<uint32_t> own_id;  // per global tile, its own alpha id or invalid
    size_t T_total = fr.tile_offset.back();
    own_id.assign(T_total, kInvalid);
    for (size_t a = 0; a < A; a++) own_id[fr.alpha_owner[a]] = (uint32_t)a;
    parallel_for((uint32_t)fr.paths.size(), threads, [&](uint32_t p) {
        const BuiltPath& bp = fr.built[p];
        for (const OFill& f : bp.fills) {
            uint32_t aid = own_id[fr.tile_offset[p] + f.local_tile];
            accumulate_fill<T>(f, &masks[(size_t)aid * 256]);
        }
    });
}

// |mask + backdrop| of one tile (the backdrop alone for a solid tile).
template <typename T>
void tile_abs_winding(const OTile& t, const std::vector<T>& masks, T* out) {
    for (int k = 0; k < 256; k++)
        out[k] = std::fabs((t.alpha_tile_id != kInvalid ? masks[(size_t)t.alpha_tile_id * 256 + k] : (T)0) +
                           (T)t.backdrop);
}

template <typename T>
void tile_coverage(const Frame& fr, uint32_t p, size_t i, const std::vector<T>& masks, T* out) {
    const PathInput& in = fr.paths[p];
    const BuiltPath& bp = fr.built[p];
    const OTile& t = bp.tiles[i];
    bool eo = !in.is_clip && in.fill_rule == PF_FILL_RULE_EVEN_ODD;
    if (t.ctrl & 0x4) {
        // behind a clip chain: the minimum over the tile and every level
        T m[256], mq[256];
        tile_abs_winding<T>(t, masks, m);
        int32_t q = in.clip_path;
        for (uint32_t it = 0; q >= 0 && it <= fr.clip_count; it++) {
            const OTile* ct = tile_at(fr, q, t.tile_x, t.tile_y);
            if (!ct) break;  // culled by prepare_tiles
            tile_abs_winding<T>(*ct, masks, mq);
            for (int k = 0; k < 256; k++) m[k] = std::min(m[k], mq[k]);
            q = fr.paths[(uint32_t)q].clip_path;
        }
        for (int k = 0; k < 256; k++) out[k] = resolve<T>(m[k], eo);
        return;
    }
    if (!bp.clips.empty() && bp.clips[i].dest_tile_id != kInvalid && bp.clips[i].src_tile_id != kInvalid) {
        // tile_clip_combine.fs.glsl:27-30, then sampleMask with backdrop 0.
        const OClip& c = bp.clips[i];
        const T* dm = &masks[(size_t)c.dest_tile_id * 256];
        const T* sm = &masks[(size_t)c.src_tile_id * 256];
        for (int k = 0; k < 256; k++) {
            T m = std::min(std::fabs(dm[k] + (T)c.dest_backdrop), std::fabs(sm[k] + (T)c.src_backdrop));
            out[k] = resolve<T>(m + (T)t.backdrop, eo);
        }
        return;
    }
    if (t.alpha_tile_id != kInvalid) {
        const T* m = &masks[(size_t)t.alpha_tile_id * 256];
        for (int k = 0; k < 256; k++) out[k] = resolve<T>(m[k] + (T)t.backdrop, eo);
        return;
    }
    T c = resolve<T>((T)t.backdrop, eo);
    for (int k = 0; k < 256; k++) out[k] = c;
}

// Paint effects of the composite.  The colour texture transform of a
// gradient for this frame is its own map composed with the inverse build
// transform (renderer/src/paint.rs:637; Transform2F * Transform2F,
// geometry/src/transform2d.rs:115-121, 301-310) in single precision, then
// rounded to binary16 as the metadata texture stores it.
void o_frame_transform(const Frame& fr, const OGrad& g, float t[6]) {
    const float* G = g.g;
    const float* R = fr.inv;
    t[0] = o_round_f16(G[0] * R[0] + G[1] * R[3]);
    t[1] = o_round_f16(G[0] * R[1] + G[1] * R[4]);
    t[2] = o_round_f16((G[0] * R[2] + G[1] * R[5]) + G[2]);
    t[3] = o_round_f16(G[3] * R[0] + G[4] * R[3]);
    t[4] = o_round_f16(G[3] * R[1] + G[4] * R[4]);
    t[5] = o_round_f16((G[3] * R[2] + G[4] * R[5]) + G[5]);
}

// Linear filtering of the ramp at u (a 256-texel RGBA8 row, clamp to edge or
// repeat in u: TextureSamplingFlags::REPEAT_U, renderer/src/paint.rs:469-474).
// A NaN coordinate gives transparent black.
template <typename T>
void o_ramp_sample(const OGrad& g, T u, T out[4]) {
    if (g.wrap == PF_GRADIENT_WRAP_REPEAT) u = u - std::floor(u);
    if (std::isnan(u)) { out[0] = out[1] = out[2] = out[3] = (T)0; return; }
    u = std::min(std::max(u, (T)-1), (T)2);
    T x = u * (T)256 - (T)0.5;
    T x0 = std::floor(x), w1 = x - x0;
    int i0 = (int)x0, i1 = i0 + 1;
    if (g.wrap == PF_GRADIENT_WRAP_REPEAT) { i0 &= 255; i1 &= 255; }
    else { i0 = std::min(std::max(i0, 0), 255); i1 = std::min(std::max(i1, 0), 255); }
    const PFColorU a = g.ramp[i0], b = g.ramp[i1];
    const T ca[4] = {(T)a.r, (T)a.g, (T)a.b, (T)a.a}, cb[4] = {(T)b.r, (T)b.g, (T)b.b, (T)b.a};
    for (int c = 0; c < 4; c++) out[c] = (ca[c] * ((T)1 - w1) + cb[c] * w1) / (T)255;
}

// One sample of a pattern's page at UV (u, v): linear filtering or the
// nearest texel, each axis repeated or clamped to the edge
// (renderer/src/paint.rs:537-548).  A NaN coordinate gives transparent black.
template <typename T>
void o_page_sample(const OGrad& g, T u, T v, T out[4]) {
    const bool rx = (g.flags & PF_PATTERN_REPEAT_X) != 0, ry = (g.flags & PF_PATTERN_REPEAT_Y) != 0;
    if (rx) u = u - std::floor(u);
    if (ry) v = v - std::floor(v);
    if (std::isnan(u) || std::isnan(v)) { out[0] = out[1] = out[2] = out[3] = (T)0; return; }
    u = std::min(std::max(u, (T)-1), (T)2);
    v = std::min(std::max(v, (T)-1), (T)2);
    const int W = g.pw, H = g.ph;
    auto wx_ = [&](long i) { return (int)(rx ? ((i % W) + W) % W : std::min<long>(std::max<long>(i, 0), W - 1)); };
    auto wy_ = [&](long i) { return (int)(ry ? ((i % H) + H) % H : std::min<long>(std::max<long>(i, 0), H - 1)); };
    auto texel = [&](int x, int y, T c[4]) {
        const PFColorU p = g.page[(size_t)y * W + x];
        c[0] = (T)p.r / (T)255; c[1] = (T)p.g / (T)255; c[2] = (T)p.b / (T)255; c[3] = (T)p.a / (T)255;
    };
    if (g.flags & PF_PATTERN_NO_SMOOTHING) {
        texel(wx_((long)std::floor(u * (T)W)), wy_((long)std::floor(v * (T)H)), out);
        return;
    }
    T x = u * (T)W - (T)0.5, y = v * (T)H - (T)0.5;
    T x0 = std::floor(x), y0 = std::floor(y), fx = x - x0, fy = y - y0;
    int ix0 = wx_((long)x0), ix1 = wx_((long)x0 + 1), iy0 = wy_((long)y0), iy1 = wy_((long)y0 + 1);
    T c00[4], c10[4], c01[4], c11[4];
    texel(ix0, iy0, c00); texel(ix1, iy0, c10); texel(ix0, iy1, c01); texel(ix1, iy1, c11);
    for (int k = 0; k < 4; k++) {
        T top = c00[k] + (c10[k] - c00[k]) * fx, bot = c01[k] + (c11[k] - c01[k]) * fx;
        out[k] = top + (bot - top) * fy;
    }
}

// A pattern's colour through its filter: filterBlur (shaders/
// tile_fragment.inc.glsl:309-347) or filterColorMatrix (:349-359).
template <typename T>
void o_pattern_color(const OGrad& g, T u, T v, T out[4]) {
    if (g.filter == PF_PATTERN_FILTER_COLOR_MATRIX) {
        T c[4];
        o_page_sample<T>(g, u, v, c);
        const float* m = g.matrix;
        for (int k = 0; k < 4; k++)
            out[k] = (T)m[k] * c[0] + (T)m[4 + k] * c[1] + (T)m[8 + k] * c[2] + (T)m[12 + k] * c[3] + (T)m[16 + k];
        return;
    }
    if (g.filter != PF_PATTERN_FILTER_BLUR_X && g.filter != PF_PATTERN_FILTER_BLUR_Y) {
        o_page_sample<T>(g, u, v, out);
        return;
    }
    const T sx = (T)g.blur[0] / (T)g.pw, sy = (T)g.blur[1] / (T)g.ph;
    const int support = (int)g.blur[2];
    T gx = g.blur[3], gy = g.blur[4];
    const T gz = g.blur[5];
    T sum = gx, c[4];
    o_page_sample<T>(g, u, v, c);
    for (int k = 0; k < 4; k++) c[k] *= gx;
    gx *= gy; gy *= gz;
    for (int i = 1; i <= support; i += 2) {
        T partial = gx;
        gx *= gy; gy *= gz;
        partial += gx;
        T o = (T)i + gx / partial;
        T a[4], b[4];
        o_page_sample<T>(g, u - sx * o, v - sy * o, a);
        o_page_sample<T>(g, u + sx * o, v + sy * o, b);
        for (int k = 0; k < 4; k++) c[k] += (a[k] + b[k]) * partial;
        sum += (T)2 * partial;
        gx *= gy; gy *= gz;
    }
    for (int k = 0; k < 4; k++) out[k] = c[k] / sum;
}

// The gradient's straight colour at pixel centre (px, py): linear, the ramp at
// u; radial, filterRadialGradient (shaders/tile_fragment.inc.glsl:274-307).
template <typename T>
void o_gradient_color(const OGrad& g, const float t[6], T px, T py, T out[4]) {
    T u = (T)t[0] * px + (T)t[1] * py + (T)t[2];
    if (g.kind == kOPattern) {
        o_pattern_color<T>(g, u, (T)t[3] * px + (T)t[4] * py + (T)t[5], out);
        return;
    }
    if (g.kind == PF_GRADIENT_LINEAR) { o_ramp_sample<T>(g, u, out); return; }
    T v = (T)t[3] * px + (T)t[4] * py + (T)t[5];
    T dpx = u - (T)g.fx, dpy = v - (T)g.fy, dcx = g.vx, dcy = g.vy;
    T dr = (T)g.r1 - (T)g.r0, r0 = g.r0;
    T a = (dcx * dcx + dcy * dcy) - dr * dr;
    T b = (dpx * dcx + dpy * dcy) + r0 * dr;
    T c = (dpx * dpx + dpy * dpy) - r0 * r0;
    T disc = b * b - a * c;
    out[0] = out[1] = out[2] = out[3] = (T)0;
    if (disc != (T)0) {
        T sq = std::sqrt(disc);
        T lo = (sq + b) / a, hi = (-sq + b) / a;
        if (lo > hi) std::swap(lo, hi);
        o_ramp_sample<T>(g, lo >= (T)0 ? lo : hi, out);
    }
}

template <typename T> T o_clamp01(T v) { return std::min(std::max(v, (T)0), (T)1); }

// compositeRGB, one separable channel (shaders/tile_fragment.inc.glsl:420-517).
template <typename T>
T o_blend_channel(uint32_t mode, T d, T s) {
    auto screen = [](T dd, T ss) { return dd + ss - dd * ss; };
    auto hard = [&](T dd, T ss) { return ss <= (T)0.5 ? dd * (T)2 * ss : screen(dd, (T)2 * ss - (T)1); };
    auto dodge = [](T dd, T ss) { return dd == (T)0 ? (T)0 : (ss == (T)1 ? (T)1 : dd / ((T)1 - ss)); };
    switch (mode) {
    case PF_BLEND_MODE_MULTIPLY: return d * s;
    case PF_BLEND_MODE_SCREEN: return screen(d, s);
    case PF_BLEND_MODE_OVERLAY: return hard(s, d);
    case PF_BLEND_MODE_DARKEN: return std::min(d, s);
    case PF_BLEND_MODE_LIGHTEN: return std::max(d, s);
    case PF_BLEND_MODE_COLOR_DODGE: return dodge(d, s);
    case PF_BLEND_MODE_COLOR_BURN: return (T)1 - dodge((T)1 - d, (T)1 - s);
    case PF_BLEND_MODE_HARD_LIGHT: return hard(d, s);
    case PF_BLEND_MODE_SOFT_LIGHT: {
        T dark = d <= (T)0.25 ? (((T)16 * d - (T)12) * d + (T)4) * d : std::sqrt(d);
        T factor = s <= (T)0.5 ? d * ((T)1 - d) : dark - d;
        return d + (s * (T)2 - (T)1) * factor;
    }
    case PF_BLEND_MODE_DIFFERENCE: return std::fabs(d - s);
    default: return d + s - (T)2 * d * s;  // Exclusion
    }
}

// compositeRGBToHSL / compositeHSLToRGB (shaders/tile_fragment.inc.glsl:431-448).
template <typename T>
void o_rgb_to_hsl(const T rgb[3], T hsl[3]) {
    const T pi3 = (T)1.0471975511965976;
    T v = std::max(std::max(rgb[0], rgb[1]), rgb[2]), lo = std::min(std::min(rgb[0], rgb[1]), rgb[2]);
    T c = v - lo, l = lo + (v - lo) * (T)0.5;
    T tx, ty, tz;
    if (rgb[0] == v) { tx = 0; ty = rgb[1]; tz = rgb[2]; }
    else if (rgb[1] == v) { tx = 2; ty = rgb[2]; tz = rgb[0]; }
    else { tx = 4; ty = rgb[0]; tz = rgb[1]; }
    hsl[0] = pi3 * (c != (T)0 ? (tx * c + ty - tz) / c : (T)0);
    hsl[1] = v != (T)0 ? c / v : (T)0;
    hsl[2] = l;
}
template <typename T>
void o_hsl_to_rgb(const T hsl[3], T rgb[3]) {
    const T six_pi = (T)1.9098593171027443;
    T a = hsl[1] * std::min(hsl[2], (T)1 - hsl[2]);
    const T k0[3] = {0, 8, 4};
    for (int i = 0; i < 3; i++) {
        T k = k0[i] + hsl[0] * six_pi;
        k = k - (T)12 * std::floor(k / (T)12);
        rgb[i] = hsl[2] - std::min(std::max(std::min(k - (T)3, (T)9 - k), (T)-1), (T)1) * a;
    }
}

// One pixel of a draw: straight source colour s, alpha a (paint alpha x
// coverage), premultiplied destination dst (4 channels, or alpha alone).
// Porter-Duff modes by their blend factors (renderer/src/gpu/blend.rs:42-144;
// Copy writes the source unblended); the others by the shader's composite()
// (shaders/tile_fragment.inc.glsl:519-537, output alpha 1).  Each result is
// clamped to [0, 1] as a UNORM framebuffer holds it.
template <typename T>
void o_blend(uint32_t mode, const T s[3], T a, T* dst, int channels) {
    T& da_ref = dst[channels == 4 ? 3 : 0];
    const T da = da_ref;
    if (mode <= PF_BLEND_MODE_LIGHTER) {
        T fs = 1, fd = (T)1 - a;
        switch (mode) {
        case PF_BLEND_MODE_CLEAR: fs = 0; fd = 0; break;
        case PF_BLEND_MODE_COPY: fs = 1; fd = 0; break;
        case PF_BLEND_MODE_SRC_IN: fs = da; fd = 0; break;
        case PF_BLEND_MODE_SRC_OUT: fs = (T)1 - da; fd = 0; break;
        case PF_BLEND_MODE_SRC_ATOP: fs = da; fd = (T)1 - a; break;
        case PF_BLEND_MODE_DEST_IN: fs = 0; fd = a; break;
        case PF_BLEND_MODE_DEST_OUT: fs = 0; fd = (T)1 - a; break;
        case PF_BLEND_MODE_DEST_OVER: fs = (T)1 - da; fd = 1; break;
        case PF_BLEND_MODE_DEST_ATOP: fs = (T)1 - da; fd = a; break;
        case PF_BLEND_MODE_XOR: fs = (T)1 - da; fd = (T)1 - a; break;
        case PF_BLEND_MODE_LIGHTER: fs = 1; fd = 1; break;
        default: break;  // SrcOver
        }
        if (channels == 4)
            for (int c = 0; c < 3; c++) dst[c] = o_clamp01(s[c] * a * fs + dst[c] * fd);
        da_ref = o_clamp01(a * fs + da * fd);
        return;
    }
    if (channels == 4) {
        // the destination composite() reads is a copy of the RGBA8 framebuffer
        // (renderer/src/gpu/d3d9/renderer.rs:405-407): quantised to 8 bits
        for (int c = 0; c < 3; c++) dst[c] = std::nearbyint(o_clamp01(dst[c]) * (T)255) / (T)255;
        const T dq = std::nearbyint(o_clamp01(da) * (T)255) / (T)255;
        T b[3];
        if (mode >= PF_BLEND_MODE_HUE) {
            T dh[3], sh[3];
            o_rgb_to_hsl<T>(dst, dh);
            o_rgb_to_hsl<T>(s, sh);
            T h[3] = {dh[0], dh[1], dh[2]};
            if (mode == PF_BLEND_MODE_HUE) h[0] = sh[0];
            else if (mode == PF_BLEND_MODE_SATURATION) h[1] = sh[1];
            else if (mode == PF_BLEND_MODE_COLOR) { h[0] = sh[0]; h[1] = sh[1]; }
            else h[2] = sh[2];
            o_hsl_to_rgb<T>(h, b);
        } else {
            for (int c = 0; c < 3; c++) b[c] = o_blend_channel<T>(mode, dst[c], s[c]);
        }
        for (int c = 0; c < 3; c++)
            dst[c] = o_clamp01(a * ((T)1 - dq) * s[c] + a * dq * b[c] + ((T)1 - a) * dst[c]);
    }
    da_ref = 1;
}

// Tile composite (shaders/d3d11/tile.cs.glsl:91-159 with calculateColor,
// shaders/tile_fragment.inc.glsl:560-613, and SrcOver, renderer/src/gpu/blend.rs:54-62):
// back to front in draw order; occluded tiles (path index < z) are skipped
// (shaders/d3d9/tile.vs.glsl:51-55).
template <typename T>
void composite(const Frame& fr, const std::vector<T>& masks, int w, int h, const T bg[4],
               std::vector<T>& fb, int channels, int threads, int ox = 0, int oy = 0) {
    // The image covers pixels [ox, ox + w) x [oy, oy + h) of the scene.
    fb.assign((size_t)w * h * channels, (T)0);
    for (size_t k = 0; k < (size_t)w * h; k++)
        for (int c = 0; c < channels; c++) fb[k * channels + c] = bg[channels == 4 ? c : 3];
    int32_t sw = std::max(0, fr.screen.width());
    // Rows of screen tiles are independent: parallelise over tile rows.
    int32_t ty0 = fr.screen.miny, ty1 = fr.screen.maxy;
    parallel_for((uint32_t)std::max(0, ty1 - ty0), threads, [&](uint32_t row) {
        int32_t ty = ty0 + (int32_t)row;
        std::vector<T> cov(256);
        for (uint32_t d = 0; d < fr.draw_count; d++) {
            uint32_t p = fr.clip_count + d;
            const BuiltPath& bp = fr.built[p];
            const PathInput& in = fr.paths[p];
            if (ty < bp.tile_rect.miny || ty >= bp.tile_rect.maxy) continue;
            int32_t bw = bp.tile_rect.width();
            for (int32_t x = 0; x < bw; x++) {
                size_t i = (size_t)(ty - bp.tile_rect.miny) * bw + x;
                const OTile& t = bp.tiles[i];
                if (t.alpha_tile_id == kInvalid && t.backdrop == 0) continue;
                if (fr.screen.contains(t.tile_x, t.tile_y)) {
                    int32_t z = fr.zbuf[(size_t)(t.tile_y - fr.screen.miny) * sw + (t.tile_x - fr.screen.minx)];
                    if ((int32_t)d < z) continue;
                }
                tile_coverage<T>(fr, p, i, masks, cov.data());
                T col[4] = {(T)in.paint.r / (T)255, (T)in.paint.g / (T)255, (T)in.paint.b / (T)255,
                            (T)in.paint.a / (T)255};
                if (in.blend != PF_BLEND_MODE_SRC_OVER || in.gradient != 0) {
                    const OGrad* g = in.gradient ? &fr.grads[in.gradient - 1] : nullptr;
                    float tt[6];
                    if (g) o_frame_transform(fr, *g, tt);
                    for (int py = 0; py < 16; py++) {
                        int Y = t.tile_y * 16 + py - oy;
                        if (Y < 0 || Y >= h) continue;
                        for (int px = 0; px < 16; px++) {
                            int X = t.tile_x * 16 + px - ox;
                            if (X < 0 || X >= w) continue;
                            T src[4] = {col[0], col[1], col[2], col[3]};
                            if (g) {  // combineColor0 SrcIn (shaders/tile_fragment.inc.glsl:81-89)
                                T tex[4];
                                o_gradient_color<T>(*g, tt, (T)(X + ox) + (T)0.5, (T)(Y + oy) + (T)0.5, tex);
                                src[0] = tex[0]; src[1] = tex[1]; src[2] = tex[2]; src[3] = tex[3] * col[3];
                            }
                            o_blend<T>(in.blend, src, src[3] * cov[py * 16 + px], &fb[((size_t)Y * w + X) * channels],
                                       channels);
                        }
                    }
                    continue;
                }
                for (int py = 0; py < 16; py++) {
                    int Y = t.tile_y * 16 + py - oy;
                    if (Y < 0 || Y >= h) continue;
                    for (int px = 0; px < 16; px++) {
                        int X = t.tile_x * 16 + px - ox;
                        if (X < 0 || X >= w) continue;
                        T a = col[3] * cov[py * 16 + px];
                        T* dst = &fb[((size_t)Y * w + X) * channels];
                        if (channels == 4) {
                            for (int c = 0; c < 3; c++) dst[c] = col[c] * a + dst[c] * ((T)1 - a);
                            dst[3] = a + dst[3] * ((T)1 - a);
                        } else {
                            dst[0] = a + dst[0] * ((T)1 - a);
                        }
                    }
                }
            }
        }
    });
}

bool make_frame(const PFCUDASceneDesc* sc, const PFCUDABuildOptions* opts, Frame& fr) {
    if (!sc || sc->memory != PF_MEMORY_HOST) return false;
    fr.view_box = RectF{sc->view_box.origin.x, sc->view_box.origin.y, sc->view_box.lower_right.x,
                        sc->view_box.lower_right.y};
    fr.clip_count = sc->clip_path_count;
    fr.draw_count = sc->draw_path_count;
    uint32_t n = fr.clip_count + fr.draw_count;
    fr.paths.assign(n, PathInput());
    bool transform = false;
    PFTransform2F tf{};
    if (opts && opts->has_transform) {
        tf = opts->transform;
        // Transform2F::is_identity (geometry/src/transform2d.rs:218-220)
        transform = !(tf.m00 == 1.0f && tf.m01 == 0.0f && tf.m10 == 0.0f && tf.m11 == 1.0f &&
                      tf.vector.x == 0.0f && tf.vector.y == 0.0f);
    }
    fr.transformed.assign(transform ? n : 0, {});
    if ((sc->gradient_count && !sc->gradients) || (sc->pattern_count && !sc->patterns)) return false;
    fr.grads.assign((size_t)sc->gradient_count + sc->pattern_count, OGrad());
    for (uint32_t q = 0; q < sc->gradient_count; q++)
        if (!o_build_gradient(sc->gradients[q], fr.grads[q])) return false;
    for (uint32_t q = 0; q < sc->pattern_count; q++)
        if (!o_build_pattern(sc->patterns[q], fr.grads[sc->gradient_count + q])) return false;
    if (transform) {
        // render_transform = the build transform's inverse (renderer/src/builder.rs:168-171)
        float det = tf.m00 * tf.m11 - tf.m01 * tf.m10;
        if (det != 0.0f) {
            float r = 1.0f / det;
            float a = r * tf.m11, b = r * -tf.m01, c = r * -tf.m10, d = r * tf.m00;
            float inv[6] = {a, b, -(a * tf.vector.x + b * tf.vector.y), c, d, -(c * tf.vector.x + d * tf.vector.y)};
            std::copy(inv, inv + 6, fr.inv);
        }
    }
    for (uint32_t p = 0; p < n; p++) {
        const PFCUDAPath& src = p < fr.clip_count ? sc->clip_paths[p] : sc->draw_paths[p - fr.clip_count];
        PathInput& in = fr.paths[p];
        in.is_clip = p < fr.clip_count;
        in.path_index = in.is_clip ? p : p - fr.clip_count;
        in.fill_rule = src.fill_rule;
        in.clip_path = src.clip_path;  // clip paths may be clipped too (clip chains)
        in.paint = src.paint;
        if (!in.is_clip) {
            if (src.blend_mode >= PF_BLEND_MODE_COUNT || src.overlay > sc->gradient_count + sc->pattern_count)
                return false;
            in.blend = src.blend_mode;
            in.gradient = src.overlay;
            // opaque paint (Paint::is_opaque, renderer/src/paint.rs:163-177) with a
            // blend mode that hides the backdrop (content/src/effects.rs:202-230)
            bool opaque = src.paint.a == 255 && (src.overlay == 0 || fr.grads[src.overlay - 1].opaque);
            in.occludes = opaque && (src.blend_mode == PF_BLEND_MODE_SRC_OVER || src.blend_mode == PF_BLEND_MODE_CLEAR);
        }
        if (src.clip_path >= (int32_t)fr.clip_count) return false;
        if (in.is_clip && src.clip_path == (int32_t)p) return false;
        if (transform) {
            // Contour::transform (content/src/outline.rs:884-893), Transform2F * Vector2F
            // (geometry/src/transform2d.rs:123-129, :312-318).
            std::vector<PFVector2F>& tp = fr.transformed[p];
            uint32_t a = sc->contour_starts[src.first_contour];
            uint32_t b = sc->contour_starts[src.first_contour + src.contour_count];
            tp.resize(b - a);
            for (uint32_t i = a; i < b; i++) {
                float x = sc->points[i].x, y = sc->points[i].y;
                float hx = tf.m00 * x, hy = tf.m10 * x, hz = tf.m01 * y, hw = tf.m11 * y;
                tp[i - a] = PFVector2F{(hx + hz) + tf.vector.x, (hy + hw) + tf.vector.y};
            }
            for (uint32_t c = 0; c < src.contour_count; c++) {
                uint32_t s0 = sc->contour_starts[src.first_contour + c];
                uint32_t s1 = sc->contour_starts[src.first_contour + c + 1];
                in.contours.push_back(Contour{tp.data() + (s0 - a), sc->point_flags + s0, s1 - s0});
            }
        } else {
            for (uint32_t c = 0; c < src.contour_count; c++) {
                uint32_t s0 = sc->contour_starts[src.first_contour + c];
                uint32_t s1 = sc->contour_starts[src.first_contour + c + 1];
                in.contours.push_back(Contour{sc->points + s0, sc->point_flags + s0, s1 - s0});
            }
        }
    }
    for (uint32_t p = 0; p < n; p++) {  // no cycles of clip paths
        uint32_t len = 0;
        for (int32_t q = fr.paths[p].clip_path; q >= 0; q = fr.paths[(uint32_t)q].clip_path)
            if (++len > fr.clip_count) return false;
    }
    return true;
}

// ---------------------------------------------------------------------------
// FP64 differentiable frame and its adjoint (checker of the CUDA adjoint)
// ---------------------------------------------------------------------------
// With each curve's subdivision held fixed, the CUDA level's differentiable
// frame is a function of the control points and the paint alphas: every
// flattened line runs between the curve points at the dyadic parameters
// [addr, addr + 1) / 2^depth that process_segment's recursion
// (renderer/src/tiler.rs:166-184) picks for the uploaded FP32 points.  Here it
// is evaluated in FP64: per path the integral of the winding number over each
// pixel (the trapezoid areas below each line, fill_area.inc.glsl:11-27, plus
// the backdrop carried down the column, taken over whole pixel columns rather
// than 16x16 tiles), the sampleMask resolve, the clip combine min(|d|, |s|)
// (tile_clip_combine.fs.glsl:27-30), SrcOver of alpha x coverage, and the
// adjoint of all of it from the first variation of the winding integral: a
// line A -> B moved by dP(u) = (1-u) dA + u dB changes a pixel's integral by
// the integral of dP . n over the part of the line inside the pixel,
// n = (-(B-A).y, (B-A).x).  The pixels a line crosses come from exact lists of
// its grid crossings.  Derivatives at the resolve's kinks are one-sided like
// the CUDA level's: nonzero d|c|/dc = +1 at c = 0 and 0 at |c| >= 1; even-odd
// +1 below the fold at 1 and -1 from it on; ties of the clip min go to the
// draw path.
struct DSeg {
    int kind;
    uint32_t idx[4];  // first, first + 1, first + 2, end (unused slots repeat)
    std::vector<std::pair<double, double>> leaves;
};
struct DPath {
    std::vector<DSeg> segs;
    bool even_odd = false, is_clip = false;
    int32_t clip = -1;                   // global index of the clip path
    int bx0 = 0, by0 = 0, bx1 = 0, by1 = 0;  // pixel box of the last render
    std::vector<double> w;               // winding integral over the box
    std::vector<double> lines;           // 4 per line (last render)
    std::vector<uint32_t> line_seg, line_leaf;
};
struct DiffFrame {
    int W = 0, H = 0, X0 = 0, Y0 = 0, X1 = 0, Y1 = 0;  // pixels inside the image and the view box
    bool transform = false;
    double m[6] = {1, 0, 0, 1, 0, 0};
    uint32_t np = 0, nclip = 0, ndraw = 0;
    uint64_t line_count = 0;
    bool limit_hit = false;
    std::vector<DPath> paths;            // clip paths, then draw paths
    std::vector<double> alpha;           // last render
    std::vector<std::vector<double>> cov, dprev, dd, dc;  // per draw path over its box
    bool rendered = false;
};

void flatten_leaves(const Segment& s, int depth, uint64_t addr, std::vector<std::pair<double, double>>& out,
                    bool* limit) {
    if (s.kind == kQuad) { flatten_leaves(to_cubic(s), depth, addr, out, limit); return; }
    if (s.kind == kLine || is_flat(s) || depth >= 32) {
        if (depth >= 32 && !is_flat(s)) *limit = true;
        out.push_back({std::ldexp((double)addr, -depth), std::ldexp((double)(addr + 1), -depth)});
        return;
    }
    Segment a, b;
    split_half(s, &a, &b);
    flatten_leaves(a, depth + 1, addr * 2, out, limit);
    flatten_leaves(b, depth + 1, addr * 2 + 1, out, limit);
}

bool make_diff_frame(const PFCUDASceneDesc* sc, const PFCUDABuildOptions* opts, int W, int H, DiffFrame& d) {
    if (!sc || sc->memory != PF_MEMORY_HOST || W <= 0 || H <= 0) return false;
    d.W = W; d.H = H;
    d.X0 = std::max(0, (int)std::ceil(sc->view_box.origin.x));
    d.Y0 = std::max(0, (int)std::ceil(sc->view_box.origin.y));
    d.X1 = std::min(W, (int)std::floor(sc->view_box.lower_right.x));
    d.Y1 = std::min(H, (int)std::floor(sc->view_box.lower_right.y));
    d.np = sc->point_count;
    d.nclip = sc->clip_path_count;
    d.ndraw = sc->draw_path_count;
    PFTransform2F tf{};
    if (opts && opts->has_transform) {
        tf = opts->transform;
        d.transform = !(tf.m00 == 1.0f && tf.m01 == 0.0f && tf.m10 == 0.0f && tf.m11 == 1.0f &&
                        tf.vector.x == 0.0f && tf.vector.y == 0.0f);
    }
    if (d.transform) {
        d.m[0] = tf.m00; d.m[1] = tf.m01; d.m[2] = tf.m10; d.m[3] = tf.m11; d.m[4] = tf.vector.x; d.m[5] = tf.vector.y;
    }
    // FP32 points as the tiler sees them (Transform2F * Vector2F in FP32)
    std::vector<PFVector2F> p32(sc->points, sc->points + d.np);
    if (d.transform)
        for (PFVector2F& v : p32) {
            float hx = tf.m00 * v.x, hy = tf.m10 * v.x, hz = tf.m01 * v.y, hw = tf.m11 * v.y;
            v = PFVector2F{(hx + hz) + tf.vector.x, (hy + hw) + tf.vector.y};
        }
    auto is_end = [&](uint32_t i) {
        return (sc->point_flags[i] & (PF_POINT_FLAG_CONTROL_POINT_0 | PF_POINT_FLAG_CONTROL_POINT_1)) == 0;
    };
    const uint32_t n = d.nclip + d.ndraw;
    d.paths.assign(n, DPath());
    for (uint32_t p = 0; p < n; p++) {
        const PFCUDAPath& src = p < d.nclip ? sc->clip_paths[p] : sc->draw_paths[p - d.nclip];
        DPath& dp = d.paths[p];
        dp.is_clip = p < d.nclip;
        dp.even_odd = src.fill_rule == PF_FILL_RULE_EVEN_ODD;
        if (!dp.is_clip && src.clip_path >= (int32_t)d.nclip) return false;
        if (dp.is_clip && src.clip_path >= 0) return false;  // clip chains: not differentiable here
        dp.clip = (!dp.is_clip && src.clip_path >= 0) ? src.clip_path : -1;
        for (uint32_t c = 0; c < src.contour_count; c++) {
            const uint32_t s0 = sc->contour_starts[src.first_contour + c];
            const uint32_t len = sc->contour_starts[src.first_contour + c + 1] - s0;
            if (len == 0) continue;
            // ContourIter::next (content/src/outline.rs:1024-1065) by point index
            uint32_t index = 1;
            for (;;) {
                if (index == len + 1) break;
                DSeg sg{};
                const uint32_t i0 = s0 + index - 1;
                if (index == len) {
                    sg.kind = kLine; sg.idx[0] = i0; sg.idx[1] = sg.idx[2] = i0; sg.idx[3] = s0;
                    index++;
                } else {
                    const uint32_t i1 = s0 + index++;
                    if (is_end(i1)) {
                        sg.kind = kLine; sg.idx[0] = i0; sg.idx[1] = sg.idx[2] = i0; sg.idx[3] = i1;
                    } else {
                        const uint32_t i2 = s0 + index++;
                        if (is_end(i2)) {
                            sg.kind = kQuad; sg.idx[0] = i0; sg.idx[1] = i1; sg.idx[2] = i0; sg.idx[3] = i2;
                        } else {
                            const uint32_t i3 = s0 + index++;
                            sg.kind = kCubic; sg.idx[0] = i0; sg.idx[1] = i1; sg.idx[2] = i2; sg.idx[3] = i3;
                        }
                    }
                }
                const PFVector2F a = p32[sg.idx[0]], e = p32[sg.idx[3]];
                Segment s32{Line{a.x, a.y, e.x, e.y}, Line{0, 0, 0, 0}, sg.kind};
                if (sg.kind == kQuad) s32.ctrl = Line{p32[sg.idx[1]].x, p32[sg.idx[1]].y, 0, 0};
                if (sg.kind == kCubic)
                    s32.ctrl = Line{p32[sg.idx[1]].x, p32[sg.idx[1]].y, p32[sg.idx[2]].x, p32[sg.idx[2]].y};
                flatten_leaves(s32, 0, 0, sg.leaves, &d.limit_hit);
                d.line_count += sg.leaves.size();
                dp.segs.push_back(std::move(sg));
            }
        }
    }
    return true;
}

// Bernstein weights of the slots (first, first + 1, first + 2, end) at t.
void diff_weights(int kind, double t, double w[4]) {
    const double s = 1.0 - t;
    if (kind == kCubic) { w[0] = s * s * s; w[1] = 3 * t * s * s; w[2] = 3 * t * t * s; w[3] = t * t * t; }
    else if (kind == kQuad) { w[0] = s * s; w[1] = 2 * t * s; w[2] = 0; w[3] = t * t; }
    else { w[0] = s; w[1] = 0; w[2] = 0; w[3] = t; }
}

// Winding integral of one path over its pixel box (rows clamp: what lies
// above the box is carried down the column, what lies below is dropped).
void diff_winding(DiffFrame& d, DPath& dp, const std::vector<double>& q) {
    dp.lines.clear(); dp.line_seg.clear(); dp.line_leaf.clear();
    double mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
    for (uint32_t si = 0; si < dp.segs.size(); si++) {
        const DSeg& sg = dp.segs[si];
        for (uint32_t li = 0; li < sg.leaves.size(); li++) {
            double e[4];
            for (int end = 0; end < 2; end++) {
                double w[4], x = 0, y = 0;
                diff_weights(sg.kind, end ? sg.leaves[li].second : sg.leaves[li].first, w);
                for (int k = 0; k < 4; k++) { x += w[k] * q[2 * sg.idx[k]]; y += w[k] * q[2 * sg.idx[k] + 1]; }
                e[2 * end] = x; e[2 * end + 1] = y;
            }
            for (double v : e) dp.lines.push_back(v);
            dp.line_seg.push_back(si);
            dp.line_leaf.push_back(li);
            mnx = std::min({mnx, e[0], e[2]}); mxx = std::max({mxx, e[0], e[2]});
            mny = std::min({mny, e[1], e[3]}); mxy = std::max({mxy, e[1], e[3]});
        }
    }
    dp.bx0 = std::max(d.X0, (int)std::floor(mnx)); dp.bx1 = std::min(d.X1, (int)std::ceil(mxx));
    dp.by0 = std::max(d.Y0, (int)std::floor(mny)); dp.by1 = std::min(d.Y1, (int)std::ceil(mxy));
    if (dp.lines.empty() || dp.bx1 <= dp.bx0 || dp.by1 <= dp.by0) { dp.bx1 = dp.bx0; dp.by1 = dp.by0; dp.w.clear(); return; }
    const int bw = dp.bx1 - dp.bx0, bh = dp.by1 - dp.by0;
    std::vector<double> acc((size_t)bw * bh, 0.0), carry((size_t)bw * bh, 0.0);
    const double Y0 = dp.by0, Y1 = dp.by1;
    for (size_t l = 0; l < dp.lines.size(); l += 4) {
        const double x0 = dp.lines[l], y0 = dp.lines[l + 1], x1 = dp.lines[l + 2], y1 = dp.lines[l + 3];
        if (x0 == x1) continue;
        const double slope = (y1 - y0) / (x1 - x0);
        const int c0 = std::max(dp.bx0, (int)std::floor(std::min(x0, x1)));
        const int c1 = std::min(dp.bx1 - 1, (int)std::ceil(std::max(x0, x1)) - 1);
        for (int px = c0; px <= c1; px++) {
            const double xa = std::min(std::max(x0, (double)px), (double)px + 1);
            const double xb = std::min(std::max(x1, (double)px), (double)px + 1);
            const double wdt = xa - xb;  // signed: right-to-left lines add area below them
            if (wdt == 0) continue;
            const double ya = y0 + (xa - x0) * slope, yb = y0 + (xb - x0) * slope;
            const double ylo = std::min(ya, yb), yhi = std::max(ya, yb);
            const int col = px - dp.bx0;
            auto add = [&](int r, double a, double cr) {
                acc[(size_t)(r - dp.by0) * bw + col] += a;
                if (r + 1 < dp.by1) carry[(size_t)(r + 1 - dp.by0) * bw + col] += cr;
            };
            // the part above the box covers every row of the column; the part
            // below it covers none
            if (yhi - ylo <= 0) {
                if (ylo < Y0) { carry[col] += wdt; continue; }
                const int r = (int)std::floor(ylo);
                if (r >= dp.by1) continue;
                add(r, wdt * ((double)(r + 1) - ylo), wdt);
                continue;
            }
            if (ylo < Y0) carry[col] += wdt * ((std::min(yhi, Y0) - ylo) / (yhi - ylo));
            const double ys = std::max(ylo, Y0), ye = std::min(yhi, Y1);
            if (!(ye > ys)) continue;
            const int r0 = (int)std::floor(ys), r1 = std::min((int)std::floor(ye), dp.by1 - 1);
            for (int r = r0; r <= r1; r++) {
                const double yt = std::max(ys, (double)r), yb2 = std::min(ye, (double)(r + 1));
                const double h = yb2 - yt;
                if (h <= 0) continue;
                const double wr = wdt * (h / (yhi - ylo));
                add(r, wr * ((double)(r + 1) - 0.5 * (yt + yb2)), wr);
            }
        }
    }
    dp.w.assign((size_t)bw * bh, 0.0);
    for (int x = 0; x < bw; x++) {
        double run = 0;
        for (int y = 0; y < bh; y++) {
            run += carry[(size_t)y * bw + x];
            dp.w[(size_t)y * bw + x] = acc[(size_t)y * bw + x] + run;
        }
    }
}

double diff_w_at(const DPath& dp, int X, int Y) {
    if (X < dp.bx0 || X >= dp.bx1 || Y < dp.by0 || Y >= dp.by1) return 0.0;
    return dp.w[(size_t)(Y - dp.by0) * (dp.bx1 - dp.bx0) + (X - dp.bx0)];
}

double diff_resolve(double c, bool even_odd, double* dcdw) {
    if (!even_odd) {
        const double a = std::fabs(c);
        *dcdw = a < 1.0 ? (c >= 0.0 ? 1.0 : -1.0) : 0.0;
        return std::min(1.0, a);
    }
    const double m = c - 2.0 * std::floor(c * 0.5);
    *dcdw = m < 1.0 ? 1.0 : -1.0;
    return std::min(1.0, 1.0 - std::fabs(1.0 - m));
}

void diff_transform(const DiffFrame& d, const double* pts, std::vector<double>& q) {
    q.assign((size_t)d.np * 2, 0.0);
    for (uint32_t i = 0; i < d.np; i++) {
        const double x = pts[2 * i], y = pts[2 * i + 1];
        q[2 * i] = d.transform ? d.m[0] * x + d.m[1] * y + d.m[4] : x;
        q[2 * i + 1] = d.transform ? d.m[2] * x + d.m[3] * y + d.m[5] : y;
    }
}

void diff_render(DiffFrame& d, const double* pts, const double* alpha, double bg, double* img) {
    std::vector<double> q;
    diff_transform(d, pts, q);
    for (DPath& dp : d.paths) diff_winding(d, dp, q);
    d.alpha.assign(alpha, alpha + d.ndraw);
    d.cov.assign(d.ndraw, {}); d.dprev.assign(d.ndraw, {}); d.dd.assign(d.ndraw, {}); d.dc.assign(d.ndraw, {});
    for (size_t k = 0; k < (size_t)d.W * d.H; k++) img[k] = bg;
    for (uint32_t k = 0; k < d.ndraw; k++) {
        const DPath& dp = d.paths[d.nclip + k];
        const int bw = dp.bx1 - dp.bx0, bh = dp.by1 - dp.by0;
        const size_t nb = (size_t)std::max(bw, 0) * std::max(bh, 0);
        d.cov[k].assign(nb, 0); d.dprev[k].assign(nb, 0); d.dd[k].assign(nb, 0); d.dc[k].assign(nb, 0);
        for (int y = 0; y < bh; y++)
            for (int x = 0; x < bw; x++) {
                const int X = dp.bx0 + x, Y = dp.by0 + y;
                const size_t i = (size_t)y * bw + x;
                const double wd = dp.w[i];
                double c, dcdm, ddv = 0, dcv = 0;
                if (dp.clip >= 0) {
                    const double wc = diff_w_at(d.paths[dp.clip], X, Y);
                    const bool own = std::fabs(wd) <= std::fabs(wc);
                    c = diff_resolve(std::min(std::fabs(wd), std::fabs(wc)), dp.even_odd, &dcdm);
                    const double s = ((own ? wd : wc) >= 0.0) ? 1.0 : -1.0;
                    (own ? ddv : dcv) = dcdm * s;
                } else {
                    c = diff_resolve(wd, dp.even_odd, &dcdm);
                    ddv = dcdm;
                }
                double& dst = img[(size_t)Y * d.W + X];
                d.cov[k][i] = c; d.dprev[k][i] = dst; d.dd[k][i] = ddv; d.dc[k][i] = dcv;
                const double a = d.alpha[k] * c;
                dst = a + dst * (1.0 - a);
            }
    }
    d.rendered = true;
}

void diff_grad(DiffFrame& d, const double* dimg, double* dpts, double* dalpha) {
    std::vector<double> G(dimg, dimg + (size_t)d.W * d.H);
    std::vector<std::vector<double>> gw(d.paths.size());
    for (size_t p = 0; p < d.paths.size(); p++) gw[p].assign(d.paths[p].w.size(), 0.0);
    for (uint32_t k = 0; k < d.ndraw; k++) dalpha[k] = 0;
    for (uint32_t k = d.ndraw; k-- > 0;) {
        const uint32_t p = d.nclip + k;
        const DPath& dp = d.paths[p];
        const int bw = dp.bx1 - dp.bx0, bh = dp.by1 - dp.by0;
        for (int y = 0; y < bh; y++)
            for (int x = 0; x < bw; x++) {
                const int X = dp.bx0 + x, Y = dp.by0 + y;
                const size_t i = (size_t)y * bw + x;
                double& g = G[(size_t)Y * d.W + X];
                const double c = d.cov[k][i], dlda = g * (1.0 - d.dprev[k][i]);
                dalpha[k] += dlda * c;
                const double dm = dlda * d.alpha[k];
                gw[p][i] += dm * d.dd[k][i];
                if (dp.clip >= 0 && d.dc[k][i] != 0) {
                    const DPath& cp = d.paths[dp.clip];
                    if (X >= cp.bx0 && X < cp.bx1 && Y >= cp.by0 && Y < cp.by1)
                        gw[dp.clip][(size_t)(Y - cp.by0) * (cp.bx1 - cp.bx0) + (X - cp.bx0)] += dm * d.dc[k][i];
                }
                g *= 1.0 - d.alpha[k] * c;
            }
    }
    std::vector<double> dq((size_t)d.np * 2, 0.0);
    std::vector<double> us;
    for (size_t p = 0; p < d.paths.size(); p++) {
        const DPath& dp = d.paths[p];
        if (dp.w.empty()) continue;
        const int bw = dp.bx1 - dp.bx0;
        for (size_t l = 0; l < dp.line_seg.size(); l++) {
            const double x0 = dp.lines[4 * l], y0 = dp.lines[4 * l + 1];
            const double dx = dp.lines[4 * l + 2] - x0, dy = dp.lines[4 * l + 3] - y0;
            if (dx == 0 && dy == 0) continue;
            us.assign({0.0, 1.0});
            if (dx != 0)
                for (double k = std::floor(std::min(x0, x0 + dx)) + 1; k < std::max(x0, x0 + dx); k += 1) {
                    const double u = (k - x0) / dx;
                    if (u > 0 && u < 1) us.push_back(u);
                }
            if (dy != 0)
                for (double k = std::floor(std::min(y0, y0 + dy)) + 1; k < std::max(y0, y0 + dy); k += 1) {
                    const double u = (k - y0) / dy;
                    if (u > 0 && u < 1) us.push_back(u);
                }
            std::sort(us.begin(), us.end());
            double GA = 0, GB = 0;
            for (size_t j = 0; j + 1 < us.size(); j++) {
                const double u0 = us[j], u1 = us[j + 1];
                if (!(u1 > u0)) continue;
                const double um = 0.5 * (u0 + u1);
                const int X = (int)std::floor(x0 + um * dx), Y = (int)std::floor(y0 + um * dy);
                if (X < dp.bx0 || X >= dp.bx1 || Y < dp.by0 || Y >= dp.by1) continue;
                const double g = gw[p][(size_t)(Y - dp.by0) * bw + (X - dp.bx0)];
                GA += g * (u1 - u0) * (1.0 - um);
                GB += g * (u1 - u0) * um;
            }
            const DSeg& sg = dp.segs[dp.line_seg[l]];
            const auto& lf = sg.leaves[dp.line_leaf[l]];
            double wa[4], wb[4];
            diff_weights(sg.kind, lf.first, wa);
            diff_weights(sg.kind, lf.second, wb);
            const int used[4] = {1, sg.kind != kLine, sg.kind == kCubic, 1};
            for (int k = 0; k < 4; k++) {
                if (!used[k]) continue;
                const double c = wa[k] * GA + wb[k] * GB;
                dq[2 * sg.idx[k]] += c * -dy;
                dq[2 * sg.idx[k] + 1] += c * dx;
            }
        }
    }
    for (uint32_t i = 0; i < d.np; i++) {
        const double gx = dq[2 * i], gy = dq[2 * i + 1];
        dpts[2 * i] = d.transform ? d.m[0] * gx + d.m[2] * gy : gx;
        dpts[2 * i + 1] = d.transform ? d.m[1] * gx + d.m[3] * gy : gy;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// C API (ctypes, test infrastructure)
// ---------------------------------------------------------------------------
struct PFOFrame {
    Frame fr;
    std::vector<double> masks64;
    bool masks_ready = false;
};

extern "C" {

// flags: PF_CUDA_RENDERER_D3D11_SEMANTICS for the D3D11 level's tiling.
PFOFrame* pfo_build(const PFCUDASceneDesc* scene, const PFCUDABuildOptions* opts, int threads,
                    uint64_t dda_limit, int32_t flags) {
    PFOFrame* f = new PFOFrame();
    if (!make_frame(scene, opts, f->fr)) { delete f; return nullptr; }
    f->fr.d3d11 = (flags & PF_CUDA_RENDERER_D3D11_SEMANTICS) != 0;
    build_frame(f->fr, threads, dda_limit ? dda_limit : (1ull << 24));
    return f;
}

void pfo_free(PFOFrame* f) { delete f; }

// counts[0..7] = paths, tiles, fills, alpha tiles, lines, screen tiles, limit_hit, clip paths
void pfo_counts(const PFOFrame* f, uint64_t* counts) {
    const Frame& fr = f->fr;
    uint64_t lines = 0;
    for (const BuiltPath& bp : fr.built) lines += bp.line_count;
    counts[0] = fr.paths.size();
    counts[1] = fr.tile_offset.back();
    counts[2] = fr.fill_offset.back();
    counts[3] = fr.alpha_owner.size();
    counts[4] = lines;
    counts[5] = fr.zbuf.size();
    counts[6] = fr.limit_hit ? 1 : 0;
    counts[7] = fr.clip_count;
}

// Fills in emission order with the global index of their tile.
void pfo_fills(const PFOFrame* f, PFCUDAFill* fills, uint32_t* fill_tile) {
    const Frame& fr = f->fr;
    for (size_t p = 0; p < fr.paths.size(); p++) {
        const BuiltPath& bp = fr.built[p];
        for (size_t k = 0; k < bp.fills.size(); k++) {
            const OFill& o = bp.fills[k];
            size_t e = fr.fill_offset[p] + k;
            fills[e] = PFCUDAFill{o.fx, o.fy, o.tx, o.ty, (uint32_t)e};
            if (fill_tile) fill_tile[e] = (uint32_t)(fr.tile_offset[p] + o.local_tile);
        }
    }
}

void pfo_tiles(const PFOFrame* f, PFCUDATile* tiles, PFCUDAClip* clips, uint32_t* path_tile_offsets,
               PFRectI* rects, int32_t* backdrops_above /* sum of column widths, may be NULL */) {
    const Frame& fr = f->fr;
    size_t col = 0;
    for (size_t p = 0; p < fr.paths.size(); p++) {
        const BuiltPath& bp = fr.built[p];
        const PathInput& in = fr.paths[p];
        if (path_tile_offsets) path_tile_offsets[p] = (uint32_t)fr.tile_offset[p];
        if (rects) rects[p] = PFRectI{{bp.tile_rect.minx, bp.tile_rect.miny}, {bp.tile_rect.maxx, bp.tile_rect.maxy}};
        for (size_t i = 0; i < bp.tiles.size(); i++) {
            const OTile& t = bp.tiles[i];
            size_t g = fr.tile_offset[p] + i;
            if (tiles) tiles[g] = PFCUDATile{t.tile_x, t.tile_y, t.alpha_tile_id, in.path_index, t.color, t.ctrl, t.backdrop};
            if (clips) {
                if (!bp.clips.empty()) {
                    const OClip& c = bp.clips[i];
                    clips[g] = PFCUDAClip{c.dest_tile_id, c.dest_backdrop, c.src_tile_id, c.src_backdrop};
                } else {
                    clips[g] = PFCUDAClip{kInvalid, 0, kInvalid, 0};
                }
            }
        }
        if (backdrops_above)
            for (size_t c = 0; c < bp.backdrops.size(); c++) backdrops_above[col + c] = bp.backdrops[c];
        col += bp.backdrops.size();
    }
    if (path_tile_offsets) path_tile_offsets[fr.paths.size()] = (uint32_t)fr.tile_offset.back();
}

void pfo_zbuffer(const PFOFrame* f, int32_t* z, PFRectI* screen) {
    const Frame& fr = f->fr;
    if (z) std::memcpy(z, fr.zbuf.data(), fr.zbuf.size() * sizeof(int32_t));
    if (screen) *screen = PFRectI{{fr.screen.minx, fr.screen.miny}, {fr.screen.maxx, fr.screen.maxy}};
}

// FP64 raw alpha masks [A][256] and resolved coverage per path tile [T][256].
void pfo_masks(PFOFrame* f, double* alpha_masks, double* tile_cov, int threads) {
    Frame& fr = f->fr;
    if (!f->masks_ready) { compute_raw_masks<double>(fr, f->masks64, threads); f->masks_ready = true; }
    if (alpha_masks) std::memcpy(alpha_masks, f->masks64.data(), f->masks64.size() * sizeof(double));
    if (tile_cov)
        parallel_for((uint32_t)fr.paths.size(), threads, [&](uint32_t p) {
            for (size_t i = 0; i < fr.built[p].tiles.size(); i++)
                tile_coverage<double>(fr, p, i, f->masks64, &tile_cov[(fr.tile_offset[p] + i) * 256]);
        });
}

// Largest |gpu - oracle| of the raw alpha masks [A][256] and of the resolved
// coverage per path tile [T][256] against the FP64 values, computed tile by
// tile, so that full-size scenes need no FP64 copy of either array.
// out_err[0]: raw masks, out_err[1]: tile coverage; out_where[0..1]: the
// first alpha tile / path tile with the largest error.
void pfo_mask_error(PFOFrame* f, const float* gpu_alpha, const float* gpu_tile, double* out_err,
                    uint64_t* out_where, int threads) {
    Frame& fr = f->fr;
    if (!f->masks_ready) { compute_raw_masks<double>(fr, f->masks64, threads); f->masks_ready = true; }
    std::mutex m;
    double ea = 0.0, et = 0.0;
    uint64_t wa = 0, wt = 0;
    const uint32_t A = (uint32_t)(f->masks64.size() / 256);
    if (gpu_alpha)
        parallel_for((A + 1023) / 1024, threads, [&](uint32_t blk) {
            double e = 0.0;
            uint64_t w = 0;
            for (uint32_t a = blk * 1024; a < std::min(A, blk * 1024 + 1024); a++)
                for (int k = 0; k < 256; k++) {
                    const double d = std::fabs((double)gpu_alpha[(size_t)a * 256 + k] - f->masks64[(size_t)a * 256 + k]);
                    if (d > e) { e = d; w = a; }
                }
            std::lock_guard<std::mutex> g(m);
            if (e > ea || (e == ea && w < wa)) { ea = e; wa = w; }
        });
    if (gpu_tile)
        parallel_for((uint32_t)fr.paths.size(), threads, [&](uint32_t p) {
            double cov[256];
            double e = 0.0;
            uint64_t w = 0;
            for (size_t i = 0; i < fr.built[p].tiles.size(); i++) {
                tile_coverage<double>(fr, p, i, f->masks64, cov);
                const size_t g = fr.tile_offset[p] + i;
                for (int k = 0; k < 256; k++) {
                    const double d = std::fabs((double)gpu_tile[g * 256 + k] - cov[k]);
                    if (d > e) { e = d; w = g; }
                }
            }
            std::lock_guard<std::mutex> g(m);
            if (e > et || (e == et && w < wt)) { et = e; wt = w; }
        });
    out_err[0] = ea;
    out_err[1] = et;
    if (out_where) { out_where[0] = wa; out_where[1] = wt; }
}

// FP64 composite into premultiplied RGBA (channels=4, rounded to u8) or a
// single FP64 channel (channels=1).
void pfo_render(PFOFrame* f, int w, int h, const PFColorF* bg, int channels, uint8_t* out_rgba8,
                double* out_f64, int threads) {
    Frame& fr = f->fr;
    if (!f->masks_ready) { compute_raw_masks<double>(fr, f->masks64, threads); f->masks_ready = true; }
    double b[4] = {0, 0, 0, 0};
    if (bg) { b[0] = bg->r; b[1] = bg->g; b[2] = bg->b; b[3] = bg->a; }
    std::vector<double> fb;
    composite<double>(fr, f->masks64, w, h, b, fb, channels, threads);
    if (out_f64) std::memcpy(out_f64, fb.data(), fb.size() * sizeof(double));
    if (out_rgba8)
        for (size_t k = 0; k < fb.size(); k++) {
            double v = std::min(std::max(fb[k], 0.0), 1.0) * 255.0;
            out_rgba8[k] = (uint8_t)std::nearbyint(v);
        }
}

// Each glyph of an atlas scene rendered as its own scene, as a batch of glyph
// scenes is: the glyph's draw path alone, view box = its cell, written into the
// cell of a w x h R8 image (FP64 coverage and composite, rounded to u8).
// Glyphs are independent: parallel over glyphs, each built on one thread.
int32_t pfo_render_glyphs(const PFCUDASceneDesc* atlas, const PFRectI* cells, uint32_t n, int w, int h,
                          uint8_t* out, int threads) {
    if (!atlas || !cells || !out || n > atlas->draw_path_count) return 1;
    std::atomic<int32_t> status{0};
    parallel_for(n, threads, [&](uint32_t g) {
        PFCUDASceneDesc d = *atlas;
        d.clip_path_count = 0;
        d.clip_paths = nullptr;
        d.draw_paths = atlas->draw_paths + g;
        d.draw_path_count = 1;
        const PFRectI c = cells[g];
        d.view_box = PFRectF{{(float)c.origin.x, (float)c.origin.y}, {(float)c.lower_right.x, (float)c.lower_right.y}};
        Frame fr;
        if (!make_frame(&d, nullptr, fr)) { status = 1; return; }
        build_frame(fr, 1, 1ull << 24);
        std::vector<double> masks, fb;
        compute_raw_masks<double>(fr, masks, 1);
        const double bg[4] = {0, 0, 0, 0};
        const int cw = c.lower_right.x - c.origin.x, ch = c.lower_right.y - c.origin.y;
        if (cw <= 0 || ch <= 0) return;
        composite<double>(fr, masks, cw, ch, bg, fb, 1, 1, c.origin.x, c.origin.y);
        for (int y = 0; y < ch; y++)
            for (int x = 0; x < cw; x++) {
                const int X = c.origin.x + x, Y = c.origin.y + y;
                if (X < 0 || Y < 0 || X >= w || Y >= h) continue;
                const double v = std::min(std::max(fb[(size_t)y * cw + x], 0.0), 1.0) * 255.0;
                out[(size_t)Y * w + X] = (uint8_t)std::nearbyint(v);
            }
    });
    return status.load();
}

// The CPU baseline: tiling + FP32 coverage + FP32 composite, all on `threads`
// host threads.  Returns wall seconds; writes RGBA8 when out is non-NULL.
double pfo_cpu_frame(const PFCUDASceneDesc* scene, const PFCUDABuildOptions* opts, int w, int h,
                     int threads, uint8_t* out_rgba8, uint64_t* out_counts) {
    auto t0 = std::chrono::steady_clock::now();
    PFOFrame f;
    if (!make_frame(scene, opts, f.fr)) return -1.0;
    build_frame(f.fr, threads, 1ull << 24);
    std::vector<float> masks;
    compute_raw_masks<float>(f.fr, masks, threads);
    float b[4] = {0, 0, 0, 0};
    std::vector<float> fb;
    composite<float>(f.fr, masks, w, h, b, fb, 4, threads);
    if (out_rgba8)
        for (size_t k = 0; k < fb.size(); k++) {
            float v = std::min(std::max(fb[k], 0.0f), 1.0f) * 255.0f;
            out_rgba8[k] = (uint8_t)std::nearbyint(v);
        }
    auto t1 = std::chrono::steady_clock::now();
    if (out_counts) pfo_counts(&f, out_counts);
    return std::chrono::duration<double>(t1 - t0).count();
}

// FP64 exact area (utils/area-lut/src/main.rs:29-65) for the LUT pin.
double pfo_area(double y, double dydx) { return area_exact<double>(y, dydx); }
// The same formula in single precision, as the reference's LUT generator
// evaluates it: round(255 * area(y - k, dydx)) for LUT texel (u, v), channel k
// (utils/area-lut/src/main.rs:77-96).  Returns the 8-bit LUT value.
uint8_t pfo_area_lut_value(int u, int v, int k) {
    if (u == 0) return 255;
    if (u == 255) return 0;
    float y = ((float)u - 128.0f) / 16.0f;
    float dydx = -((float)v) / 16.0f;
    float a = area_exact<float>(y - (float)k, dydx) * 255.0f;
    float r = std::round(a);  // f32::round: half away from zero
    if (!(r > 0.0f)) return 0;  // `as u8` saturates (NaN -> 0)
    if (r > 255.0f) return 255;
    return (uint8_t)r;
}
// FP64 coverage of one fill over one 16x16 tile (the D3D9 fill quad).
void pfo_fill_coverage(const uint16_t seg[4], double* mask) {
    OFill f{seg[0], seg[1], seg[2], seg[3], 0, 0, 0};
    accumulate_fill<double>(f, mask);
}
int32_t pfo_sse_cvt(float x) { return sse_cvt(x); }

// ---- FP64 differentiable frame ---------------------------------------------
struct PFODiff { DiffFrame d; };

PFODiff* pfo_diff_build(const PFCUDASceneDesc* scene, const PFCUDABuildOptions* opts, int width, int height) {
    PFODiff* f = new PFODiff();
    if (!make_diff_frame(scene, opts, width, height, f->d)) { delete f; return nullptr; }
    return f;
}

void pfo_diff_free(PFODiff* f) { delete f; }

// info[0..4] = points, clip paths, draw paths, flattened lines, depth limit hit
void pfo_diff_info(const PFODiff* f, uint64_t* info) {
    info[0] = f->d.np; info[1] = f->d.nclip; info[2] = f->d.ndraw; info[3] = f->d.line_count;
    info[4] = f->d.limit_hit ? 1 : 0;
}

// points: 2 per scene point (input space); alpha: one per draw path; image: W x H.
void pfo_diff_render(PFODiff* f, const double* points, const double* alpha, double background, double* image) {
    diff_render(f->d, points, alpha, background, image);
}

// Adjoint of the last pfo_diff_render: dL/dimage -> dL/dpoints (2 per point), dL/dalpha.
int32_t pfo_diff_grad(PFODiff* f, const double* d_image, double* d_points, double* d_alpha) {
    if (!f->d.rendered) return -1;
    diff_grad(f->d, d_image, d_points, d_alpha);
    return 0;
}


// Gradient::sample of the gradient's stops (ordered as Gradient::add orders them).
int32_t pfo_gradient_sample(const PFCUDAGradient* g, float t, PFColorU* out) {
    if (!g || !out || (g->stop_count && !g->stops)) return 1;
    *out = o_gradient_sample(o_ordered_stops(*g), t);
    return 0;
}

float pfo_round_f16(float x) { return o_round_f16(x); }

}  // extern "C"

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
};

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
    if (!clip_line_segment_to_rect(seg, clip_box)) return;

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
        add_fill(ctx, Line{cx, cy, npx, npy}, tcx, tcy);

        if (stepy < 0 && dir == kY) {
            add_fill(ctx, Line{npx, npy, (float)tcx * 16.0f, (float)tcy * 16.0f}, tcx, tcy);
        } else if (stepy > 0 && last == kY) {
            add_fill(ctx, Line{(float)tcx * 16.0f, (float)tcy * 16.0f, cx, cy}, tcx, tcy);
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

// process_segment (renderer/src/tiler.rs:166-184), recursive as in the reference.
void process_segment(Ctx& ctx, const Segment& s, int depth) {
    if (s.kind == kQuad) { process_segment(ctx, to_cubic(s), depth); return; }
    if (s.kind == kLine || is_flat(s) || depth >= 32) {
        if (depth >= 32 && s.kind == kCubic && !is_flat(s)) ctx.bp->limit_hit = true;
        process_line_segment(ctx, s.base);
        return;
    }
    Segment a, b;
    split_half(s, &a, &b);
    process_segment(ctx, a, depth + 1);
    process_segment(ctx, b, depth + 1);
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
    bool limit_hit = false;
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
    Ctx ctx{fr.view_box, &bp, dda_limit};
    for (const Contour& c : in.contours)
        for_each_segment(c, [&](const Segment& s) { process_segment(ctx, s, 0); });
}

// Tiler::prepare_tiles (renderer/src/tiler.rs:93-163).
void prepare_tiles(Frame& fr, uint32_t p) {
    const PathInput& in = fr.paths[p];
    BuiltPath& bp = fr.built[p];
    const BuiltPath* clip = nullptr;
    if (!in.is_clip && in.clip_path >= 0) clip = &fr.built[(uint32_t)in.clip_path];
    int32_t w = bp.tile_rect.width();
    for (size_t i = 0; i < bp.tiles.size(); i++) {
        OTile& t = bp.tiles[i];
        size_t column = i % (size_t)w;
        int32_t delta = t.backdrop;
        uint32_t draw_alpha = t.alpha_tile_id;
        int8_t draw_backdrop = (int8_t)(uint8_t)(uint32_t)bp.backdrops[column];
        if (clip) {
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
        if (in.paint.a != 255) continue;
        const BuiltPath& bp = fr.built[fr.clip_count + d];
        bool eo = in.fill_rule == PF_FILL_RULE_EVEN_ODD;
        for (const OTile& t : bp.tiles) {
            if (t.alpha_tile_id != kInvalid) continue;
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

template <typename T>
void tile_coverage(const Frame& fr, uint32_t p, size_t i, const std::vector<T>& masks, T* out) {
    const PathInput& in = fr.paths[p];
    const BuiltPath& bp = fr.built[p];
    const OTile& t = bp.tiles[i];
    bool eo = !in.is_clip && in.fill_rule == PF_FILL_RULE_EVEN_ODD;
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

// Tile composite (shaders/d3d11/tile.cs.glsl:91-159 with calculateColor,
// shaders/tile_fragment.inc.glsl:560-613, and SrcOver, renderer/src/gpu/blend.rs:54-62):
// back to front in draw order; occluded tiles (path index < z) are skipped
// (shaders/d3d9/tile.vs.glsl:51-55).
template <typename T>
void composite(const Frame& fr, const std::vector<T>& masks, int w, int h, const T bg[4],
               std::vector<T>& fb, int channels, int threads) {
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
                for (int py = 0; py < 16; py++) {
                    int Y = t.tile_y * 16 + py;
                    if (Y < 0 || Y >= h) continue;
                    for (int px = 0; px < 16; px++) {
                        int X = t.tile_x * 16 + px;
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
    for (uint32_t p = 0; p < n; p++) {
        const PFCUDAPath& src = p < fr.clip_count ? sc->clip_paths[p] : sc->draw_paths[p - fr.clip_count];
        PathInput& in = fr.paths[p];
        in.is_clip = p < fr.clip_count;
        in.path_index = in.is_clip ? p : p - fr.clip_count;
        in.fill_rule = src.fill_rule;
        in.clip_path = in.is_clip ? -1 : src.clip_path;
        in.paint = src.paint;
        if (!in.is_clip && src.clip_path >= (int32_t)fr.clip_count) return false;
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
    return true;
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

PFOFrame* pfo_build(const PFCUDASceneDesc* scene, const PFCUDABuildOptions* opts, int threads,
                    uint64_t dda_limit) {
    PFOFrame* f = new PFOFrame();
    if (!make_frame(scene, opts, f->fr)) { delete f; return nullptr; }
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

}  // extern "C"

// pf_device.cuh — device-side records and building blocks of the CUDA level.
//
// Bit-exactness: the tiler functions below reproduce the reference CPU
// tiler's single-precision arithmetic (renderer/src/tiler.rs,
// content/src/segment.rs, content/src/clip.rs, renderer/src/builder.rs) with
// explicit round-to-nearest intrinsics, so no multiply-add is ever contracted
// (the reference runs SSE mulps/addps; simd/src/x86/mod.rs).  Their
// translation unit is also compiled with -fmad=false.
#pragma once

#include <cstdint>
#include <climits>
#include <cmath>
#include <cuda_runtime.h>

namespace pf {

// ---------------------------------------------------------------------------
// Programmatic dependent launch.  A frame kernel may be launched before its
// predecessor on the stream has finished (pdl_launch), so that its blocks
// take the multiprocessors as the predecessor's last blocks retire instead of
// after the grid boundary.  Every such kernel calls pdl_wait() before
// anything else: it returns once the predecessor grid has completed and its
// writes are visible (at once when the kernel was launched normally), and as
// no block of the kernel exits before it, the kernel cannot complete before
// its predecessor, which keeps the stream's order for whatever follows.
// pdl_trigger() lets the kernel's own successor be scheduled.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_enter() { pdl_wait(); pdl_trigger(); }

// ---------------------------------------------------------------------------
// Constants
// ---------------------------------------------------------------------------
constexpr uint32_t kInvalid = 0xffffffffu;
constexpr int kTileSize = 16;             // renderer/src/tiles.rs:19-20
constexpr int kMaxFlattenDepth = 32;      // depth bound of the subdivision walk
constexpr uint32_t kSegLine = 1, kSegQuad = 2, kSegCubic = 3;

// status bits (device word, OR-ed)
constexpr uint32_t kStatusFillCapacity   = 1u << 0;
constexpr uint32_t kStatusTileCapacity   = 1u << 1;
constexpr uint32_t kStatusVisibleCapacity= 1u << 2;
constexpr uint32_t kStatusDdaLimit       = 1u << 3;
constexpr uint32_t kStatusDepthLimit     = 1u << 4;
constexpr uint32_t kStatusMalformed      = 1u << 5;
constexpr uint32_t kStatusColumnCapacity = 1u << 6;
constexpr uint32_t kStatusAlphaCapacity  = 1u << 7;
constexpr uint32_t kStatusLineCapacity   = 1u << 8;
// A bounded wait for a bulk copy gave up (the tile was computed from global
// memory instead); reported as a launch error.
constexpr uint32_t kStatusCopyStall      = 1u << 9;
// A bounded wait of a single-pass scan gave up: the offsets it produced are
// not valid (reported as a launch error).
constexpr uint32_t kStatusScanStall      = 1u << 10;

// ---------------------------------------------------------------------------
// Records in HBM
// ---------------------------------------------------------------------------
// One input segment (the role of SegmentIndicesD3D11, renderer/src/gpu_data.rs):
// x = index of its first point, y = index of its end point (the contour start
// for the closing line), z = kind, w = global path index.
using SegRec = int4;

// Per-path data, one struct-of-arrays per field (PathDev).
struct PathDev {
    uint32_t* first_ord_contour;   // [P+1] range into the ordered contour list
    uint32_t* paint;               // [P] RGBA8 (r in the low byte)
    int32_t*  clip_gpath;          // [P] global index of the clip path, or -1
    uint8_t*  rule;                // [P] PF_FILL_RULE_*
    uint8_t*  is_clip;             // [P]
    uint32_t* local_index;         // [P] index within clip paths / draw paths
    uint32_t* scene;               // [P] scene of the path (batched frames)
    int4*     tile_rect;           // [P] tile rect (min x, min y, max x, max y)
    uint32_t* tile_offset;         // [P+1] global tile index of the path's first tile
    uint32_t* col_offset;          // [P+1] offset of its above-rect column backdrops
    // differentiable frames only (NULL otherwise): paint alpha per draw path
    const float* alpha_f;          // [draw paths of the batch]
    const uint32_t* draw_index;    // [P] index of the path among the batch's draw paths
    // paint: blend mode (PF_BLEND_MODE_*) and overlay (index + 1, 0 = none) per path
    const uint8_t*  blend;         // [P]
    const uint32_t* overlay;       // [P]
    const uint8_t*  occludes;      // [P] opaque paint with a blend mode that hides what lies below
};

// Blend modes whose paths cover the whole view box (BlendMode::is_destructive,
// content/src/effects.rs:233-262).
__host__ __device__ __forceinline__ bool blend_is_destructive(uint32_t m) {
    return m == 1u /* Clear */ || m == 2u /* Copy */ || m == 3u /* SrcIn */ || m == 4u /* SrcOut */ ||
           m == 6u /* DestIn */ || m == 9u /* DestAtop */;
}

// A paint overlay of the batch: a gradient (a ramp of 256 RGBA8 texels) or an
// image pattern (a texture page), both in `texels`.  `g` maps scene
// coordinates to the colour texture coordinate before the frame's inverse
// build transform is composed in: linear gradients, u = g0 x + g1 y + g2 (the
// projection onto the line); radial gradients, the inverse of the gradient's
// transform; patterns, page UV = scale(1 / page size) * inverse(pattern
// transform).  Filter parameters are stored rounded to binary16, as the
// reference's RGBA16F metadata texture holds them
// (renderer/src/gpu/renderer.rs:702-763).
constexpr int32_t kOverlayPattern = 2;  // after PF_GRADIENT_LINEAR / PF_GRADIENT_RADIAL
struct OverlayDev {
    int32_t kind, wrap;            // PF_GRADIENT_* or kOverlayPattern; gradient wrap
    float g[6];                    // row-major 2x3: [m11 m12 m13; m21 m22 m23]
    float from_x, from_y;          // radial: first centre
    float vec_x, vec_y;            // radial: vector between the centres
    float r0, r1;                  // radial: radii
    uint32_t texel_offset;         // first texel of the ramp or page in `texels`
    uint32_t page_w, page_h;       // page size (ramps: 256 x 1)
    uint32_t flags;                // patterns: PF_PATTERN_* bits
    int32_t filter;                // patterns: PF_PATTERN_FILTER_*
    float blur[6];                 // blur: source offset (x, y), support, Gaussian coefficients (x, y, z)
    float matrix[20];              // colour matrix columns
};

// Round a float to the nearest binary16 value (ties to even), kept as float;
// overflow gives infinity.  Used for the metadata the reference stores as f16.
__host__ __device__ inline float round_f16(float x) {
    if (!(x == x)) return x;
    const float ax = fabsf(x);
    if (ax >= 65520.0f) return x > 0.0f ? INFINITY : -INFINITY;
    if (ax < 6.103515625e-05f) {  // below 2^-14: fixed quantum 2^-24
        const float q = 5.9604644775390625e-08f;
        return nearbyintf(x / q) * q;
    }
    int e;
    frexpf(ax, &e);                          // ax = m * 2^e, m in [0.5, 1)
    const float q = ldexpf(1.0f, e - 11);    // 11 significant bits
    return nearbyintf(x / q) * q;
}

// Per-scene data.
struct SceneDev {
    float4 view_box;               // min x, min y, max x, max y
    int4   screen;                 // screen tile rect = round_out(view_box / 16)
    uint32_t screen_offset;        // first global screen tile
    uint32_t first_path;           // global index of the first path
    uint32_t clip_count, draw_count;
    // output placement: scene pixel (x, y) inside `clip` goes to element
    // out_offset + (y - origin_y) * pitch + (x - origin_x)
    int4   clip;                   // x0, y0, x1, y1 (exclusive)
    int32_t origin_x, origin_y;
    int32_t pitch;
    int32_t pad;
    uint64_t out_offset;
};

// Device counters written by the pipeline (one struct, zeroed per frame).
struct Counters {
    uint32_t status;
    uint32_t pad0;
    uint64_t tiles;        // T
    uint64_t columns;      // sum of tile rect widths
    uint64_t fills;        // F
    uint64_t alpha_tiles;  // A
    uint64_t lines;        // flattened lines (one-pass flattening: those within one tile)
    uint64_t lines_back;   // one-pass flattening: lines beyond one tile, at the line array's end
    uint64_t visible;      // composited tiles
    uint64_t needed_fills, needed_tiles, needed_visible, needed_lines;
    uint32_t composite_next;   // work counter of the persistent composite (screen tiles handed out)
    uint32_t mask_items;       // visible tiles with a mask (k_mask's work list)
    uint64_t mask_fills;       // fills of those tiles
};

// ---------------------------------------------------------------------------
// Exact single-precision helpers (SSE lane semantics, simd/src/x86/mod.rs)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
// _mm_min_ps / _mm_max_ps: the second operand wins when either is NaN.
__device__ __forceinline__ float smin(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float smax(float a, float b) { return a > b ? a : b; }
// _mm_cvtps_epi32: nearest even, 0x80000000 out of range or NaN.
__device__ __forceinline__ int32_t cvt_rne(float x) {
    if (!(x >= -2147483648.0f && x < 2147483648.0f)) return INT_MIN;
    return __float2int_rn(x);
}
__device__ __forceinline__ float i2f(int32_t v) { return __int2float_rn(v); }

struct Line { float fx, fy, tx, ty; };
struct Cubic { Line base; Line ctrl; };

// Segment::to_cubic (content/src/segment.rs:171-182).
__device__ __forceinline__ Cubic quad_to_cubic(float p0x, float p0y, float cx, float cy, float p3x, float p3y) {
    const float third = 1.0f / 3.0f;
    float p12x = fadd(cx, cx), p12y = fadd(cy, cy);
    Cubic c;
    c.base = Line{p0x, p0y, p3x, p3y};
    c.ctrl = Line{fmul(fadd(p0x, p12x), third), fmul(fadd(p0y, p12y), third),
                  fmul(fadd(p12x, p3x), third), fmul(fadd(p12y, p3y), third)};
    return c;
}

// CubicSegment::is_flat(0.25) (content/src/segment.rs:292-300).
__device__ __forceinline__ bool cubic_is_flat(const Cubic& s) {
    float u0 = fmul(3.0f, s.ctrl.fx), u1 = fmul(3.0f, s.ctrl.fy);
    float u2 = fmul(3.0f, s.ctrl.tx), u3 = fmul(3.0f, s.ctrl.ty);
    u0 = fsub(fsub(fsub(u0, s.base.fx), s.base.fx), s.base.tx);
    u1 = fsub(fsub(fsub(u1, s.base.fy), s.base.fy), s.base.ty);
    u2 = fsub(fsub(fsub(u2, s.base.tx), s.base.tx), s.base.fx);
    u3 = fsub(fsub(fsub(u3, s.base.ty), s.base.ty), s.base.fy);
    u0 = fmul(u0, u0); u1 = fmul(u1, u1); u2 = fmul(u2, u2); u3 = fmul(u3, u3);
    return fadd(smax(u0, u2), smax(u1, u3)) <= 1.0f;  // 16 * 0.25 * 0.25
}

// CubicSegment::split at t = 0.5 (content/src/segment.rs:307-359).
__device__ __forceinline__ void cubic_split_half(const Cubic& s, Cubic& a, Cubic& b) {
    const float t = 0.5f;
    float p0x = s.base.fx, p0y = s.base.fy, p3x = s.base.tx, p3y = s.base.ty;
    float p1x = s.ctrl.fx, p1y = s.ctrl.fy, p2x = s.ctrl.tx, p2y = s.ctrl.ty;
    float p01x = fadd(p0x, fmul(t, fsub(p1x, p0x))), p01y = fadd(p0y, fmul(t, fsub(p1y, p0y)));
    float p12x = fadd(p1x, fmul(t, fsub(p2x, p1x))), p12y = fadd(p1y, fmul(t, fsub(p2y, p1y)));
    float p23x = fadd(p2x, fmul(t, fsub(p3x, p2x))), p23y = fadd(p2y, fmul(t, fsub(p3y, p2y)));
    float p012x = fadd(p01x, fmul(t, fsub(p12x, p01x))), p012y = fadd(p01y, fmul(t, fsub(p12y, p01y)));
    float p123x = fadd(p12x, fmul(t, fsub(p23x, p12x))), p123y = fadd(p12y, fmul(t, fsub(p23y, p12y)));
    float mx = fadd(p012x, fmul(t, fsub(p123x, p012x))), my = fadd(p012y, fmul(t, fsub(p123y, p012y)));
    a.base = Line{p0x, p0y, mx, my};  a.ctrl = Line{p01x, p01y, p012x, p012y};
    b.base = Line{mx, my, p3x, p3y};  b.ctrl = Line{p123x, p123y, p23x, p23y};
}

// Per-path context for the DDA.
// A path's binning context, one 48-byte record per path written once per
// frame, so a line's path costs one dependent read of three 16-byte words.
struct __align__(16) PathCtx {
    int32_t minx, miny, maxx, maxy;  // tile rect
    uint32_t tile_base;              // global tile index of (minx, miny)
    uint32_t col_base;               // first above-rect column backdrop
    float vminx, vmaxx, vmaxy;       // clip box x range and max y (view box)
    uint32_t pad[3];
};

__device__ __forceinline__ uint32_t outcode(float x, float y, float minx, float maxx, float maxy) {
    uint32_t o = 0;
    if (x < minx) o |= 1u;
    // y < -inf never holds (TOP)
    if (x > maxx) o |= 2u;
    if (y > maxy) o |= 8u;
    return o;
}
__device__ __forceinline__ float lerpf(float a, float b, float t) { return fadd(a, fmul(fsub(b, a), t)); }

// clip_line_segment_to_rect (content/src/clip.rs:494-560) against
// (view min x, -inf) .. (view max x, view max y) (renderer/src/tiler.rs:194-200).
__device__ __forceinline__ bool clip_to_view(Line& s, float minx, float maxx, float maxy) {
    uint32_t of = outcode(s.fx, s.fy, minx, maxx, maxy), ot = outcode(s.tx, s.ty, minx, maxx, maxy);
    for (int it = 0; it < 8; it++) {
        if ((of | ot) == 0) return true;
        if ((of & ot) != 0) return false;
        bool clip_from = of > ot;
        uint32_t oc = clip_from ? of : ot;
        float px = clip_from ? s.fx : s.tx, py = clip_from ? s.fy : s.ty;
        if (oc & 1u) {
            px = minx; py = lerpf(s.fy, s.ty, fdiv(fsub(minx, s.fx), fsub(s.tx, s.fx)));
        } else if (oc & 2u) {
            px = maxx; py = lerpf(s.fy, s.ty, fdiv(fsub(maxx, s.fx), fsub(s.tx, s.fx)));
        } else if (oc & 8u) {
            px = lerpf(s.fx, s.tx, fdiv(fsub(maxy, s.fy), fsub(s.ty, s.fy))); py = maxy;
        }
        if (clip_from) { s.fx = px; s.fy = py; of = outcode(px, py, minx, maxx, maxy); }
        else { s.tx = px; s.ty = py; ot = outcode(px, py, minx, maxx, maxy); }
    }
    return false;
}

// The differentiable form keeps each fill's FP32 tile-local endpoints (the
// 8.8 rounding would make coverage piecewise constant in the control points)
// and culls only fills of exactly zero width.
__device__ __forceinline__ bool make_fill_f(const PathCtx& pc, Line s, int32_t tx, int32_t ty, float4& rec,
                                            uint32_t& g) {
    if (!(pc.minx <= tx && pc.miny <= ty && tx <= pc.maxx - 1 && ty <= pc.maxy - 1)) return false;
    const float ulx = (float)tx * 16.0f, uly = (float)ty * 16.0f;
    rec = make_float4(fminf(fmaxf(s.fx - ulx, 0.0f), 16.0f), fminf(fmaxf(s.fy - uly, 0.0f), 16.0f),
                      fminf(fmaxf(s.tx - ulx, 0.0f), 16.0f), fminf(fmaxf(s.ty - uly, 0.0f), 16.0f));
    if (!(fabsf(rec.x - rec.z) >= 1e-7f)) return false;  // width below 1e-7 px: area below 2e-6 px^2
    g = pc.tile_base + (uint32_t)(tx - pc.minx) + (uint32_t)(pc.maxx - pc.minx) * (uint32_t)(ty - pc.miny);
    return true;
}

// ObjectBuilder::add_fill (renderer/src/builder.rs:509-553) without the push:
// returns false when the fill is culled, else the packed LineSegmentU16 and the
// global tile index.
__device__ __forceinline__ bool make_fill(const PathCtx& pc, Line s, int32_t tx, int32_t ty,
                                          uint2& rec, uint32_t& g) {
    if (!(pc.minx <= tx && pc.miny <= ty && tx <= pc.maxx - 1 && ty <= pc.maxy - 1)) return false;
    float ulx = fmul(i2f(tx), 16.0f), uly = fmul(i2f(ty), 16.0f);
    const float hi = 4095.0f;
    int32_t i0 = cvt_rne(smin(smax(fmul(fsub(s.fx, ulx), 256.0f), 0.0f), hi));
    int32_t i1 = cvt_rne(smin(smax(fmul(fsub(s.fy, uly), 256.0f), 0.0f), hi));
    int32_t i2 = cvt_rne(smin(smax(fmul(fsub(s.tx, ulx), 256.0f), 0.0f), hi));
    int32_t i3 = cvt_rne(smin(smax(fmul(fsub(s.ty, uly), 256.0f), 0.0f), hi));
    if (i0 == i2) return false;
    rec.x = (uint32_t)i0 | ((uint32_t)i1 << 16);
    rec.y = (uint32_t)i2 | ((uint32_t)i3 << 16);
    g = pc.tile_base + (uint32_t)(tx - pc.minx) + (uint32_t)(pc.maxx - pc.minx) * (uint32_t)(ty - pc.miny);
    return true;
}

// addFill of the D3D11 level (shaders/d3d11/bin.cs.glsl:100-125): tile-rect
// cull, 8.8 conversion by truncation (no clamp to 4095; a negative value,
// undefined in GLSL, converts to 0), cull when from.x == to.x.
__device__ __forceinline__ bool make_fill_d3d11(const PathCtx& pc, Line s, int32_t tx, int32_t ty, uint2& rec,
                                                uint32_t& g) {
    if (!(pc.minx <= tx && pc.miny <= ty && tx <= pc.maxx - 1 && ty <= pc.maxy - 1)) return false;
    const float ulx = fmul(i2f(tx), 16.0f), uly = fmul(i2f(ty), 16.0f);
    auto q = [](float v) { return (uint32_t)fminf(fmaxf(v, 0.0f), 65535.0f); };  // truncates
    const uint32_t i0 = q(fmul(fsub(s.fx, ulx), 256.0f)), i1 = q(fmul(fsub(s.fy, uly), 256.0f));
    const uint32_t i2 = q(fmul(fsub(s.tx, ulx), 256.0f)), i3 = q(fmul(fsub(s.ty, uly), 256.0f));
    if (i0 == i2) return false;
    rec.x = i0 | (i1 << 16);
    rec.y = i2 | (i3 << 16);
    g = pc.tile_base + (uint32_t)(tx - pc.minx) + (uint32_t)(pc.maxx - pc.minx) * (uint32_t)(ty - pc.miny);
    return true;
}

// Fill conversions of the binning pass.
enum FillMode : int {
    kFillCpu = 0,    // the CPU tiler: view-box clip, 8.8 round-to-nearest-even clamped to 4095
    kFillF32 = 1,    // differentiable frames: FP32 tile-local endpoints
    kFillD3D11 = 2,  // the D3D11 level: no view-box clip, truncating 8.8 conversion
};

// process_line_segment (renderer/src/tiler.rs:191-308).  `sink` receives
// sink.fill(rec, g) for every kept fill in emission order and
// sink.backdrop(tx, ty, delta) for every backdrop adjustment.  kFillF32
// fills reach sink.fill as float4, the others as packed LineSegmentU16.
// ONE_TILE: a line within one tile takes a short path without the walk's
// divisions (the count pass gains from it; in the emit pass the two paths'
// divergence costs more than the divisions).
template <int MODE = kFillCpu, bool ONE_TILE = false, class Sink>
__device__ __forceinline__ void dda_line(const PathCtx& pc, Line seg, Sink& sink, uint32_t dda_limit,
                                         uint32_t* status) {
    if (MODE != kFillD3D11 && !clip_to_view(seg, pc.vminx, pc.vmaxx, pc.vmaxy)) return;
    const float r = 1.0f / 16.0f;
    int32_t ftx = cvt_rne(floorf(fmul(seg.fx, r))), fty = cvt_rne(floorf(fmul(seg.fy, r)));
    int32_t ttx = cvt_rne(floorf(fmul(seg.tx, r))), tty = cvt_rne(floorf(fmul(seg.ty, r)));
    float vx = fsub(seg.tx, seg.fx), vy = fsub(seg.ty, seg.fy);
    if (ONE_TILE && ftx == ttx && fty == tty && dda_limit > 0) {
        // One tile: the walk's single step.  Its next_t is min(t_max, 1) = 1
        // (the line ends before the next tile boundary in x and in y, so both
        // t_max are at least 1), it stops there (dir 0) with no y piece and no
        // backdrop: one fill from the start to start + v.
        const Line l{seg.fx, seg.fy, fadd(seg.fx, fmul(vx, 1.0f)), fadd(seg.fy, fmul(vy, 1.0f))};
        uint32_t g;
        if constexpr (MODE == kFillF32) {
            float4 rec;
            if (make_fill_f(pc, l, ftx, fty, rec, g)) sink.fill(rec, g);
        } else if constexpr (MODE == kFillD3D11) {
            uint2 rec;
            if (make_fill_d3d11(pc, l, ftx, fty, rec, g)) sink.fill(rec, g);
        } else {
            uint2 rec;
            if (make_fill(pc, l, ftx, fty, rec, g)) sink.fill(rec, g);
        }
        return;
    }
    bool negx = vx < 0.0f, negy = vy < 0.0f;
    int32_t stepx = negx ? -1 : 1, stepy = negy ? -1 : 1;
    float fcx = fmul(i2f(ftx + (negx ? 0 : 1)), 16.0f), fcy = fmul(i2f(fty + (negy ? 0 : 1)), 16.0f);
    float tmx = fdiv(fsub(fcx, seg.fx), vx), tmy = fdiv(fsub(fcy, seg.fy), vy);
    float tdx = fabsf(fdiv(16.0f, vx)), tdy = fabsf(fdiv(16.0f, vy));
    float cx = seg.fx, cy = seg.fy;
    int32_t tcx = ftx, tcy = fty;
    int last = 0;  // 0 none, 1 X, 2 Y
    for (uint32_t it = 0;; it++) {
        if (it >= dda_limit) { atomicOr(status, kStatusDdaLimit); return; }
        int dir;
        if (tmx < tmy) dir = 1;
        else if (tmx > tmy) dir = 2;
        else dir = stepx > 0 ? 1 : 2;
        float next_t = fminf(dir == 1 ? tmx : tmy, 1.0f);
        if (tcx == ttx && tcy == tty) dir = 0;
        float npx = fadd(seg.fx, fmul(vx, next_t)), npy = fadd(seg.fy, fmul(vy, next_t));
        auto add = [&](Line l) {
            uint32_t g;
            if constexpr (MODE == kFillF32) {
                float4 rec;
                if (make_fill_f(pc, l, tcx, tcy, rec, g)) sink.fill(rec, g);
            } else if constexpr (MODE == kFillD3D11) {
                uint2 rec;
                if (make_fill_d3d11(pc, l, tcx, tcy, rec, g)) sink.fill(rec, g);
            } else {
                uint2 rec;
                if (make_fill(pc, l, tcx, tcy, rec, g)) sink.fill(rec, g);
            }
        };
        add(Line{cx, cy, npx, npy});
        if (stepy < 0 && dir == 2) add(Line{npx, npy, fmul(i2f(tcx), 16.0f), fmul(i2f(tcy), 16.0f)});
        else if (stepy > 0 && last == 2) add(Line{fmul(i2f(tcx), 16.0f), fmul(i2f(tcy), 16.0f), cx, cy});
        if (stepx < 0 && last == 1) sink.backdrop(tcx, tcy, 1);
        else if (stepx > 0 && dir == 1) sink.backdrop(tcx, tcy, -1);
        if (dir == 0) break;
        if (dir == 1) {
            if (tcx == ttx) break;
            tmx = fadd(tmx, tdx); tmy = fadd(tmy, 0.0f);
            tcx += stepx;
        } else {
            if (tcy == tty) break;
            tmx = fadd(tmx, 0.0f); tmy = fadd(tmy, tdy);
            tcy += stepy;
        }
        cx = npx; cy = npy;
        last = dir;
    }
}

// process_segment (renderer/src/tiler.rs:166-184) without recursion: calls
// emit(Line, addr, depth) for every flattened line in the same depth-first
// order as the reference's recursion.
// A segment with a non-finite coordinate gives no lines and flags the frame
// malformed (the reference's recursion would not end on it); a segment gives
// at most kMaxSegmentLines lines (depth first), then flags the depth limit, so
// huge coordinates cannot make the walk exponential.
constexpr uint32_t kMaxSegmentLines = 1u << 20;
__host__ __device__ __forceinline__ bool finite2(float2 p) { return isfinite(p.x) && isfinite(p.y); }

// The root of a segment's subdivision: a curve as a cubic (a quadratic
// elevated by Segment::to_cubic), a line as its base.  Returns 0 for a segment
// with a non-finite point (flagged malformed), 1 for a line, 2 for a curve.
enum : int { kRootInvalid = 0, kRootLine = 1, kRootCurve = 2 };
__device__ __forceinline__ int segment_root(const float2* pts, SegRec sr, Cubic& c, uint32_t* status) {
    const float2 p0 = pts[sr.x], pe = pts[sr.y];
    if (!finite2(p0) || !finite2(pe)) { atomicOr(status, kStatusMalformed); return kRootInvalid; }
    c.base = Line{p0.x, p0.y, pe.x, pe.y};
    c.ctrl = c.base;
    if (sr.z == (int)kSegLine) return kRootLine;
    if (sr.z == (int)kSegQuad) {
        const float2 q = pts[sr.x + 1];
        if (!finite2(q)) { atomicOr(status, kStatusMalformed); return kRootInvalid; }
        c = quad_to_cubic(p0.x, p0.y, q.x, q.y, pe.x, pe.y);
    } else {
        const float2 c0 = pts[sr.x + 1], c1 = pts[sr.x + 2];
        if (!finite2(c0) || !finite2(c1)) { atomicOr(status, kStatusMalformed); return kRootInvalid; }
        c.ctrl = Line{c0.x, c0.y, c1.x, c1.y};
    }
    return kRootCurve;
}

// The node of a subdivision at split path `addr` (d bits, first split most
// significant) of the root: exactly the splits the recursion performs.
__device__ __forceinline__ Cubic subdivision_node(Cubic c, uint32_t addr, int d) {
    for (int i = d - 1; i >= 0; i--) {
        Cubic a, b;
        cubic_split_half(c, a, b);
        c = ((addr >> i) & 1u) ? b : a;
    }
    return c;
}

template <class Emit>
__device__ __forceinline__ void flatten_segment(const float2* pts, SegRec sr, Emit&& emit, uint32_t* status) {
    Cubic c;
    const int kind = segment_root(pts, sr, c, status);
    if (kind == kRootInvalid) return;
    if (kind == kRootLine) {
        emit(c.base, 0u, 0);
        return;
    }
    uint32_t emitted = 0;
    // Depth-first without a stack: the current node is named by its split
    // path `addr` (d bits, first split most significant; the leaf covers
    // [addr, addr + 1) / 2^d of the curve parameter).  Descending left splits
    // the current node; moving to a right sibling recomputes it from the root
    // along its path, i.e. with exactly the splits the recursion performs, so
    // every node, flatness decision and line is bit-identical to it.
    const Cubic root = c;
    uint32_t addr = 0;
    int d = 0;
    for (;;) {
        const bool flat = cubic_is_flat(c);
        if (!flat && d < kMaxFlattenDepth) {
            Cubic a, b;
            cubic_split_half(c, a, b);
            c = a;
            addr <<= 1;
            d++;
            continue;
        }
        if (!flat) atomicOr(status, kStatusDepthLimit);
        emit(c.base, addr, d);
        if (++emitted >= kMaxSegmentLines) { atomicOr(status, kStatusDepthLimit); break; }
        while (d > 0 && (addr & 1u)) { addr >>= 1; d--; }  // climb past right children
        if (d == 0) break;
        addr |= 1u;  // the right sibling
        c = subdivision_node(root, addr, d);
    }
}

// ---------------------------------------------------------------------------
// Uniform dicing of the D3D11 level (shaders/d3d11/dice.cs.glsl:133-217):
// a curve is cut into n pieces of equal parameter length, n from Sederberg's
// error bound for tolerance 0.25; a line into n pieces of at most 16 px; the
// piece ends are rounded to 1/256 px (the packed microline, :83-97).  The FP32
// op order here is this level's own definition (the oracle repeats it).
// ---------------------------------------------------------------------------
constexpr float kDiceTolerance = 0.25f, kMicrolineLength = 16.0f;
constexpr uint32_t kMaxDicePieces = 1u << 16;

struct DiceSeg { float2 p0, c0, c1, p3; bool curve; };
__device__ __forceinline__ bool dice_finite(const DiceSeg& d) {
    return finite2(d.p0) && finite2(d.c0) && finite2(d.c1) && finite2(d.p3);
}

__device__ __forceinline__ DiceSeg dice_seg(const float2* pts, SegRec sr) {
    DiceSeg d;
    d.p0 = pts[sr.x];
    d.p3 = pts[sr.y];
    d.curve = sr.z != (int)kSegLine;
    d.c0 = d.p0; d.c1 = d.p3;
    if (sr.z == (int)kSegQuad) {
        const float2 q = pts[sr.x + 1];
        const float third = 1.0f / 3.0f;
        const float qx2 = fadd(q.x, q.x), qy2 = fadd(q.y, q.y);
        d.c0 = make_float2(fmul(fadd(d.p0.x, qx2), third), fmul(fadd(d.p0.y, qy2), third));
        d.c1 = make_float2(fmul(fadd(d.p3.x, qx2), third), fmul(fadd(d.p3.y, qy2), third));
    } else if (sr.z == (int)kSegCubic) {
        d.c0 = pts[sr.x + 1];
        d.c1 = pts[sr.x + 2];
    }
    return d;
}

// Pieces of one segment (1 .. kMaxDicePieces; *limited when capped or not finite).
__device__ __forceinline__ uint32_t dice_count(const DiceSeg& d, bool* limited) {
    float n;
    if (d.curve) {
        auto dd = [](float a, float b, float c) { return fabsf(fadd(fsub(c, fmul(2.0f, b)), a)); };
        const float bx = fmul(6.0f, fmaxf(dd(d.p0.x, d.c0.x, d.c1.x), dd(d.c0.x, d.c1.x, d.p3.x)));
        const float by = fmul(6.0f, fmaxf(dd(d.p0.y, d.c0.y, d.c1.y), dd(d.c0.y, d.c1.y, d.p3.y)));
        const float len = __fsqrt_rn(fadd(fmul(bx, bx), fmul(by, by)));
        n = __fsqrt_rn(fdiv(len, 8.0f * kDiceTolerance));
    } else {
        const float dx = fsub(d.p3.x, d.p0.x), dy = fsub(d.p3.y, d.p0.y);
        n = fdiv(__fsqrt_rn(fadd(fmul(dx, dx), fmul(dy, dy))), kMicrolineLength);
    }
    if (!(n <= (float)kMaxDicePieces)) {  // too many pieces, or not finite
        *limited = true;
        return n > (float)kMaxDicePieces ? kMaxDicePieces : 1u;
    }
    const uint32_t k = (uint32_t)ceilf(n);
    return k > 1u ? k : 1u;
}

__device__ __forceinline__ float dice_lerp(float a, float b, float t) { return fadd(a, fmul(fsub(b, a), t)); }
__device__ __forceinline__ float dice_q(float v) {  // round to 1/256 px (microline packing)
    return fmul(rintf(fmul(fminf(fmaxf(v, -32768.0f), 32767.0f), 256.0f)), 1.0f / 256.0f);
}

// Point of piece end k (1 .. n) of the segment, rounded to 1/256 px.
__device__ __forceinline__ float2 dice_point(const DiceSeg& d, uint32_t k, uint32_t n) {
    const float t = fdiv((float)k, (float)n);
    float x, y;
    if (d.curve) {
        const float ax = dice_lerp(d.p0.x, d.c0.x, t), ay = dice_lerp(d.p0.y, d.c0.y, t);
        const float bx = dice_lerp(d.c0.x, d.c1.x, t), by = dice_lerp(d.c0.y, d.c1.y, t);
        const float cx = dice_lerp(d.c1.x, d.p3.x, t), cy = dice_lerp(d.c1.y, d.p3.y, t);
        const float abx = dice_lerp(ax, bx, t), aby = dice_lerp(ay, by, t);
        const float bcx = dice_lerp(bx, cx, t), bcy = dice_lerp(by, cy, t);
        x = dice_lerp(abx, bcx, t);
        y = dice_lerp(aby, bcy, t);
    } else {
        x = dice_lerp(d.p0.x, d.p3.x, t);
        y = dice_lerp(d.p0.y, d.p3.y, t);
    }
    return make_float2(dice_q(x), dice_q(y));
}

// ---------------------------------------------------------------------------
// Coverage: exact signed area below each fill inside each pixel.
//
// The reference evaluates, per fill and per pixel, dX * area(y, -|d dX|)
// (shaders/fill_area.inc.glsl:11-27 with utils/area-lut/src/main.rs:29-65):
// the area of the pixel lying below the fill inside the fill's x-window,
// signed by direction.  The same quantity is accumulated here cell by cell:
// the fill is cut at pixel columns and rows; each piece adds its trapezoid
// area to its own cell and its x-extent to every cell below it in the column
// (a carry resolved by a prefix down the column).  Sums are kept in 2^-22
// fixed point so the result does not depend on summation order.
// ---------------------------------------------------------------------------
constexpr float kCovScale = 4194304.0f;      // 2^22
constexpr float kCovInvScale = 1.0f / 4194304.0f;

// Accumulate the part of a fill (x0,y0)->(x1,y1) (tile pixels, x0 != x1,
// slope = dy/dx) that lies in pixel column px into acc[row][col] and
// carry[row][col].  The row split uses the fast division: its relative error
// (~2^-22) is at the level of the fixed-point accumulation.
__device__ __forceinline__ void accumulate_fill_column(float x0, float y0, float x1, float slope, int px, int* acc,
                                                       int* carry) {
    const float lo = (float)px, hi = (float)(px + 1);
    const float xa = fminf(fmaxf(x0, lo), hi), xb = fminf(fmaxf(x1, lo), hi);
    const float w = xa - xb;  // oriented x-extent (window.x - window.y)
    if (w == 0.0f) return;
    const float ya = y0 + (xa - x0) * slope, yb = y0 + (xb - x0) * slope;
    float ylo = fminf(ya, yb), yhi = fmaxf(ya, yb);
    ylo = fminf(fmaxf(ylo, 0.0f), 16.0f);
    yhi = fminf(fmaxf(yhi, 0.0f), 16.0f);
    if (!(yhi - ylo > 1e-6f)) {  // flat piece (and no division by a vanishing height)
        const int r = (int)floorf(ylo);
        if (r > 15) return;
        atomicAdd(&acc[r * 16 + px], __float2int_rn(w * ((float)(r + 1) - ylo) * kCovScale));
        if (r + 1 < 16) atomicAdd(&carry[(r + 1) * 16 + px], __float2int_rn(w * kCovScale));
        return;
    }
    // Row r of the piece gets the trapezoid below the piece in its own cell
    // plus the x-extent of the part of the piece above the row,
    // w (max(ylo, r) - ylo) / (yhi - ylo); the rows below the piece get its
    // whole extent w through the column carry.  One atomic per row.
    const float ws = w * __fdividef(1.0f, yhi - ylo);  // extent per unit of height
    const int r0 = (int)floorf(ylo), r1 = min((int)floorf(yhi), 15);
    for (int r = r0; r <= r1; r++) {
        const float yt = fmaxf(ylo, (float)r), yb2 = fminf(yhi, (float)(r + 1));
        const float h = fmaxf(yb2 - yt, 0.0f);
        const float a = ws * (h * ((float)(r + 1) - 0.5f * (yt + yb2)) + (yt - ylo));
        atomicAdd(&acc[r * 16 + px], __float2int_rn(a * kCovScale));
    }
    if (r1 + 1 < 16) atomicAdd(&carry[(r1 + 1) * 16 + px], __float2int_rn(w * kCovScale));
}

// sampleMask resolve (shaders/tile_fragment.inc.glsl:539-556).
__device__ __forceinline__ float resolve_coverage(float c, bool even_odd) {
    if (!even_odd) c = fabsf(c);
    else {
        float m = c - 2.0f * floorf(c * 0.5f);
        c = 1.0f - fabsf(1.0f - m);
    }
    return fminf(1.0f, c);
}

// resolve_coverage and its derivative d(coverage)/dc, one-sided at the kinks:
// nonzero d|c|/dc = +1 at c = 0 and 0 once clamped at |c| >= 1; even-odd +1
// on the rising half of the period (m < 1), -1 on the falling half.
__device__ __forceinline__ float resolve_coverage_d(float c, bool even_odd, float* dc) {
    if (!even_odd) {
        const float a = fabsf(c);
        *dc = a < 1.0f ? (c >= 0.0f ? 1.0f : -1.0f) : 0.0f;
        return fminf(1.0f, a);
    }
    const float m = c - 2.0f * floorf(c * 0.5f);
    *dc = m < 1.0f ? 1.0f : -1.0f;
    return fminf(1.0f, 1.0f - fabsf(1.0f - m));
}

}  // namespace pf

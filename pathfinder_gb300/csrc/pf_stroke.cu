// pf_stroke.cu — stroke to fill on the GPU: OutlineStrokeToFill
// (content/src/stroke.rs:24-465) for a batch of outlines.
//
// The reference strokes one contour at a time: each segment is offset by
// half the line width, split at t = 1/2 until the offset is within 0.01 of
// the true offset at 17 samples, with the stroke's join pushed before every
// offset piece after the first segment, then caps (open contours) or a
// closing join (closed contours).  Here the work is split so every stage is
// data parallel and the output is the reference's, point for point:
//   1. a thread per contour cuts it into segments (ContourIter,
//      content/src/outline.rs:1020-1065);
//   2. a thread per (contour, pass, segment) walks its segment's offset
//      recursion depth first and counts its points: pieces exactly, the join
//      before each piece after the first exactly, a closing join exactly, a
//      cap as an upper bound (16); it records the recursion's leaves and its
//      first and last pieces' points, and the join before each first piece
//      is counted from those records (the previous item's last piece);
//   3. the same threads write their points at the scanned offsets,
//      recomputing only the recorded leaves;
//   4. a thread per open contour writes its caps, which look back through
//      the points written so far (add_cap's search for a distinct point);
//   5. the points are compacted over the unused cap slots (a warp per 32
//      items, whose output is one contiguous range).
// The unit is compiled with -fmad=false: single-precision ops round as the
// reference's SSE lanes do, so the points are bit-identical to the
// reference's op order (IEEE division and square root).
#include "pf_kernels.cuh"
#include "pathfinder_cuda.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace pf {

namespace {

struct V { float x, y; };
__device__ __forceinline__ V vadd(V a, V b) { return V{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ V vsub(V a, V b) { return V{a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ V vmul(V a, float s) { return V{a.x * s, a.y * s}; }
__device__ __forceinline__ V vmulv(V a, V b) { return V{a.x * b.x, a.y * b.y}; }
__device__ __forceinline__ bool veq(V a, V b) { return a.x == b.x && a.y == b.y; }
__device__ __forceinline__ float vsqlen(V v) { return v.x * v.x + v.y * v.y; }
__device__ __forceinline__ V vyx(V v) { return V{v.y, v.x}; }
// Vector2F::normalize: v * (1 / |v|) (geometry/src/vector.rs:118-126)
__device__ __forceinline__ V vnormalize(V v) { const float r = 1.0f / sqrtf(vsqlen(v)); return vmul(v, r); }
__device__ __forceinline__ V vlerp(V a, V b, float t) { return vadd(a, vmul(vsub(b, a), t)); }
__device__ __forceinline__ float lane_max(float a, float b) { return a > b ? a : b; }  // _mm_max_ps

struct L { V f, t; };
__device__ __forceinline__ V lvec(L l) { return vsub(l.t, l.f); }
__device__ __forceinline__ V lsample(L l, float t) { return vadd(l.f, vmul(lvec(l), t)); }

// LineSegment2F::offset (geometry/src/line_segment.rs:241-247)
__device__ L loffset(L l, float d) {
    const V v = lvec(l);
    if (v.x == 0.0f && v.y == 0.0f) return l;
    const V o = vmulv(vnormalize(vyx(v)), V{-d, d});
    return L{vadd(l.f, o), vadd(l.t, o)};
}

// LineSegment2F::intersection_t (:219-228): the y of inverse(M) * (from - other.from)
__device__ bool intersection_t(L self, L other, float* t) {
    const V p0p1 = lvec(self), ov = lvec(other);
    const float m11 = ov.x, m21 = ov.y, m12 = -p0p1.x, m22 = -p0p1.y;
    const float det = m11 * m22 - m12 * m21;
    if (fabsf(det) < 0.0001f) return false;
    const float r = 1.0f / det;
    const float i21 = r * -m21, i22 = r * m11;
    const V v = vsub(self.f, other.f);
    *t = i21 * v.x + i22 * v.y;
    return true;
}

enum : int { kKindLine = 1, kKindQuad = 2, kKindCubic = 3 };
struct Seg { L base, ctrl; int kind; };
__device__ __forceinline__ Seg mk_line(L l) { return Seg{l, L{{0.0f, 0.0f}, {0.0f, 0.0f}}, kKindLine}; }
__device__ __forceinline__ Seg mk_quad(L b, V c) { return Seg{b, L{c, {0.0f, 0.0f}}, kKindQuad}; }
__device__ __forceinline__ Seg mk_cubic(L b, L c) { return Seg{b, c, kKindCubic}; }

// Segment::to_cubic (content/src/segment.rs:171-182)
__device__ Seg to_cubic(const Seg& s) {
    if (s.kind == kKindCubic) return s;
    Seg c = s;
    const V p12 = vadd(s.ctrl.f, s.ctrl.f);
    const float third = 1.0f / 3.0f;
    c.ctrl = L{vmul(vadd(s.base.f, p12), third), vmul(vadd(p12, s.base.t), third)};
    c.kind = kKindCubic;
    return c;
}

// CubicSegment::split (:307-359)
__device__ void cubic_split(const Seg& s, float t, Seg* a, Seg* b) {
    if (t <= 0.0f) {
        *a = mk_cubic(L{s.base.f, s.base.f}, L{s.base.f, s.base.f});
        *b = mk_cubic(s.base, s.ctrl);
        return;
    }
    if (t >= 1.0f) {
        *a = mk_cubic(s.base, s.ctrl);
        *b = mk_cubic(L{s.base.t, s.base.t}, L{s.base.t, s.base.t});
        return;
    }
    const V p0 = s.base.f, p3 = s.base.t, p1 = s.ctrl.f, p2 = s.ctrl.t;
    const V p01 = vadd(p0, vmul(vsub(p1, p0), t)), p12 = vadd(p1, vmul(vsub(p2, p1), t));
    const V p23 = vadd(p2, vmul(vsub(p3, p2), t));
    const V p012 = vadd(p01, vmul(vsub(p12, p01), t)), p123 = vadd(p12, vmul(vsub(p23, p12), t));
    const V p0123 = vadd(p012, vmul(vsub(p123, p012), t));
    *a = mk_cubic(L{p0, p0123}, L{p01, p012});
    *b = mk_cubic(L{p0123, p3}, L{p123, p23});
}

// Segment::split at t (:211-219): lines as lines, curves as cubics
__device__ void seg_split(const Seg& s, float t, Seg* a, Seg* b) {
    if (s.kind == kKindLine) {
        const V mid = vadd(s.base.f, vmul(lvec(s.base), t));
        *a = mk_line(L{s.base.f, mid});
        *b = mk_line(L{mid, s.base.t});
        return;
    }
    cubic_split(to_cubic(s), t, a, b);
}

// Segment::sample (:226-233)
__device__ V seg_sample(const Seg& s, float t) {
    if (s.kind == kKindLine) return lsample(s.base, t);
    Seg a, b;
    cubic_split(to_cubic(s), t, &a, &b);
    return a.base.t;
}

// Segment::reversed (:186-197)
__device__ Seg seg_reversed(const Seg& s) {
    Seg r = s;
    r.base = L{s.base.t, s.base.f};
    if (s.kind != kKindQuad) r.ctrl = L{s.ctrl.t, s.ctrl.f};
    return r;
}

// Transform2F: matrix lanes (m11, m21, m12, m22) and a vector
// (geometry/src/transform2d.rs:34-47, 115-129, 148-175, 254-256, 301-326).
struct T2 { float m[4]; V v; };
__device__ __forceinline__ T2 t2_identity() { return T2{{1.0f, 0.0f, 0.0f, 1.0f}, {0.0f, 0.0f}}; }
__device__ __forceinline__ T2 t2_scale(float s) { return T2{{s, 0.0f, 0.0f, s}, {0.0f, 0.0f}}; }
__device__ __forceinline__ T2 t2_rotation(V u) { return T2{{u.x, u.y, -u.y, u.x}, {0.0f, 0.0f}}; }
__device__ __forceinline__ V t2_apply(const T2& t, V p) {
    return vadd(V{t.m[0] * p.x + t.m[2] * p.y, t.m[1] * p.x + t.m[3] * p.y}, t.v);
}
__device__ T2 t2_mul(const T2& a, const T2& b) {
    T2 r;
    r.m[0] = a.m[0] * b.m[0] + a.m[2] * b.m[1];
    r.m[1] = a.m[1] * b.m[0] + a.m[3] * b.m[1];
    r.m[2] = a.m[0] * b.m[2] + a.m[2] * b.m[3];
    r.m[3] = a.m[1] * b.m[2] + a.m[3] * b.m[3];
    r.v = t2_apply(a, b.v);
    return r;
}
__device__ __forceinline__ T2 t2_translate(const T2& t, V p) { T2 tr = t2_identity(); tr.v = p; return t2_mul(tr, t); }
__device__ Seg seg_transform(const Seg& s, const T2& t) {
    Seg r = s;
    r.base = L{t2_apply(t, s.base.f), t2_apply(t, s.base.t)};
    r.ctrl = L{t2_apply(t, s.ctrl.f), t2_apply(t, s.ctrl.t)};
    return r;
}

// UnitVector (geometry/src/unit_vector.rs:24-45)
__device__ __forceinline__ V uv_rotate_by(V s, V o) { return V{s.x * o.x - s.y * o.y, s.y * o.x + s.x * o.y}; }
__device__ __forceinline__ V uv_rev_rotate_by(V s, V o) { return V{s.x * o.x + s.y * o.y, s.y * o.x - s.x * o.y}; }
__device__ __forceinline__ V uv_halve_angle(V s) {
    const float x = s.x;
    return V{sqrtf(lane_max(0.5f * (1.0f + x), 0.0f)), sqrtf(lane_max(0.5f * (1.0f + -x), 0.0f))};
}

// Segment::arc_from_cos / quarter_circle_arc (content/src/segment.rs:94-122)
__device__ Seg arc_from_cos(float c) {
    if (c >= 1.0f - 0.001f) return mk_line(L{{1.0f, 0.0f}, {1.0f, 0.0f}});
    const float a = sqrtf((1.0f + c) * 0.5f), b = sqrtf((1.0f + -c) * 0.5f);
    const V p3{a * 1.0f, b * -1.0f}, p0{a * 1.0f, b * 1.0f};
    const float p1x = 4.0f - p0.x, p1y = (1.0f - p0.x) * (3.0f - p0.x) / p0.y;
    const float third = 1.0f / 3.0f;
    return mk_cubic(L{p3, p0}, L{V{p1x * third, -p1y * third}, V{p1x * third, p1y * third}});
}
__device__ Seg quarter_circle_arc() {
    const float sqrt2 = 1.41421356237309504880f;
    const V p0{sqrt2 * 0.5f, sqrt2 * 0.5f};
    const V p1{-sqrt2 / 6.0f + 4.0f / 3.0f, 7.0f * sqrt2 / 6.0f - 4.0f / 3.0f};
    return mk_cubic(L{V{p0.x * 1.0f, p0.y * -1.0f}, p0}, L{V{p1.x * 1.0f, p1.y * -1.0f}, p1});
}

constexpr float kStrokeTolerance = 0.01f;  // content/src/stroke.rs:22
constexpr float kGeomEpsilon = 0.001f;     // geometry/src/util.rs:15
constexpr int kStrokeMaxDepth = 32;        // bound of the offset recursion
constexpr uint32_t kCapReserve = 16;       // a cap is at most four cubic arcs
constexpr uint32_t kMaxStrokePieces = 1u << 16;  // offset pieces per segment (huge input cannot explode)

// Points written by a work item: counted only when pts is NULL.
struct Sink {
    float2* pts;
    uint8_t* flags;
    uint32_t n;
    __device__ void push(V p, uint8_t f) {
        if (pts) { pts[n] = make_float2(p.x, p.y); flags[n] = f; }
        n++;
    }
    // Contour::push_segment (content/src/outline.rs:576-600): the from point always
    __device__ void push_segment(const Seg& s) {
        push(s.base.f, 0);
        if (s.kind != kKindLine) {
            push(s.ctrl.f, PF_POINT_FLAG_CONTROL_POINT_0);
            if (s.kind != kKindQuad) push(s.ctrl.t, PF_POINT_FLAG_CONTROL_POINT_1);
        }
        push(s.base.t, 0);
    }
    // Contour::push_arc_from_unit_chord, clockwise (outline.rs:630-669)
    __device__ void push_arc(const T2& transform, L chord) {
        const T2 dir = t2_identity();
        V vector = chord.f;
        const V end_vector = chord.t;
        for (int i = 0; i < 4; i++) {
            V sweep = uv_rev_rotate_by(end_vector, vector);
            const bool last = sweep.x >= -0.001f && sweep.y >= -0.001f;
            Seg seg;
            if (!last) {
                sweep = V{0.0f, 1.0f};
                seg = quarter_circle_arc();
            } else {
                seg = arc_from_cos(sweep.x);
            }
            const V half = uv_halve_angle(sweep);
            seg = seg_transform(seg, t2_mul(t2_mul(transform, dir), t2_rotation(uv_rotate_by(half, vector))));
            push_segment(seg);
            if (last) break;
            vector = uv_rotate_by(vector, sweep);
        }
    }
};

// The last two points a piece pushes (position_of_last(2), (1)).
__device__ __forceinline__ void last_two(const Seg& s, V* p0, V* p1) {
    *p0 = s.kind == kKindLine ? s.base.f : (s.kind == kKindQuad ? s.ctrl.f : s.ctrl.t);
    *p1 = s.base.t;
}

// Contour::add_join (content/src/stroke.rs:412-448), the contour ending in p0, p1.
__device__ void add_join(Sink& k, V p0, V p1, float distance, int join, float miter_limit, V join_point,
                         L next_tangent) {
    const L prev{p0, p1};
    if (vsqlen(lvec(prev)) < kGeomEpsilon || vsqlen(lvec(next_tangent)) < kGeomEpsilon) return;
    if (join == PF_LINE_JOIN_MITER) {
        float t;
        if (intersection_t(prev, next_tangent, &t)) {
            if (t < -kGeomEpsilon) return;
            const V miter_endpoint = lsample(prev, t);
            const float threshold = miter_limit * distance;
            if (vsqlen(vsub(miter_endpoint, join_point)) > threshold * threshold) return;
            k.push(miter_endpoint, 0);
        }
    } else if (join == PF_LINE_JOIN_ROUND) {
        // a chord end at the join point has no direction: the reference would
        // push NaN points (normalising a zero vector); no join is pushed here
        const V cf = vsub(prev.t, join_point), ct = vsub(next_tangent.t, join_point);
        if ((cf.x == 0.0f && cf.y == 0.0f) || (ct.x == 0.0f && ct.y == 0.0f)) return;
        const T2 transform = t2_translate(t2_scale(fabsf(distance)), join_point);
        k.push_arc(transform, L{vnormalize(cf), vnormalize(ct)});
    }
}

// Offset::offset_once (content/src/stroke.rs:281-362)
__device__ V ctrl_of(L a, L b) {
    float t;
    return intersection_t(a, b, &t) ? lsample(a, t) : vlerp(a.t, b.f, 0.5f);
}
__device__ Seg offset_once(const Seg& s, float d) {
    if (s.kind == kKindLine) return mk_line(loffset(s.base, d));
    if (s.kind == kKindQuad) {
        const L s0 = loffset(L{s.base.f, s.ctrl.f}, d), s1 = loffset(L{s.ctrl.f, s.base.t}, d);
        return mk_quad(L{s0.f, s1.t}, ctrl_of(s0, s1));
    }
    if (veq(s.base.f, s.ctrl.f)) {
        const L s0 = loffset(L{s.base.f, s.ctrl.t}, d), s1 = loffset(L{s.ctrl.t, s.base.t}, d);
        return mk_cubic(L{s0.f, s1.t}, L{s0.f, ctrl_of(s0, s1)});
    }
    if (veq(s.ctrl.t, s.base.t)) {
        const L s0 = loffset(L{s.base.f, s.ctrl.f}, d), s1 = loffset(L{s.ctrl.f, s.base.t}, d);
        return mk_cubic(L{s0.f, s1.t}, L{ctrl_of(s0, s1), s1.t});
    }
    const L s0 = loffset(L{s.base.f, s.ctrl.f}, d), s1 = loffset(L{s.ctrl.f, s.ctrl.t}, d);
    const L s2 = loffset(L{s.ctrl.t, s.base.t}, d);
    float t0, t1;
    const bool h0 = intersection_t(s0, s1, &t0), h1 = intersection_t(s1, s2, &t1);
    if (h0 && h1) return mk_cubic(L{s0.f, s2.t}, L{lsample(s0, t0), lsample(s1, t1)});
    return mk_cubic(L{s0.f, s2.t}, L{vlerp(s0.t, s1.f, 0.5f), vlerp(s1.t, s2.f, 0.5f)});
}

// Offset::error_is_within_tolerance (:364-391): 17 samples
__device__ bool within_tolerance(const Seg& self, const Seg& other, float distance) {
    float mn = fabsf(distance) - kStrokeTolerance, mx = fabsf(distance) + kStrokeTolerance;
    mn = mn <= 0.0f ? 0.0f : mn * mn;
    mx = mx <= 0.0f ? 0.0f : mx * mx;
    for (uint32_t n = 0; n <= 16; n++) {
        const float t = (float)n / 16.0f;
        const float sq = vsqlen(vsub(seg_sample(self, t), seg_sample(other, t)));
        if (sq < mn || sq > mx) return false;
    }
    return true;
}

// One node of the offset recursion (Offset::offset, :238-254): true when it
// is a leaf, with the piece to push (the segment itself when tiny).
__device__ bool offset_leaf(const Seg& s, float d, int depth, Seg* piece, bool* limited) {
    if (vsqlen(lvec(s.base)) < kStrokeTolerance * kStrokeTolerance) { *piece = s; return true; }
    const Seg cand = offset_once(s, d);
    if (within_tolerance(s, cand, d)) { *piece = cand; return true; }
    if (depth >= kStrokeMaxDepth) { *piece = cand; *limited = true; return true; }
    return false;
}

// The first or the last piece of a segment's recursion (leftmost / rightmost leaf).
__device__ Seg edge_leaf(Seg s, float d, bool rightmost, bool* limited) {
    for (int depth = 0;; depth++) {
        Seg piece;
        if (offset_leaf(s, d, depth, &piece, limited)) return piece;
        Seg a, b;
        seg_split(s, 0.5f, &a, &b);
        s = rightmost ? b : a;
    }
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
struct StrokeDev {
    const float2* pts;
    const uint8_t* pflags;
    const uint32_t* cstarts;
    const uint8_t* closed;
    const PFCUDAStrokeStyle* styles;
    const uint32_t* contour_outline;  // [C] outline of each contour
    uint32_t C;
    uint32_t* cnt;                    // [C] per-contour counts before a scan
    uint32_t* nseg;                   // [C + 1] first segment of each contour (scanned)
    Seg* segs;                        // [S]
    uint32_t* item_base;              // [C + 1] first work item of each contour (scanned)
    uint32_t* item_cnt;               // [I] reserved points per item
    uint32_t* item_off;               // [I + 1] their scan
    uint32_t* actual;                 // [I] points written per item
    uint32_t* final_off;              // [I + 1] their scan
    float2* res_pts;                  // reserved layout
    uint8_t* res_flags;
    uint32_t* status;                 // bit 0: recursion depth bound reached
    unsigned long long* item_leaves;  // [I] the count pass's leaf slots of the item's recursion (0: not recorded)
    float4* item_last;                // [I] the last two points of the item's last piece
    float4* item_first;               // [I] the first piece's next_tangent (its to and from points)
    float2* item_first_at;            // [I] the first leaf's from point (the join point)
};

__device__ __forceinline__ bool is_end(const uint8_t* fl, uint32_t i) {
    return (fl[i] & (PF_POINT_FLAG_CONTROL_POINT_0 | PF_POINT_FLAG_CONTROL_POINT_1)) == 0;
}

// ContourIter (content/src/outline.rs:1020-1065): count (out == NULL) or write
// the segments of one contour.
__device__ uint32_t contour_segments(const StrokeDev& d, uint32_t c, Seg* out) {
    const uint32_t a = d.cstarts[c], n = d.cstarts[c + 1] - a;
    const bool closed = d.closed[c] != 0;
    const float2* p = d.pts + a;
    const uint8_t* fl = d.pflags + a;
    // indices past the end (a contour ending on a control point, which the
    // reference would read out of bounds) are clamped to the last point
    auto P = [&](uint32_t i) { const uint32_t j = i < n ? i : n - 1; return V{p[j].x, p[j].y}; };
    uint32_t count = 0, index = 1;
    while (n != 0 && index <= n && !(index == n && !closed)) {
        Seg sg;
        const V p0 = P(index - 1);
        if (index == n) {
            index++;
            sg = mk_line(L{p0, P(0)});
        } else {
            const uint32_t i1 = index++;
            if (is_end(fl, i1)) {
                sg = mk_line(L{p0, P(i1)});
            } else {
                const uint32_t i2 = index++;
                if (i2 >= n || is_end(fl, i2)) {
                    sg = mk_quad(L{p0, P(i2)}, P(i1));
                } else {
                    const uint32_t i3 = index++;
                    sg = mk_cubic(L{p0, P(i3)}, L{P(i1), P(i2)});
                }
            }
        }
        if (out) out[count] = sg;
        count++;
    }
    return count;
}

__global__ void k_stroke_count_segs(StrokeDev d) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < d.C) d.cnt[c] = contour_segments(d, c, nullptr);
}

__global__ void k_stroke_emit_segs(StrokeDev d) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < d.C) contour_segments(d, c, d.segs + d.nseg[c]);
}

// Items per contour: forward segments, forward tail, backward segments, backward tail.
__global__ void k_stroke_items(StrokeDev d) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < d.C) d.cnt[c] = 2u * (d.nseg[c + 1] - d.nseg[c]) + 2u;
}

__device__ __forceinline__ uint32_t upper_bound_items(const uint32_t* a, uint32_t n, uint32_t v) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] <= v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

struct ItemRef { uint32_t c, n, i; bool backward, tail; };
__device__ ItemRef item_ref(const StrokeDev& d, uint32_t g) {
    ItemRef r;
    r.c = upper_bound_items(d.item_base, d.C + 1, g) - 1;
    r.n = d.nseg[r.c + 1] - d.nseg[r.c];
    const uint32_t j = g - d.item_base[r.c];
    r.backward = j > r.n;
    r.i = r.backward ? j - r.n - 1 : j;
    r.tail = r.i == r.n;
    return r;
}

// Segment i of a pass: forward, the contour's segments in order; backward,
// reversed and in reverse order (offset_backward, content/src/stroke.rs:217-230).
__device__ __forceinline__ Seg pass_segment(const StrokeDev& d, const ItemRef& r, uint32_t i) {
    const Seg* sg = d.segs + d.nseg[r.c];
    return r.backward ? seg_reversed(sg[r.n - 1 - i]) : sg[i];
}

// The count pass records each segment's recursion as leaf start slots on a
// grid of 2^kStrokeLeafLevels parameter slots (as the flattening does), when
// every leaf lies at most that deep, the last two points of its last piece
// and what the join before its first piece needs of it.  The join before an
// item's first piece needs the previous item's last piece: k_stroke_joins
// counts it from the records once every item is walked, and the emit pass
// takes it from the previous item's record; no item descends the previous
// segment's recursion.  The emit pass recomputes only the recorded leaves
// (the splits from the root along each leaf's path, then one offset_once)
// instead of testing every node against the tolerance again.
constexpr int kStrokeLeafLevels = 6;

// One work item: count (sink without storage; records the item's leaves) or
// write its points (replaying recorded leaves).
__device__ void stroke_item(const StrokeDev& d, const ItemRef& r, uint32_t g, Sink& k, bool* limited) {
    const bool counting = k.pts == nullptr;
    const PFCUDAStrokeStyle st = d.styles[d.contour_outline[r.c]];
    const float radius = st.line_width * 0.5f;
    const bool closed = d.closed[r.c] != 0;
    if (r.tail) {
        // push_stroked_contour's closing join (:135-149); caps are written later
        if (!closed) { if (st.line_cap != PF_LINE_CAP_BUTT) k.n = kCapReserve; return; }
        if (r.n == 0 || (st.line_join != PF_LINE_JOIN_MITER && st.line_join != PF_LINE_JOIN_ROUND)) return;
        const Seg first = edge_leaf(pass_segment(d, r, 0), -radius, false, limited);
        const Seg last = edge_leaf(pass_segment(d, r, r.n - 1), -radius, true, limited);
        V p0, p1;
        last_two(last, &p0, &p1);
        const V q0 = first.base.f, q1 = first.kind == kKindLine ? first.base.t : first.ctrl.f;
        const V input_first = V{d.pts[d.cstarts[r.c]].x, d.pts[d.cstarts[r.c]].y};
        add_join(k, p0, p1, radius, st.line_join, st.miter_limit, input_first, L{q1, q0});
        return;
    }
    // the first segment of a pass joins with Bevel (offset_forward/backward, :208-230)
    const int join = r.i == 0 ? PF_LINE_JOIN_BEVEL : st.line_join;
    const bool joins = join == PF_LINE_JOIN_MITER || join == PF_LINE_JOIN_ROUND;
    const unsigned long long replay = counting ? 0ull : d.item_leaves[g];
    V p0{0.0f, 0.0f}, p1{0.0f, 0.0f};
    if (joins && !counting) {
        // the previous piece: the last piece of the previous item (same pass, segment i - 1)
        const float4 q = d.item_last[g - 1];
        p0 = V{q.x, q.y};
        p1 = V{q.z, q.w};
    }
    // Offset::add_to_contour (:256-279) for one leaf `s` with its piece; the
    // count pass leaves the first join to k_stroke_joins
    bool first = true;
    auto add = [&](const Seg& s, const Seg& piece) {
        const V q3 = piece.base.f, q4 = piece.kind == kKindLine ? piece.base.t : piece.ctrl.f;
        if (counting && first) {
            d.item_first[g] = make_float4(q4.x, q4.y, q3.x, q3.y);
            d.item_first_at[g] = make_float2(s.base.f.x, s.base.f.y);
        } else if (joins) {
            add_join(k, p0, p1, -radius, join, st.miter_limit, s.base.f, L{q4, q3});
        }
        first = false;
        k.push_segment(piece);
        last_two(piece, &p0, &p1);
    };
    if (replay) {
        // the recorded leaves in depth-first order: each recomputed from the root
        const Seg root = pass_segment(d, r, r.i);
        for (unsigned long long m = replay; m;) {
            const uint32_t start = (uint32_t)__ffsll((long long)m) - 1u;
            m &= m - 1ull;
            const uint32_t next = m ? (uint32_t)__ffsll((long long)m) - 1u : 64u;
            const int depth = kStrokeLeafLevels - (31 - __clz((int)(next - start)));
            const uint32_t addr = start >> (kStrokeLeafLevels - depth);
            Seg s = root;
            for (int lv = depth - 1; lv >= 0; lv--) {
                Seg a, b;
                seg_split(s, 0.5f, &a, &b);
                s = ((addr >> lv) & 1u) ? b : a;
            }
            // offset_leaf's piece for a leaf above the depth bound: the segment
            // itself when tiny, else its offset (which the count pass found
            // within the tolerance)
            const Seg piece = vsqlen(lvec(s.base)) < kStrokeTolerance * kStrokeTolerance ? s : offset_once(s, -radius);
            add(s, piece);
        }
        return;
    }
    // depth-first walk of the offset recursion (Offset::offset, :238-254)
    Seg stack[kStrokeMaxDepth + 2];
    int depth_of[kStrokeMaxDepth + 2];
    uint32_t addr_of[kStrokeMaxDepth + 2];
    int sp = 0;
    stack[sp] = pass_segment(d, r, r.i);
    depth_of[sp] = 0;
    addr_of[sp++] = 0;
    uint32_t pieces = 0;  // at most kMaxStrokePieces per segment, then the walk stops
    unsigned long long leaves = 0;
    bool recordable = true;
    while (sp > 0) {
        const Seg s = stack[--sp];
        const int depth = depth_of[sp];
        const uint32_t addr = addr_of[sp];
        Seg piece;
        if (!offset_leaf(s, -radius, depth, &piece, limited)) {
            Seg a, b;
            seg_split(s, 0.5f, &a, &b);
            stack[sp] = b; depth_of[sp] = depth + 1; addr_of[sp++] = 2u * addr + 1u;
            stack[sp] = a; depth_of[sp] = depth + 1; addr_of[sp++] = 2u * addr;
            continue;
        }
        if (depth <= kStrokeLeafLevels) leaves |= 1ull << (addr << (kStrokeLeafLevels - depth));
        else recordable = false;
        add(s, piece);
        if (++pieces >= kMaxStrokePieces) { *limited = true; recordable = false; break; }
    }
    if (counting) {
        d.item_leaves[g] = recordable ? leaves : 0ull;
        d.item_last[g] = make_float4(p0.x, p0.y, p1.x, p1.y);
    }
}

__global__ void k_stroke_count(StrokeDev d, uint32_t items) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < items; g += gridDim.x * blockDim.x) {
        bool limited = false;
        Sink k{nullptr, nullptr, 0};
        stroke_item(d, item_ref(d, g), g, k, &limited);
        d.item_cnt[g] = k.n;
        if (limited) atomicOr(d.status, 1u);
    }
}

// The join before each item's first piece (count pass): from the previous
// item's last piece and the item's first, as recorded.
__global__ void k_stroke_joins(StrokeDev d, uint32_t items) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < items; g += gridDim.x * blockDim.x) {
        const ItemRef r = item_ref(d, g);
        if (r.tail || r.i == 0) continue;  // tails count their own joins; a pass's first segment joins with Bevel
        const PFCUDAStrokeStyle st = d.styles[d.contour_outline[r.c]];
        if (st.line_join != PF_LINE_JOIN_MITER && st.line_join != PF_LINE_JOIN_ROUND) continue;
        const float4 last = d.item_last[g - 1], nt = d.item_first[g];
        const float2 at = d.item_first_at[g];
        Sink k{nullptr, nullptr, 0};
        add_join(k, V{last.x, last.y}, V{last.z, last.w}, -(st.line_width * 0.5f), st.line_join, st.miter_limit,
                 V{at.x, at.y}, L{V{nt.x, nt.y}, V{nt.z, nt.w}});
        d.item_cnt[g] += k.n;
    }
}

__global__ void k_stroke_emit(StrokeDev d, uint32_t items) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < items; g += gridDim.x * blockDim.x) {
        const ItemRef r = item_ref(d, g);
        const uint32_t off = d.item_off[g], reserved = d.item_off[g + 1] - off;
        if (r.tail && d.closed[r.c] == 0) continue;  // caps: k_stroke_caps
        bool limited = false;
        Sink k{d.res_pts + off, d.res_flags + off, 0};
        stroke_item(d, r, g, k, &limited);
        d.actual[g] = reserved;
    }
}

// OutlineStrokeToFill::add_cap (content/src/stroke.rs:151-199) on an output
// contour read through `at` (logical point index -> reserved slot).
template <class At>
__device__ void write_cap(const StrokeDev& d, const PFCUDAStrokeStyle& st, At at, uint32_t len, Sink& k) {
    if (st.line_cap == PF_LINE_CAP_BUTT || len < 2) return;
    auto get = [&](uint32_t i) { const float2 q = d.res_pts[at(i)]; return V{q.x, q.y}; };
    const float width = st.line_width;
    const V p1 = get(len - 1);
    V p0;
    uint32_t i = len - 2;
    for (;;) {
        p0 = get(i);
        if (vsqlen(vsub(p1, p0)) > kGeomEpsilon) break;
        if (i == 0) return;
        i--;
    }
    const V gradient = vnormalize(vsub(p1, p0));
    if (st.line_cap == PF_LINE_CAP_SQUARE) {
        const V offset = vmul(gradient, width * 0.5f);
        const V p2 = vadd(p1, offset);
        const V p3 = vadd(p2, vmulv(vyx(gradient), V{-width, width}));
        k.push(p2, 0);
        k.push(p3, 0);
        k.push(vsub(p3, offset), 0);
    } else {
        const V offset = vmulv(vyx(gradient), V{-1.0f, 1.0f});
        const V translation = vadd(p1, vmul(offset, width * 0.5f));
        k.push_arc(t2_translate(t2_scale(width * 0.5f), translation), L{vmul(offset, -1.0f), offset});
    }
}

// Caps of open contours: after the forward pass, then after the backward one
// (whose contour also holds the forward cap's points).
__global__ void k_stroke_caps(StrokeDev d) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.C || d.closed[c] != 0) return;
    const PFCUDAStrokeStyle st = d.styles[d.contour_outline[c]];
    const uint32_t n = d.nseg[c + 1] - d.nseg[c], g0 = d.item_base[c];
    const uint32_t f0 = d.item_off[g0], fcap = d.item_off[g0 + n];
    const uint32_t b0 = d.item_off[g0 + n + 1], bcap = d.item_off[g0 + 2 * n + 1];
    const uint32_t lf = fcap - f0, lb = bcap - b0;
    Sink k1{d.res_pts + fcap, d.res_flags + fcap, 0};
    write_cap(d, st, [&](uint32_t i) { return f0 + i; }, lf, k1);
    d.actual[g0 + n] = k1.n;
    Sink k2{d.res_pts + bcap, d.res_flags + bcap, 0};
    const uint32_t n1 = k1.n;
    write_cap(d, st, [&](uint32_t i) { return i < lf ? f0 + i : (i < lf + n1 ? fcap + (i - lf) : b0 + (i - lf - n1)); },
              lf + n1 + lb, k2);
    d.actual[g0 + 2 * n + 1] = k2.n;
}

// Gather every item's written points to their final places.
// A warp per 32 items: their output points are one contiguous range, which
// the lanes copy in order (each point's item found among the warp's 32 by a
// search over their output offsets), so the stores coalesce.
__global__ void k_stroke_compact(StrokeDev d, uint32_t items, float2* out_pts, uint8_t* out_flags) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t g0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32u; g0 < items; g0 += warps * 32u) {
        const uint32_t g = g0 + lane;
        const uint32_t last = min(g0 + 32u, items);  // the range ends at the first item past the warp's
        const uint32_t dst = g < items ? d.final_off[g] : d.final_off[last];
        const uint32_t src = g < items ? d.item_off[g] : 0u;
        const uint32_t begin = __shfl_sync(0xffffffffu, dst, 0), end = d.final_off[last];
        for (uint32_t o0 = begin; o0 < end; o0 += 32u) {  // warp-uniform: every lane shuffles
            const uint32_t o = o0 + lane;
            uint32_t j = 0;  // the last lane whose output starts at or before o
#pragma unroll
            for (uint32_t step = 16; step > 0; step >>= 1) {
                const uint32_t v = __shfl_sync(0xffffffffu, dst, (int)(j + step));
                if (v <= o) j += step;
            }
            const uint32_t from = __shfl_sync(0xffffffffu, src, (int)j) + (o - __shfl_sync(0xffffffffu, dst, (int)j));
            if (o < end) {
                out_pts[o] = d.res_pts[from];
                out_flags[o] = d.res_flags[from];
            }
        }
    }
}

// Output contours: two per closed input contour (forward, backward), one per
// open one; cbase = scanned output contour index per input contour.
__global__ void k_stroke_ncont(StrokeDev d) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < d.C) d.cnt[c] = d.closed[c] != 0 ? 2u : 1u;
}
__global__ void k_stroke_contours(StrokeDev d, const uint32_t* cbase, uint32_t* out_cstarts, uint32_t total_points) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < d.C) {
        const uint32_t n = d.nseg[c + 1] - d.nseg[c], g0 = d.item_base[c], o = cbase[c];
        out_cstarts[o] = d.final_off[g0];
        if (d.closed[c] != 0) out_cstarts[o + 1] = d.final_off[g0 + n + 1];
    }
    if (c == 0) out_cstarts[cbase[d.C]] = total_points;
}

// ---- dashes: OutlineDash (content/src/dash.rs:18-152) -----------------------
// The distance left in the current dash is carried from segment to segment in
// single precision, and each cut's remainder is the next step's segment, so an
// outline is one sequential walk; a thread walks one outline, twice (count,
// then write at the scanned offsets).  Outlines without a pattern are copied
// by a thread per point and a thread per contour.
constexpr float kDashEpsilon = 0.0001f;       // content/src/dash.rs:16
constexpr uint32_t kMaxDashSteps = 1u << 20;  // steps per outline (a cut or a whole segment each)

struct DashDev {
    const float2* pts;
    const uint8_t* pflags;
    const uint32_t* cstarts;   // [C + 1]
    const uint8_t* closed;     // [C]
    const uint32_t* ostarts;   // [O + 1] contours of each outline
    const uint32_t* opstarts;  // [O + 1] points of each outline (cstarts[ostarts[o]])
    const float* dashes;
    const uint32_t* dstarts;   // [O + 1] each outline's pattern
    const float* offsets;      // [O]
    uint32_t O, C;
    uint32_t* cnt_pts;         // [O] output points per outline, then scanned into pbase
    uint32_t* cnt_cont;        // [O] output contours per outline, then scanned into cbase
    const uint32_t* pbase;     // [O + 1]
    const uint32_t* cbase;     // [O + 1]
    float2* out_pts;
    uint8_t* out_flags;
    uint32_t* out_cstarts;
    uint8_t* out_closed;
    uint32_t* status;          // bit 0: an outline reached the step bound
};

// ContourIter (content/src/outline.rs:1020-1065) as a cursor, closing segment
// included; indices past the end clamp to the last point, as contour_segments.
struct SegCursor {
    const float2* p;
    const uint8_t* fl;
    uint32_t n, index;
    bool closed;
    __device__ V P(uint32_t i) const { const uint32_t j = i < n ? i : n - 1; return V{p[j].x, p[j].y}; }
    __device__ bool next(Seg* sg) {
        if (n == 0 || index > n || (index == n && !closed)) return false;
        const V p0 = P(index - 1);
        if (index == n) { index++; *sg = mk_line(L{p0, P(0)}); return true; }
        const uint32_t i1 = index++;
        if (is_end(fl, i1)) { *sg = mk_line(L{p0, P(i1)}); return true; }
        const uint32_t i2 = index++;
        if (i2 >= n || is_end(fl, i2)) { *sg = mk_quad(L{p0, P(i2)}, P(i1)); return true; }
        const uint32_t i3 = index++;
        *sg = mk_cubic(L{p0, P(i3)}, L{P(i1), P(i2)});
        return true;
    }
};

// The dashes' output of one outline: counts when pts is NULL, else writes
// from the outline's scanned bases.
struct DashSink {
    float2* pts;
    uint8_t* flags;
    uint32_t* cstarts;
    uint8_t* closed;
    uint32_t pbase, cbase;
    uint32_t n, nc, start;  // points, finished contours, first point of the open contour
    __device__ void push(V q, uint8_t f) {
        if (pts) { pts[pbase + n] = make_float2(q.x, q.y); flags[pbase + n] = f; }
        n++;
    }
    // Contour::push_segment (content/src/outline.rs:576-600): the from point always
    __device__ void push_segment(const Seg& s) {
        push(s.base.f, 0);
        if (s.kind != kKindLine) {
            push(s.ctrl.f, PF_POINT_FLAG_CONTROL_POINT_0);
            if (s.kind != kKindQuad) push(s.ctrl.t, PF_POINT_FLAG_CONTROL_POINT_1);
        }
        push(s.base.t, 0);
    }
    // Outline::push_contour of the dash's open contour (outline.rs:180-192):
    // an empty one is dropped
    __device__ void end_contour() {
        if (n == start) return;
        if (pts) { cstarts[cbase + nc] = pbase + start; closed[cbase + nc] = 0; }
        nc++;
        start = n;
    }
};

// Segment::arc_length (content/src/segment.rs:246-249): the chord's length
__device__ __forceinline__ float chord_length(const Seg& s) { return sqrtf(vsqlen(lvec(s.base))); }

// OutlineDash::dash + into_outline (dash.rs:46-57) for outline o with a
// non-empty pattern; returns true when the step bound cut it short.
__device__ bool dash_outline(const DashDev& d, uint32_t o, DashSink& k) {
    const float* dashes = d.dashes + d.dstarts[o];
    const uint32_t nd = d.dstarts[o + 1] - d.dstarts[o];
    // DashState::new (:124-145): the offset modulo the pattern's sum (a fold
    // from zero), then the whole dashes it covers are skipped; the distance
    // left starts at what remains of the offset
    float total = 0.0f;
    for (uint32_t i = 0; i < nd; i++) total = total + dashes[i];
    float offset = fmodf(d.offsets[o], total);
    uint32_t idx = 0;
    while (idx < nd) {
        if (offset < dashes[idx]) break;
        offset = offset - dashes[idx];
        idx++;
    }
    float left = offset;
    uint32_t steps = 0;
    bool limited = false;
    // ContourDash::dash (:73-113) over every contour; the open dash contour
    // carries from one contour to the next
    for (uint32_t c = d.ostarts[o]; c < d.ostarts[o + 1] && !limited; c++) {
        const uint32_t a = d.cstarts[c];
        SegCursor it{d.pts + a, d.pflags + a, d.cstarts[c + 1] - a, 1u, d.closed[c] != 0};
        Seg queued;
        bool have = false;
        for (;;) {
            if (!have && !it.next(&queued)) break;
            if (steps++ == kMaxDashSteps) { limited = true; break; }
            Seg cur = queued;
            have = false;
            float distance = left;
            const float t = distance / chord_length(cur);  // time_for_distance (segment.rs:251-254)
            if (t < 1.0f) {
                Seg a0, b0;
                seg_split(cur, t, &a0, &b0);
                cur = a0;
                queued = b0;
                have = true;
            } else {
                distance = chord_length(cur);
            }
            const bool on = (idx & 1u) == 0u;  // DashState::is_on (:147-150)
            if (on) k.push_segment(cur);
            left = left - distance;
            if (left < kDashEpsilon) {
                if (on) k.end_contour();
                // the next dash, wrapping (an offset rounding onto the pattern's
                // end wraps here too; the reference would index past it)
                idx++;
                if (idx >= nd) idx = 0;
                left = dashes[idx];
            }
        }
    }
    if ((idx & 1u) == 0u) k.end_contour();
    return limited;
}

__global__ void k_dash_count(DashDev d) {
    for (uint32_t o = blockIdx.x * blockDim.x + threadIdx.x; o < d.O; o += gridDim.x * blockDim.x) {
        if (d.dstarts[o + 1] == d.dstarts[o]) {
            d.cnt_pts[o] = d.opstarts[o + 1] - d.opstarts[o];
            d.cnt_cont[o] = d.ostarts[o + 1] - d.ostarts[o];
            continue;
        }
        DashSink k{nullptr, nullptr, nullptr, nullptr, 0u, 0u, 0u, 0u, 0u};
        if (dash_outline(d, o, k)) atomicOr(d.status, 1u);
        d.cnt_pts[o] = k.n;
        d.cnt_cont[o] = k.nc;
    }
}

__global__ void k_dash_emit(DashDev d) {
    for (uint32_t o = blockIdx.x * blockDim.x + threadIdx.x; o < d.O; o += gridDim.x * blockDim.x) {
        if (d.dstarts[o + 1] == d.dstarts[o]) continue;
        DashSink k{d.out_pts, d.out_flags, d.out_cstarts, d.out_closed, d.pbase[o], d.cbase[o], 0u, 0u, 0u};
        dash_outline(d, o, k);
    }
}

// Points of outlines without a pattern, unchanged: a thread per input point.
__global__ void k_dash_copy_points(DashDev d) {
    const uint32_t end = d.opstarts[d.O];
    for (uint32_t p = d.opstarts[0] + blockIdx.x * blockDim.x + threadIdx.x; p < end; p += gridDim.x * blockDim.x) {
        const uint32_t o = upper_bound_items(d.opstarts, d.O + 1, p) - 1;
        if (d.dstarts[o + 1] != d.dstarts[o]) continue;
        const uint32_t q = d.pbase[o] + (p - d.opstarts[o]);
        d.out_pts[q] = d.pts[p];
        d.out_flags[q] = d.pflags[p];
    }
}

// Contours of outlines without a pattern, with their closed flags; thread 0
// also ends the contour list.
__global__ void k_dash_copy_contours(DashDev d, uint32_t total_points) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < d.C; c += gridDim.x * blockDim.x) {
        const uint32_t o = upper_bound_items(d.ostarts, d.O + 1, c) - 1;
        if (o >= d.O || d.dstarts[o + 1] != d.dstarts[o]) continue;
        const uint32_t q = d.cbase[o] + (c - d.ostarts[o]);
        d.out_cstarts[q] = d.pbase[o] + (d.cstarts[c] - d.opstarts[o]);
        d.out_closed[q] = d.closed[c];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) d.out_cstarts[d.cbase[d.O]] = total_points;
}

}  // namespace
}  // namespace pf

namespace pf {
namespace {
template <class T>
struct SBuf {
    T* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t n) {
        if (n <= cap && p) return cudaSuccess;
        if (p) { cudaFree(p); p = nullptr; cap = 0; }
        const size_t want = n > 0 ? n : 1;
        const cudaError_t e = cudaMalloc((void**)&p, want * sizeof(T));
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; cap = 0; }
};
int32_t cuda_status_of(cudaError_t e) {
    return e == cudaErrorMemoryAllocation ? PF_CUDA_ERR_CAPACITY : PF_CUDA_ERR_LAUNCH;
}
#define PF_STROKE_TRY(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return cuda_status_of(e_); } while (0)
uint32_t grid_for(uint64_t n) {
    const uint64_t b = (n + 255) / 256;
    const uint64_t cap = (uint64_t)device_sm_count() * 8;
    return (uint32_t)(b == 0 ? 1 : (b > cap ? cap : b));
}
}  // namespace

struct StrokeWork {
    SBuf<float2> pts, res_pts, out_pts;
    SBuf<uint8_t> pflags, closed, res_flags, out_flags;
    SBuf<uint32_t> cstarts, contour_outline, cnt, nseg, item_base, item_cnt, item_off, actual, final_off, cbase,
        out_cstarts, status, partials;
    SBuf<PFCUDAStrokeStyle> styles;
    SBuf<Seg> segs;
    SBuf<unsigned long long> item_leaves;
    SBuf<float4> item_last, item_first;
    SBuf<float2> item_first_at;
    // dashes: the input's index arrays, the patterns, counts and their scans,
    // and the dashed outlines (the stroke's input when both run)
    SBuf<uint32_t> d_cstarts, d_ostarts, d_opstarts, d_dstarts, d_cnt_p, d_cnt_c, d_pbase, d_cbase, dash_cstarts,
        dash_ostarts;
    SBuf<float> d_dashes, d_offsets;
    SBuf<float2> dash_pts;
    SBuf<uint8_t> dash_flags, dash_closed;
    SBuf<PFCUDAStrokeStyle> dash_styles;
};

StrokeWork* stroke_work_create() { return new StrokeWork(); }

void stroke_work_destroy(StrokeWork* w) {
    if (!w) return;
    w->pts.release(); w->res_pts.release(); w->out_pts.release(); w->pflags.release(); w->closed.release();
    w->res_flags.release(); w->out_flags.release(); w->cstarts.release(); w->contour_outline.release();
    w->cnt.release(); w->nseg.release(); w->item_base.release(); w->item_cnt.release(); w->item_off.release();
    w->actual.release(); w->final_off.release(); w->cbase.release(); w->out_cstarts.release();
    w->status.release(); w->partials.release(); w->styles.release(); w->segs.release();
    w->item_leaves.release(); w->item_last.release(); w->item_first.release(); w->item_first_at.release();
    w->d_cstarts.release(); w->d_ostarts.release(); w->d_opstarts.release(); w->d_dstarts.release();
    w->d_cnt_p.release(); w->d_cnt_c.release(); w->d_pbase.release(); w->d_cbase.release();
    w->dash_cstarts.release(); w->dash_ostarts.release(); w->d_dashes.release(); w->d_offsets.release();
    w->dash_pts.release(); w->dash_flags.release(); w->dash_closed.release(); w->dash_styles.release();
    delete w;
}

// Host copies of an outline set's index arrays, checked before any kernel
// reads them: contour starts in order and within the points, outline starts
// in order from 0 to the contour count.
int32_t read_index_arrays(const PFCUDAStrokeInput* in, std::vector<uint32_t>& hc, std::vector<uint32_t>& ho) {
    if (in->memory != PF_MEMORY_HOST && in->memory != PF_MEMORY_DEVICE) return PF_CUDA_ERR_INVALID;
    const uint32_t NP = in->point_count, C = in->contour_count, O = in->outline_count;
    if (NP >= 0x40000000u || C >= 0x20000000u || O >= 0x20000000u) return PF_CUDA_ERR_INVALID;
    if ((NP && (!in->points || !in->point_flags)) || !in->contour_starts || (C && !in->contour_closed) ||
        !in->outline_starts)
        return PF_CUDA_ERR_INVALID;
    const cudaMemcpyKind down = in->memory == PF_MEMORY_DEVICE ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost;
    hc.assign(C + 1, 0u);
    ho.assign(O + 1, 0u);
    PF_STROKE_TRY(cudaMemcpy(hc.data(), in->contour_starts, sizeof(uint32_t) * (C + 1), down));
    PF_STROKE_TRY(cudaMemcpy(ho.data(), in->outline_starts, sizeof(uint32_t) * (O + 1), down));
    for (uint32_t c = 0; c < C; c++)
        if (hc[c] > hc[c + 1]) return PF_CUDA_ERR_INVALID;
    if (hc[C] > NP || ho[0] != 0 || ho[O] != C) return PF_CUDA_ERR_INVALID;
    for (uint32_t o = 0; o < O; o++)
        if (ho[o] > ho[o + 1]) return PF_CUDA_ERR_INVALID;
    return PF_CUDA_OK;
}

int32_t stroke_run(StrokeWork* w, cudaStream_t s, const PFCUDAStrokeInput* in, PFCUDAStrokeOutput* out) {
    if (!w || !in || !out) return PF_CUDA_ERR_INVALID;
    if (out->memory != PF_MEMORY_HOST && out->memory != PF_MEMORY_DEVICE) return PF_CUDA_ERR_INVALID;
    std::vector<uint32_t> hc, ho;
    const int32_t irc = read_index_arrays(in, hc, ho);
    if (irc != PF_CUDA_OK) return irc;
    const uint32_t NP = in->point_count, C = in->contour_count, O = in->outline_count;
    if (O && !in->styles) return PF_CUDA_ERR_INVALID;
    const bool dev_in = in->memory == PF_MEMORY_DEVICE;
    const cudaMemcpyKind up = dev_in ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    std::vector<PFCUDAStrokeStyle> hs(O);
    const cudaMemcpyKind down = dev_in ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost;
    if (O) PF_STROKE_TRY(cudaMemcpy(hs.data(), in->styles, sizeof(PFCUDAStrokeStyle) * O, down));
    std::vector<uint32_t> outline_of(C > 0 ? C : 1);
    for (uint32_t o = 0; o < O; o++) {
        const PFCUDAStrokeStyle& st = hs[o];
        if (!(st.line_width >= 0.0f && st.line_width < 1e30f) || st.line_cap < 0 || st.line_cap > 2 ||
            st.line_join < 0 || st.line_join > 2 || !(std::fabs(st.miter_limit) < 1e30f))
            return PF_CUDA_ERR_INVALID;
        for (uint32_t c = ho[o]; c < ho[o + 1]; c++) outline_of[c] = o;
    }

    PF_STROKE_TRY(w->contour_outline.ensure(C + 1));
    PF_STROKE_TRY(w->styles.ensure(O + 1));
    PF_STROKE_TRY(w->cnt.ensure(C + 1));
    PF_STROKE_TRY(w->nseg.ensure(C + 1));
    PF_STROKE_TRY(w->item_base.ensure(C + 1));
    PF_STROKE_TRY(w->cbase.ensure(C + 1));
    PF_STROKE_TRY(w->status.ensure(1));
    PF_STROKE_TRY(w->partials.ensure((size_t)C / 2048 + 2));
    StrokeDev d{};
    if (dev_in) {
        d.pts = (const float2*)in->points;
        d.pflags = in->point_flags;
        d.closed = in->contour_closed;
    } else {
        PF_STROKE_TRY(w->pts.ensure(NP + 1));
        PF_STROKE_TRY(w->pflags.ensure(NP + 1));
        PF_STROKE_TRY(w->closed.ensure(C + 1));
        if (NP) {
            PF_STROKE_TRY(cudaMemcpyAsync(w->pts.p, in->points, sizeof(float2) * NP, up, s));
            PF_STROKE_TRY(cudaMemcpyAsync(w->pflags.p, in->point_flags, NP, up, s));
        }
        if (C) PF_STROKE_TRY(cudaMemcpyAsync(w->closed.p, in->contour_closed, C, up, s));
        d.pts = w->pts.p;
        d.pflags = w->pflags.p;
        d.closed = w->closed.p;
    }
    PF_STROKE_TRY(w->cstarts.ensure(C + 1));
    PF_STROKE_TRY(cudaMemcpyAsync(w->cstarts.p, hc.data(), sizeof(uint32_t) * (C + 1), cudaMemcpyHostToDevice, s));
    PF_STROKE_TRY(cudaMemcpyAsync(w->contour_outline.p, outline_of.data(), sizeof(uint32_t) * outline_of.size(),
                                  cudaMemcpyHostToDevice, s));
    if (O) PF_STROKE_TRY(cudaMemcpyAsync(w->styles.p, hs.data(), sizeof(PFCUDAStrokeStyle) * O, cudaMemcpyHostToDevice, s));
    d.cstarts = w->cstarts.p;
    d.styles = w->styles.p;
    d.contour_outline = w->contour_outline.p;
    d.C = C;
    d.cnt = w->cnt.p;
    d.nseg = w->nseg.p;
    d.item_base = w->item_base.p;
    d.status = w->status.p;
    PF_STROKE_TRY(cudaMemsetAsync(w->status.p, 0, sizeof(uint32_t), s));
    ScanTemp tmp{w->partials.p, (uint32_t)w->partials.cap};
    const uint32_t gc = (C + 255) / 256 > 0 ? (C + 255) / 256 : 1;

    // 1. segments
    if (C) { count_launch(); k_stroke_count_segs<<<gc, 256, 0, s>>>(d); }
    launch_scan(w->cnt.p, w->nseg.p, nullptr, C, C, 0, nullptr, tmp, s);
    uint32_t S = 0;
    PF_STROKE_TRY(cudaMemcpyAsync(&S, w->nseg.p + C, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    PF_STROKE_TRY(cudaStreamSynchronize(s));
    PF_STROKE_TRY(w->segs.ensure((size_t)S + 1));
    d.segs = w->segs.p;
    if (C) { count_launch(); k_stroke_emit_segs<<<gc, 256, 0, s>>>(d); }
    if (C) { count_launch(); k_stroke_items<<<gc, 256, 0, s>>>(d); }
    launch_scan(w->cnt.p, w->item_base.p, nullptr, C, C, 0, nullptr, tmp, s);
    const uint64_t I64 = 2ull * S + 2ull * C;
    if (I64 >= 0x40000000ull) return PF_CUDA_ERR_CAPACITY;
    const uint32_t I = (uint32_t)I64;

    // 2. counts, 3. points, 4. caps
    PF_STROKE_TRY(w->item_cnt.ensure(I + 1));
    PF_STROKE_TRY(w->item_off.ensure(I + 1));
    PF_STROKE_TRY(w->actual.ensure(I + 1));
    PF_STROKE_TRY(w->final_off.ensure(I + 1));
    PF_STROKE_TRY(w->item_leaves.ensure(I + 1));
    PF_STROKE_TRY(w->item_last.ensure(I + 1));
    PF_STROKE_TRY(w->item_first.ensure(I + 1));
    PF_STROKE_TRY(w->item_first_at.ensure(I + 1));
    PF_STROKE_TRY(w->partials.ensure((size_t)(I > C ? I : C) / 2048 + 2));
    tmp = ScanTemp{w->partials.p, (uint32_t)w->partials.cap};
    d.item_cnt = w->item_cnt.p;
    d.item_off = w->item_off.p;
    d.actual = w->actual.p;
    d.final_off = w->final_off.p;
    d.item_leaves = w->item_leaves.p;
    d.item_last = w->item_last.p;
    d.item_first = w->item_first.p;
    d.item_first_at = w->item_first_at.p;
    if (I) { count_launch(); k_stroke_count<<<grid_for(I), 256, 0, s>>>(d, I); }
    if (I) { count_launch(); k_stroke_joins<<<grid_for(I), 256, 0, s>>>(d, I); }
    launch_scan(w->item_cnt.p, w->item_off.p, nullptr, I, I, 0, nullptr, tmp, s);
    uint32_t R = 0;
    PF_STROKE_TRY(cudaMemcpyAsync(&R, w->item_off.p + I, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    PF_STROKE_TRY(cudaStreamSynchronize(s));
    PF_STROKE_TRY(w->res_pts.ensure((size_t)R + 1));
    PF_STROKE_TRY(w->res_flags.ensure((size_t)R + 1));
    d.res_pts = w->res_pts.p;
    d.res_flags = w->res_flags.p;
    PF_STROKE_TRY(cudaMemsetAsync(w->actual.p, 0, sizeof(uint32_t) * (I + 1), s));
    if (I) { count_launch(); k_stroke_emit<<<grid_for(I), 256, 0, s>>>(d, I); }
    if (C) { count_launch(); k_stroke_caps<<<gc, 256, 0, s>>>(d); }
    launch_scan(w->actual.p, w->final_off.p, nullptr, I, I, 0, nullptr, tmp, s);
    if (C) { count_launch(); k_stroke_ncont<<<gc, 256, 0, s>>>(d); }
    launch_scan(w->cnt.p, w->cbase.p, nullptr, C, C, 0, nullptr, tmp, s);
    uint32_t P = 0, OC = 0, status = 0;
    PF_STROKE_TRY(cudaMemcpyAsync(&P, w->final_off.p + I, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    PF_STROKE_TRY(cudaMemcpyAsync(&OC, w->cbase.p + C, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    PF_STROKE_TRY(cudaMemcpyAsync(&status, w->status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    std::vector<uint32_t> hcb(C + 1);
    PF_STROKE_TRY(cudaMemcpyAsync(hcb.data(), w->cbase.p, sizeof(uint32_t) * (C + 1), cudaMemcpyDeviceToHost, s));
    PF_STROKE_TRY(cudaStreamSynchronize(s));
    PF_STROKE_TRY(cudaGetLastError());

    // 5. compaction into the output
    out->point_count = P;
    out->contour_count = OC;
    if (out->point_capacity < P || out->contour_capacity < OC) return PF_CUDA_ERR_CAPACITY;
    if ((P && (!out->points || !out->point_flags)) || !out->contour_starts || !out->outline_starts)
        return PF_CUDA_ERR_INVALID;
    std::vector<uint32_t> hos(O + 1);
    for (uint32_t o = 0; o <= O; o++) hos[o] = hcb[ho[o]];
    const bool dev_out = out->memory == PF_MEMORY_DEVICE;
    float2* dst_pts = (float2*)out->points;
    uint8_t* dst_flags = out->point_flags;
    uint32_t* dst_cs = out->contour_starts;
    if (!dev_out) {
        PF_STROKE_TRY(w->out_pts.ensure((size_t)P + 1));
        PF_STROKE_TRY(w->out_flags.ensure((size_t)P + 1));
        PF_STROKE_TRY(w->out_cstarts.ensure((size_t)OC + 1));
        dst_pts = w->out_pts.p;
        dst_flags = w->out_flags.p;
        dst_cs = w->out_cstarts.p;
    }
    if (I) { count_launch(); k_stroke_compact<<<grid_for(I), 256, 0, s>>>(d, I, dst_pts, dst_flags); }
    { count_launch(); k_stroke_contours<<<gc, 256, 0, s>>>(d, w->cbase.p, dst_cs, P); }
    if (dev_out) {
        PF_STROKE_TRY(cudaMemcpyAsync(out->outline_starts, hos.data(), sizeof(uint32_t) * (O + 1),
                                      cudaMemcpyHostToDevice, s));
    } else {
        if (P) {
            PF_STROKE_TRY(cudaMemcpyAsync(out->points, dst_pts, sizeof(float2) * P, cudaMemcpyDeviceToHost, s));
            PF_STROKE_TRY(cudaMemcpyAsync(out->point_flags, dst_flags, P, cudaMemcpyDeviceToHost, s));
        }
        PF_STROKE_TRY(cudaMemcpyAsync(out->contour_starts, dst_cs, sizeof(uint32_t) * (OC + 1), cudaMemcpyDeviceToHost, s));
        std::memcpy(out->outline_starts, hos.data(), sizeof(uint32_t) * (O + 1));
    }
    PF_STROKE_TRY(cudaStreamSynchronize(s));
    PF_STROKE_TRY(cudaGetLastError());
    return (status & 1u) ? PF_CUDA_ERR_LIMIT : PF_CUDA_OK;
}

namespace {
// Blocks of 64 threads for the walks (a thread per outline), so that a few
// hundred outlines still spread over the SMs.
uint32_t walk_grid(uint64_t n) {
    const uint64_t b = (n + 63) / 64;
    const uint64_t cap = (uint64_t)device_sm_count() * 32;
    return (uint32_t)(b == 0 ? 1 : (b > cap ? cap : b));
}

// The dashed outlines, in the work's dash buffers on the device.
struct DashResult {
    uint32_t P = 0, OC = 0;
    std::vector<uint32_t> ostarts;  // host copy of the output outline starts
    bool limited = false;
};

int32_t dash_run(StrokeWork* w, cudaStream_t s, const PFCUDAStrokeInput* in, const PFCUDADashInput* dash,
                 DashResult* r) {
    if (!w || !in || !dash) return PF_CUDA_ERR_INVALID;
    std::vector<uint32_t> hc, ho;
    const int32_t irc = read_index_arrays(in, hc, ho);
    if (irc != PF_CUDA_OK) return irc;
    const uint32_t NP = in->point_count, C = in->contour_count, O = in->outline_count;
    if (!dash->dash_starts || (O && !dash->offsets)) return PF_CUDA_ERR_INVALID;
    const bool dev_in = in->memory == PF_MEMORY_DEVICE;
    const cudaMemcpyKind down = dev_in ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost;
    std::vector<uint32_t> hd(O + 1);
    PF_STROKE_TRY(cudaMemcpy(hd.data(), dash->dash_starts, sizeof(uint32_t) * (O + 1), down));
    if (hd[0] != 0) return PF_CUDA_ERR_INVALID;
    for (uint32_t o = 0; o < O; o++)
        if (hd[o] > hd[o + 1]) return PF_CUDA_ERR_INVALID;
    const uint32_t ND = hd[O];
    if (ND >= 0x40000000u || (ND && !dash->dashes)) return PF_CUDA_ERR_INVALID;
    std::vector<float> hv(ND), hoff(O);
    if (ND) PF_STROKE_TRY(cudaMemcpy(hv.data(), dash->dashes, sizeof(float) * ND, down));
    if (O) PF_STROKE_TRY(cudaMemcpy(hoff.data(), dash->offsets, sizeof(float) * O, down));
    for (uint32_t o = 0; o < O; o++) {
        if (hd[o + 1] == hd[o]) continue;
        float total = 0.0f;
        for (uint32_t i = hd[o]; i < hd[o + 1]; i++) {
            if (!(hv[i] >= 0.0f) || !std::isfinite(hv[i])) return PF_CUDA_ERR_INVALID;
            total = total + hv[i];
        }
        if (!(total > 0.0f) || !std::isfinite(total) || !std::isfinite(hoff[o])) return PF_CUDA_ERR_INVALID;
    }
    std::vector<uint32_t> hop(O + 1);
    for (uint32_t o = 0; o <= O; o++) hop[o] = hc[ho[o]];

    PF_STROKE_TRY(w->d_cstarts.ensure(C + 1));
    PF_STROKE_TRY(w->d_ostarts.ensure(O + 1));
    PF_STROKE_TRY(w->d_opstarts.ensure(O + 1));
    PF_STROKE_TRY(w->d_dstarts.ensure(O + 1));
    PF_STROKE_TRY(w->d_dashes.ensure((size_t)ND + 1));
    PF_STROKE_TRY(w->d_offsets.ensure(O + 1));
    PF_STROKE_TRY(w->d_cnt_p.ensure(O + 1));
    PF_STROKE_TRY(w->d_cnt_c.ensure(O + 1));
    PF_STROKE_TRY(w->d_pbase.ensure(O + 1));
    PF_STROKE_TRY(w->d_cbase.ensure(O + 1));
    PF_STROKE_TRY(w->status.ensure(1));
    PF_STROKE_TRY(w->partials.ensure(2 * ((size_t)O / 2048 + 2)));  // two scan lanes
    DashDev d{};
    if (dev_in) {
        d.pts = (const float2*)in->points;
        d.pflags = in->point_flags;
        d.closed = in->contour_closed;
    } else {
        const cudaMemcpyKind up = cudaMemcpyHostToDevice;
        PF_STROKE_TRY(w->pts.ensure(NP + 1));
        PF_STROKE_TRY(w->pflags.ensure(NP + 1));
        PF_STROKE_TRY(w->closed.ensure(C + 1));
        if (NP) {
            PF_STROKE_TRY(cudaMemcpyAsync(w->pts.p, in->points, sizeof(float2) * NP, up, s));
            PF_STROKE_TRY(cudaMemcpyAsync(w->pflags.p, in->point_flags, NP, up, s));
        }
        if (C) PF_STROKE_TRY(cudaMemcpyAsync(w->closed.p, in->contour_closed, C, up, s));
        d.pts = w->pts.p;
        d.pflags = w->pflags.p;
        d.closed = w->closed.p;
    }
    PF_STROKE_TRY(cudaMemcpyAsync(w->d_cstarts.p, hc.data(), sizeof(uint32_t) * (C + 1), cudaMemcpyHostToDevice, s));
    PF_STROKE_TRY(cudaMemcpyAsync(w->d_ostarts.p, ho.data(), sizeof(uint32_t) * (O + 1), cudaMemcpyHostToDevice, s));
    PF_STROKE_TRY(cudaMemcpyAsync(w->d_opstarts.p, hop.data(), sizeof(uint32_t) * (O + 1), cudaMemcpyHostToDevice, s));
    PF_STROKE_TRY(cudaMemcpyAsync(w->d_dstarts.p, hd.data(), sizeof(uint32_t) * (O + 1), cudaMemcpyHostToDevice, s));
    if (ND) PF_STROKE_TRY(cudaMemcpyAsync(w->d_dashes.p, hv.data(), sizeof(float) * ND, cudaMemcpyHostToDevice, s));
    if (O) PF_STROKE_TRY(cudaMemcpyAsync(w->d_offsets.p, hoff.data(), sizeof(float) * O, cudaMemcpyHostToDevice, s));
    PF_STROKE_TRY(cudaMemsetAsync(w->status.p, 0, sizeof(uint32_t), s));
    d.cstarts = w->d_cstarts.p;
    d.ostarts = w->d_ostarts.p;
    d.opstarts = w->d_opstarts.p;
    d.dashes = w->d_dashes.p;
    d.dstarts = w->d_dstarts.p;
    d.offsets = w->d_offsets.p;
    d.O = O;
    d.C = C;
    d.cnt_pts = w->d_cnt_p.p;
    d.cnt_cont = w->d_cnt_c.p;
    d.pbase = w->d_pbase.p;
    d.cbase = w->d_cbase.p;
    d.status = w->status.p;
    ScanTemp tmp{w->partials.p, (uint32_t)w->partials.cap};

    if (O) { count_launch(); k_dash_count<<<walk_grid(O), 64, 0, s>>>(d); }
    ScanLanes lanes{};
    lanes.count = 2;
    lanes.in[0] = w->d_cnt_p.p; lanes.out[0] = w->d_pbase.p;
    lanes.in[1] = w->d_cnt_c.p; lanes.out[1] = w->d_cbase.p;
    launch_scan_multi(lanes, nullptr, O, tmp, s);
    uint32_t status = 0;
    r->ostarts.assign(O + 1, 0u);
    PF_STROKE_TRY(cudaMemcpyAsync(r->ostarts.data(), w->d_cbase.p, sizeof(uint32_t) * (O + 1),
                                  cudaMemcpyDeviceToHost, s));
    PF_STROKE_TRY(cudaMemcpyAsync(&r->P, w->d_pbase.p + O, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    PF_STROKE_TRY(cudaMemcpyAsync(&status, w->status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    PF_STROKE_TRY(cudaStreamSynchronize(s));
    PF_STROKE_TRY(cudaGetLastError());
    r->OC = r->ostarts[O];
    r->limited = (status & 1u) != 0;
    if (r->P >= 0x40000000u || r->OC >= 0x20000000u) return PF_CUDA_ERR_CAPACITY;
    PF_STROKE_TRY(w->dash_pts.ensure((size_t)r->P + 1));
    PF_STROKE_TRY(w->dash_flags.ensure((size_t)r->P + 1));
    PF_STROKE_TRY(w->dash_cstarts.ensure((size_t)r->OC + 1));
    PF_STROKE_TRY(w->dash_closed.ensure((size_t)r->OC + 1));
    d.out_pts = w->dash_pts.p;
    d.out_flags = w->dash_flags.p;
    d.out_cstarts = w->dash_cstarts.p;
    d.out_closed = w->dash_closed.p;
    if (O) { count_launch(); k_dash_emit<<<walk_grid(O), 64, 0, s>>>(d); }
    if (hop[O] > hop[0]) { count_launch(); k_dash_copy_points<<<grid_for(hop[O] - hop[0]), 256, 0, s>>>(d); }
    { count_launch(); k_dash_copy_contours<<<grid_for(C), 256, 0, s>>>(d, r->P); }
    PF_STROKE_TRY(cudaGetLastError());
    return PF_CUDA_OK;
}
}  // namespace

int32_t dash_outlines(StrokeWork* w, cudaStream_t s, const PFCUDAStrokeInput* in, const PFCUDADashInput* dash,
                      PFCUDAOutlineOutput* out) {
    if (!out || (out->memory != PF_MEMORY_HOST && out->memory != PF_MEMORY_DEVICE)) return PF_CUDA_ERR_INVALID;
    DashResult r;
    const int32_t rc = dash_run(w, s, in, dash, &r);
    if (rc != PF_CUDA_OK) return rc;
    const uint32_t O = in->outline_count;
    out->point_count = r.P;
    out->contour_count = r.OC;
    if (out->point_capacity < r.P || out->contour_capacity < r.OC) {
        PF_STROKE_TRY(cudaStreamSynchronize(s));
        return PF_CUDA_ERR_CAPACITY;
    }
    if ((r.P && (!out->points || !out->point_flags)) || !out->contour_starts || (r.OC && !out->contour_closed) ||
        !out->outline_starts) {
        PF_STROKE_TRY(cudaStreamSynchronize(s));
        return PF_CUDA_ERR_INVALID;
    }
    const cudaMemcpyKind k = out->memory == PF_MEMORY_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (r.P) {
        PF_STROKE_TRY(cudaMemcpyAsync(out->points, w->dash_pts.p, sizeof(float2) * r.P, k, s));
        PF_STROKE_TRY(cudaMemcpyAsync(out->point_flags, w->dash_flags.p, r.P, k, s));
    }
    PF_STROKE_TRY(cudaMemcpyAsync(out->contour_starts, w->dash_cstarts.p, sizeof(uint32_t) * (r.OC + 1), k, s));
    if (r.OC) PF_STROKE_TRY(cudaMemcpyAsync(out->contour_closed, w->dash_closed.p, r.OC, k, s));
    if (out->memory == PF_MEMORY_DEVICE)
        PF_STROKE_TRY(cudaMemcpyAsync(out->outline_starts, r.ostarts.data(), sizeof(uint32_t) * (O + 1),
                                      cudaMemcpyHostToDevice, s));
    else
        std::memcpy(out->outline_starts, r.ostarts.data(), sizeof(uint32_t) * (O + 1));
    PF_STROKE_TRY(cudaStreamSynchronize(s));
    PF_STROKE_TRY(cudaGetLastError());
    return r.limited ? PF_CUDA_ERR_LIMIT : PF_CUDA_OK;
}

int32_t stroke_dashed(StrokeWork* w, cudaStream_t s, const PFCUDAStrokeInput* in, const PFCUDADashInput* dash,
                      PFCUDAStrokeOutput* out) {
    if (!w || !in || !out || (in->outline_count && !in->styles)) return PF_CUDA_ERR_INVALID;
    DashResult r;
    const int32_t rc = dash_run(w, s, in, dash, &r);
    if (rc != PF_CUDA_OK) return rc;
    const uint32_t O = in->outline_count;
    PF_STROKE_TRY(w->dash_styles.ensure(O + 1));
    PF_STROKE_TRY(w->dash_ostarts.ensure(O + 1));
    const cudaMemcpyKind up = in->memory == PF_MEMORY_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (O) PF_STROKE_TRY(cudaMemcpyAsync(w->dash_styles.p, in->styles, sizeof(PFCUDAStrokeStyle) * O, up, s));
    PF_STROKE_TRY(cudaMemcpyAsync(w->dash_ostarts.p, r.ostarts.data(), sizeof(uint32_t) * (O + 1),
                                  cudaMemcpyHostToDevice, s));
    PF_STROKE_TRY(cudaStreamSynchronize(s));
    PFCUDAStrokeInput dashed{};
    dashed.points = (const PFVector2F*)w->dash_pts.p;
    dashed.point_flags = w->dash_flags.p;
    dashed.contour_starts = w->dash_cstarts.p;
    dashed.contour_closed = w->dash_closed.p;
    dashed.outline_starts = w->dash_ostarts.p;
    dashed.styles = w->dash_styles.p;
    dashed.point_count = r.P;
    dashed.contour_count = r.OC;
    dashed.outline_count = O;
    dashed.memory = PF_MEMORY_DEVICE;
    const int32_t src = stroke_run(w, s, &dashed, out);
    if (src != PF_CUDA_OK) return src;
    return r.limited ? PF_CUDA_ERR_LIMIT : PF_CUDA_OK;
}

}  // namespace pf

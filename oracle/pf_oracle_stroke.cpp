// pf_oracle_stroke.cpp — TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// CPU restatement of the reference's stroke-to-fill conversion,
// OutlineStrokeToFill (content/src/stroke.rs:24-465), with the geometry it
// uses: LineSegment2F offset / intersection_t / sample / split
// (geometry/src/line_segment.rs:91-251), Segment sample / split / reversed /
// to_cubic / arc_from_cos / quarter_circle_arc (content/src/segment.rs:52-380),
// UnitVector rotations (geometry/src/unit_vector.rs), Transform2F products
// (geometry/src/transform2d.rs), Contour::push_segment and
// push_arc_from_unit_chord (content/src/outline.rs:560-669) and ContourIter
// (outline.rs:1020-1065); and the dashing pass before it, OutlineDash
// (content/src/dash.rs:18-152).  Single precision in the reference's op
// order, built with -ffp-contract=off; the checker of the CUDA stroker and
// dasher.
#include "../include/pathfinder_cuda.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct V { float x, y; };
inline V vadd(V a, V b) { return V{a.x + b.x, a.y + b.y}; }
inline V vsub(V a, V b) { return V{a.x - b.x, a.y - b.y}; }
inline V vmul(V a, float s) { return V{a.x * s, a.y * s}; }
inline V vmulv(V a, V b) { return V{a.x * b.x, a.y * b.y}; }
inline bool veq(V a, V b) { return a.x == b.x && a.y == b.y; }
inline float vsqlen(V v) { return v.x * v.x + v.y * v.y; }
inline V vyx(V v) { return V{v.y, v.x}; }
inline V vnormalize(V v) { const float r = 1.0f / std::sqrt(vsqlen(v)); return vmul(v, r); }
inline V vlerp(V a, V b, float t) { return vadd(a, vmul(vsub(b, a), t)); }
inline float smax(float a, float b) { return a > b ? a : b; }  // _mm_max_ps lane

struct L { V f, t; };
inline V lvec(L l) { return vsub(l.t, l.f); }
inline V lsample(L l, float t) { return vadd(l.f, vmul(lvec(l), t)); }
inline L lreversed(L l) { return L{l.t, l.f}; }

// LineSegment2F::offset (geometry/src/line_segment.rs:241-247)
L loffset(L l, float d) {
    const V v = lvec(l);
    if (v.x == 0.0f && v.y == 0.0f) return l;
    const V o = vmulv(vnormalize(vyx(v)), V{-d, d});
    return L{vadd(l.f, o), vadd(l.t, o)};
}

// LineSegment2F::intersection_t (:219-228)
bool intersection_t(L self, L other, float* t) {
    const V p0p1 = lvec(self), ov = lvec(other);
    const float m11 = ov.x, m21 = ov.y, m12 = -p0p1.x, m22 = -p0p1.y;
    const float det = m11 * m22 - m12 * m21;
    if (std::fabs(det) < 0.0001f) return false;
    const float r = 1.0f / det;
    const float i21 = r * -m21, i22 = r * m11;
    const V v = vsub(self.f, other.f);
    *t = i21 * v.x + i22 * v.y;
    return true;
}

enum Kind { kNone = 0, kLine = 1, kQuad = 2, kCubic = 3 };
struct Seg { L base, ctrl; int kind; };

inline Seg seg_line(L l) { return Seg{l, L{{0, 0}, {0, 0}}, kLine}; }
inline Seg seg_quad(L b, V c) { return Seg{b, L{c, {0, 0}}, kQuad}; }
inline Seg seg_cubic(L b, L c) { return Seg{b, c, kCubic}; }

// Segment::to_cubic (content/src/segment.rs:171-182)
Seg to_cubic(const Seg& s) {
    if (s.kind == kCubic) return s;
    Seg c = s;
    const V p12 = vadd(s.ctrl.f, s.ctrl.f);
    const float third = 1.0f / 3.0f;
    c.ctrl = L{vmul(vadd(s.base.f, p12), third), vmul(vadd(p12, s.base.t), third)};
    c.kind = kCubic;
    return c;
}

// CubicSegment::split (:307-359)
void cubic_split(const Seg& s, float t, Seg* a, Seg* b) {
    if (t <= 0.0f) {
        *a = seg_cubic(L{s.base.f, s.base.f}, L{s.base.f, s.base.f});
        *b = seg_cubic(s.base, s.ctrl);
        return;
    }
    if (t >= 1.0f) {
        *a = seg_cubic(s.base, s.ctrl);
        *b = seg_cubic(L{s.base.t, s.base.t}, L{s.base.t, s.base.t});
        return;
    }
    const V p0 = s.base.f, p3 = s.base.t, p1 = s.ctrl.f, p2 = s.ctrl.t;
    const V p01 = vadd(p0, vmul(vsub(p1, p0), t)), p12 = vadd(p1, vmul(vsub(p2, p1), t));
    const V p23 = vadd(p2, vmul(vsub(p3, p2), t));
    const V p012 = vadd(p01, vmul(vsub(p12, p01), t)), p123 = vadd(p12, vmul(vsub(p23, p12), t));
    const V p0123 = vadd(p012, vmul(vsub(p123, p012), t));
    *a = seg_cubic(L{p0, p0123}, L{p01, p012});
    *b = seg_cubic(L{p0123, p3}, L{p123, p23});
}

// Segment::split (:211-219): lines split as lines, curves as cubics
void seg_split(const Seg& s, float t, Seg* a, Seg* b) {
    if (s.kind == kLine) {
        const V d = lvec(s.base), mid = vadd(s.base.f, vmul(d, t));
        *a = seg_line(L{s.base.f, mid});
        *b = seg_line(L{mid, s.base.t});
        return;
    }
    cubic_split(to_cubic(s), t, a, b);
}

// Segment::sample (:226-233)
V seg_sample(const Seg& s, float t) {
    if (s.kind == kLine) return lsample(s.base, t);
    Seg a, b;
    cubic_split(to_cubic(s), t, &a, &b);
    return a.base.t;
}

// Segment::reversed (:186-197)
Seg seg_reversed(const Seg& s) {
    Seg r = s;
    r.base = lreversed(s.base);
    if (s.kind != kQuad) r.ctrl = lreversed(s.ctrl);
    return r;
}

// Transform2F as (m11, m21, m12, m22) lanes and a vector.
struct T2 { float m[4]; V v; };
T2 t2_scale(float s) { return T2{{s, 0.0f, 0.0f, s}, {0.0f, 0.0f}}; }
T2 t2_rotation(V u) { return T2{{u.x, u.y, -u.y, u.x}, {0.0f, 0.0f}}; }
T2 t2_identity() { return T2{{1.0f, 0.0f, 0.0f, 1.0f}, {0.0f, 0.0f}}; }
V t2_apply_m(const float m[4], V p) {  // Matrix2x2F * Vector2F
    return V{m[0] * p.x + m[2] * p.y, m[1] * p.x + m[3] * p.y};
}
V t2_apply(const T2& t, V p) { return vadd(t2_apply_m(t.m, p), t.v); }
T2 t2_mul(const T2& a, const T2& b) {  // a * b (b first)
    T2 r;
    r.m[0] = a.m[0] * b.m[0] + a.m[2] * b.m[1];
    r.m[1] = a.m[1] * b.m[0] + a.m[3] * b.m[1];
    r.m[2] = a.m[0] * b.m[2] + a.m[2] * b.m[3];
    r.m[3] = a.m[1] * b.m[2] + a.m[3] * b.m[3];
    r.v = t2_apply(a, b.v);
    return r;
}
T2 t2_translate(const T2& t, V p) { T2 tr = t2_identity(); tr.v = p; return t2_mul(tr, t); }
Seg seg_transform(const Seg& s, const T2& t) {
    Seg r = s;
    r.base = L{t2_apply(t, s.base.f), t2_apply(t, s.base.t)};
    r.ctrl = L{t2_apply(t, s.ctrl.f), t2_apply(t, s.ctrl.t)};
    return r;
}

// UnitVector (geometry/src/unit_vector.rs)
V uv_rotate_by(V s, V o) { return V{s.x * o.x - s.y * o.y, s.y * o.x + s.x * o.y}; }
V uv_rev_rotate_by(V s, V o) { return V{s.x * o.x + s.y * o.y, s.y * o.x - s.x * o.y}; }
V uv_halve_angle(V s) {
    const float x = s.x;
    return V{std::sqrt(smax(0.5f * (1.0f + x), 0.0f)), std::sqrt(smax(0.5f * (1.0f + -x), 0.0f))};
}

// Segment::arc_from_cos / quarter_circle_arc (content/src/segment.rs:94-122)
Seg arc_from_cos(float c) {
    if (c >= 1.0f - 0.001f) return seg_line(L{{1.0f, 0.0f}, {1.0f, 0.0f}});
    const float a = std::sqrt((1.0f + c) * 0.5f), b = std::sqrt((1.0f + -c) * 0.5f);
    const V p3{a * 1.0f, b * -1.0f}, p0{a * 1.0f, b * 1.0f};
    const float p1x = 4.0f - p0.x, p1y = (1.0f - p0.x) * (3.0f - p0.x) / p0.y;
    const float third = 1.0f / 3.0f;
    const V p2{p1x * third, -p1y * third}, p1{p1x * third, p1y * third};
    return seg_cubic(L{p3, p0}, L{p2, p1});
}
Seg quarter_circle_arc() {
    const float sqrt2 = 1.41421356237309504880f;
    const V p0{sqrt2 * 0.5f, sqrt2 * 0.5f};
    const V p1{-sqrt2 / 6.0f + 4.0f / 3.0f, 7.0f * sqrt2 / 6.0f - 4.0f / 3.0f};
    const V p2{p1.x * 1.0f, p1.y * -1.0f}, p3{p0.x * 1.0f, p0.y * -1.0f};
    return seg_cubic(L{p3, p0}, L{p2, p1});
}

// Contour under construction (points + flags; Contour::push_point, outline.rs:560-573).
struct OutContour {
    std::vector<V> pts;
    std::vector<uint8_t> flags;
    uint32_t len() const { return (uint32_t)pts.size(); }
    V last(uint32_t k) const { return pts[pts.size() - k]; }  // position_of_last
    void push(V p, uint8_t f) { pts.push_back(p); flags.push_back(f); }
    // Contour::push_segment (outline.rs:576-600): the from point always
    void push_segment(const Seg& s) {
        if (s.kind == kNone) return;
        push(s.base.f, 0);
        if (s.kind != kLine) {
            push(s.ctrl.f, PF_POINT_FLAG_CONTROL_POINT_0);
            if (s.kind != kQuad) push(s.ctrl.t, PF_POINT_FLAG_CONTROL_POINT_1);
        }
        push(s.base.t, 0);
    }
    // push_arc_from_unit_chord, clockwise (outline.rs:630-669)
    void push_arc_from_unit_chord(const T2& transform, L chord) {
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
            const T2 rotation = t2_rotation(uv_rotate_by(half, vector));
            seg = seg_transform(seg, t2_mul(t2_mul(transform, dir), rotation));
            push_segment(seg);
            if (last) break;
            vector = uv_rotate_by(vector, sweep);
        }
    }
};

struct Style { float width; int cap, join; float miter; };
const float kTolerance = 0.01f;     // content/src/stroke.rs:22
const float kEpsilon = 0.001f;      // geometry/src/util.rs:15

bool might_need_join(const OutContour& c, int join) {
    return c.len() >= 2 && (join == PF_LINE_JOIN_MITER || join == PF_LINE_JOIN_ROUND);
}

// Contour::add_join (content/src/stroke.rs:412-448)
void add_join(OutContour& c, float distance, int join, float miter_limit, V join_point, L next_tangent) {
    const V p0 = c.last(2), p1 = c.last(1);
    const L prev_tangent{p0, p1};
    if (vsqlen(lvec(prev_tangent)) < kEpsilon || vsqlen(lvec(next_tangent)) < kEpsilon) return;
    if (join == PF_LINE_JOIN_MITER) {
        float t;
        if (intersection_t(prev_tangent, next_tangent, &t)) {
            if (t < -kEpsilon) return;
            const V miter_endpoint = lsample(prev_tangent, t);
            const float threshold = miter_limit * distance;
            if (vsqlen(vsub(miter_endpoint, join_point)) > threshold * threshold) return;
            c.push(miter_endpoint, 0);
        }
    } else if (join == PF_LINE_JOIN_ROUND) {
        // a chord end at the join point has no direction: the reference would
        // push NaN points (normalising a zero vector); no join is pushed here
        const V cf = vsub(prev_tangent.t, join_point), ct = vsub(next_tangent.t, join_point);
        if ((cf.x == 0.0f && cf.y == 0.0f) || (ct.x == 0.0f && ct.y == 0.0f)) return;
        const float scale = std::fabs(distance);
        const T2 transform = t2_translate(t2_scale(scale), join_point);
        c.push_arc_from_unit_chord(transform, L{vnormalize(cf), vnormalize(ct)});
    }
}

// Offset::offset_once (:281-362)
Seg offset_once(const Seg& s, float d) {
    if (s.kind == kLine) return seg_line(loffset(s.base, d));
    auto ctrl_of = [](L a, L b) {
        float t;
        return intersection_t(a, b, &t) ? lsample(a, t) : vlerp(a.t, b.f, 0.5f);
    };
    if (s.kind == kQuad) {
        const L s0 = loffset(L{s.base.f, s.ctrl.f}, d), s1 = loffset(L{s.ctrl.f, s.base.t}, d);
        return seg_quad(L{s0.f, s1.t}, ctrl_of(s0, s1));
    }
    if (veq(s.base.f, s.ctrl.f)) {
        const L s0 = loffset(L{s.base.f, s.ctrl.t}, d), s1 = loffset(L{s.ctrl.t, s.base.t}, d);
        return seg_cubic(L{s0.f, s1.t}, L{s0.f, ctrl_of(s0, s1)});
    }
    if (veq(s.ctrl.t, s.base.t)) {
        const L s0 = loffset(L{s.base.f, s.ctrl.f}, d), s1 = loffset(L{s.ctrl.f, s.base.t}, d);
        return seg_cubic(L{s0.f, s1.t}, L{ctrl_of(s0, s1), s1.t});
    }
    const L s0 = loffset(L{s.base.f, s.ctrl.f}, d), s1 = loffset(L{s.ctrl.f, s.ctrl.t}, d);
    const L s2 = loffset(L{s.ctrl.t, s.base.t}, d);
    float t0, t1;
    const bool h0 = intersection_t(s0, s1, &t0), h1 = intersection_t(s1, s2, &t1);
    V c0, c1;
    if (h0 && h1) { c0 = lsample(s0, t0); c1 = lsample(s1, t1); }
    else { c0 = vlerp(s0.t, s1.f, 0.5f); c1 = vlerp(s1.t, s2.f, 0.5f); }
    return seg_cubic(L{s0.f, s2.t}, L{c0, c1});
}

// Offset::error_is_within_tolerance (:364-391), 17 samples
bool error_within_tolerance(const Seg& self, const Seg& other, float distance) {
    float mn = std::fabs(distance) - kTolerance, mx = std::fabs(distance) + kTolerance;
    mn = mn <= 0.0f ? 0.0f : mn * mn;
    mx = mx <= 0.0f ? 0.0f : mx * mx;
    for (uint32_t n = 0; n <= 16; n++) {
        const float t = (float)n / (float)16;
        const float sq = vsqlen(vsub(seg_sample(self, t), seg_sample(other, t)));
        if (sq < mn || sq > mx) return false;
    }
    return true;
}

struct Stroker { Style st; OutContour out; bool depth_limit = false; uint32_t pieces = 0; };
const uint32_t kMaxStrokePieces = 1u << 16;  // per segment, as the CUDA stroker bounds it

// Offset::add_to_contour (:256-279)
void add_to_contour(Stroker& k, const Seg& s, float distance, int join, V join_point) {
    if (might_need_join(k.out, join)) {
        const V p3 = s.base.f, p4 = s.kind == kLine ? s.base.t : s.ctrl.f;
        add_join(k.out, distance, join, k.st.miter, join_point, L{p4, p3});
    }
    k.out.push_segment(s);
}

// Offset::offset (:238-254), with the recursion bounded at depth 32 as the
// CUDA stroker bounds it (the reference recurses without bound).
// Returns false once the segment's piece budget is spent (the walk stops).
bool offset_segment(Stroker& k, const Seg& s, float distance, int join, int depth) {
    const V join_point = s.base.f;
    if (vsqlen(lvec(s.base)) < kTolerance * kTolerance) {
        add_to_contour(k, s, distance, join, join_point);
        if (++k.pieces >= kMaxStrokePieces) { k.depth_limit = true; return false; }
        return true;
    }
    const Seg cand = offset_once(s, distance);
    if (error_within_tolerance(s, cand, distance) || depth >= 32) {
        if (depth >= 32 && !error_within_tolerance(s, cand, distance)) k.depth_limit = true;
        add_to_contour(k, cand, distance, join, join_point);
        if (++k.pieces >= kMaxStrokePieces) { k.depth_limit = true; return false; }
        return true;
    }
    Seg a, b;
    seg_split(s, 0.5f, &a, &b);
    if (!offset_segment(k, a, distance, join, depth + 1)) return false;
    return offset_segment(k, b, distance, join, depth + 1);
}

// ContourIter (content/src/outline.rs:1020-1065) with ContourIterFlags::empty()
std::vector<Seg> contour_segments(const PFVector2F* pts, const uint8_t* flags, uint32_t n, bool closed) {
    std::vector<Seg> out;
    // indices past the end (a contour ending on a control point; the reference
    // would read out of bounds) clamp to the last point, as the CUDA stroker does
    auto P = [&](uint32_t i) { const uint32_t j = i < n ? i : n - 1; return V{pts[j].x, pts[j].y}; };
    auto is_end = [&](uint32_t i) {
        return (flags[i] & (PF_POINT_FLAG_CONTROL_POINT_0 | PF_POINT_FLAG_CONTROL_POINT_1)) == 0;
    };
    uint32_t index = 1;
    while (n != 0 && index <= n && !(index == n && !closed)) {
        const V p0 = P(index - 1);
        if (index == n) { index++; out.push_back(seg_line(L{p0, P(0)})); continue; }
        const uint32_t i1 = index++;
        if (is_end(i1)) { out.push_back(seg_line(L{p0, P(i1)})); continue; }
        const uint32_t i2 = index++;
        if (i2 >= n || is_end(i2)) { out.push_back(seg_quad(L{p0, P(i2)}, P(i1))); continue; }
        const uint32_t i3 = index++;
        out.push_back(seg_cubic(L{p0, P(i3)}, L{P(i1), P(i2)}));
    }
    return out;
}

// OutlineStrokeToFill::add_cap (content/src/stroke.rs:151-199)
void add_cap(Stroker& k) {
    OutContour& c = k.out;
    if (k.st.cap == PF_LINE_CAP_BUTT || c.len() < 2) return;
    const float width = k.st.width;
    const V p1 = c.last(1);
    V p0;
    uint32_t p0_index = c.len() - 2;
    for (;;) {
        p0 = c.pts[p0_index];
        if (vsqlen(vsub(p1, p0)) > kEpsilon) break;
        if (p0_index == 0) return;
        p0_index--;
    }
    const V gradient = vnormalize(vsub(p1, p0));
    if (k.st.cap == PF_LINE_CAP_SQUARE) {
        const V offset = vmul(gradient, width * 0.5f);
        const V p2 = vadd(p1, offset);
        const V p3 = vadd(p2, vmulv(vyx(gradient), V{-width, width}));
        const V p4 = vsub(p3, offset);
        c.push(p2, 0);
        c.push(p3, 0);
        c.push(p4, 0);
    } else {
        const float scale = width * 0.5f;
        const V offset = vmulv(vyx(gradient), V{-1.0f, 1.0f});
        const V translation = vadd(p1, vmul(offset, width * 0.5f));
        const T2 transform = t2_translate(t2_scale(scale), translation);
        c.push_arc_from_unit_chord(transform, L{vmul(offset, -1.0f), offset});
    }
}

}  // namespace

// OutlineStrokeToFill::offset + push_stroked_contour (content/src/stroke.rs:88-149)
// over a batch of outlines.
struct StrokeResult {
    std::vector<PFVector2F> pts;
    std::vector<uint8_t> flags;
    std::vector<uint32_t> contour_starts{0};
    std::vector<uint32_t> outline_starts{0};
    bool depth_limit = false;
};

namespace {

void push_stroked_contour(StrokeResult& r, Stroker& k, bool closed, V input_first) {
    if (closed && might_need_join(k.out, k.st.join)) {
        const V p1 = k.out.pts[1], p0 = k.out.pts[0];
        add_join(k.out, k.st.width * 0.5f, k.st.join, k.st.miter, input_first, L{p1, p0});
    }
    for (uint32_t i = 0; i < k.out.len(); i++) {
        r.pts.push_back(PFVector2F{k.out.pts[i].x, k.out.pts[i].y});
        r.flags.push_back(k.out.flags[i]);
    }
    r.contour_starts.push_back((uint32_t)r.pts.size());
    r.depth_limit = r.depth_limit || k.depth_limit;
    k.out = OutContour();
}

void stroke_contour(StrokeResult& r, const Style& st, const PFVector2F* pts, const uint8_t* flags, uint32_t n,
                    bool closed) {
    const std::vector<Seg> segs = contour_segments(pts, flags, n, closed);
    const float radius = st.width * 0.5f;
    const V first = n ? V{pts[0].x, pts[0].y} : V{0.0f, 0.0f};
    Stroker k;
    k.st = st;
    // offset_forward (:208-215): the first segment joins with Bevel
    for (size_t i = 0; i < segs.size(); i++) {
        k.pieces = 0;
        offset_segment(k, segs[i], -radius, i == 0 ? PF_LINE_JOIN_BEVEL : st.join, 0);
    }
    if (closed) push_stroked_contour(r, k, true, first);
    else add_cap(k);
    // offset_backward (:217-230): reversed segments in reverse order
    for (size_t i = 0; i < segs.size(); i++) {
        k.pieces = 0;
        offset_segment(k, seg_reversed(segs[segs.size() - 1 - i]), -radius, i == 0 ? PF_LINE_JOIN_BEVEL : st.join, 0);
    }
    if (!closed) add_cap(k);
    push_stroked_contour(r, k, closed, first);
}

// ---- OutlineDash (content/src/dash.rs:18-152) --------------------------------
constexpr float kDashEpsilon = 0.0001f;       // dash.rs:16
constexpr uint32_t kMaxDashSteps = 1u << 20;  // the CUDA library's step bound per outline

struct DashResult {
    std::vector<PFVector2F> pts;
    std::vector<uint8_t> flags;
    std::vector<uint32_t> contour_starts{0};
    std::vector<uint8_t> closed;
    std::vector<uint32_t> outline_starts{0};
    bool limited = false;
};

// Contour::push_segment (content/src/outline.rs:576-600) onto the open dash contour
void push_dash_segment(std::vector<PFVector2F>& c, std::vector<uint8_t>& f, const Seg& s) {
    c.push_back(PFVector2F{s.base.f.x, s.base.f.y});
    f.push_back(0);
    if (s.kind != kLine) {
        c.push_back(PFVector2F{s.ctrl.f.x, s.ctrl.f.y});
        f.push_back(PF_POINT_FLAG_CONTROL_POINT_0);
        if (s.kind != kQuad) {
            c.push_back(PFVector2F{s.ctrl.t.x, s.ctrl.t.y});
            f.push_back(PF_POINT_FLAG_CONTROL_POINT_1);
        }
    }
    c.push_back(PFVector2F{s.base.t.x, s.base.t.y});
    f.push_back(0);
}

// OutlineDash::new + dash + into_outline for one outline: DashState::new
// (:124-145), ContourDash::dash (:73-113), is_on (:147-150), into_outline
// (:52-57); arc_length and time_for_distance are the chord's
// (content/src/segment.rs:246-254).
void dash_outline(DashResult& r, const PFCUDAStrokeInput* in, uint32_t o, const float* dashes, uint32_t nd,
                  float offset0) {
    std::vector<PFVector2F> cur_pts;
    std::vector<uint8_t> cur_flags;
    auto push_contour = [&]() {  // Outline::push_contour drops an empty contour (outline.rs:180-192)
        if (cur_pts.empty()) return;
        r.pts.insert(r.pts.end(), cur_pts.begin(), cur_pts.end());
        r.flags.insert(r.flags.end(), cur_flags.begin(), cur_flags.end());
        r.contour_starts.push_back((uint32_t)r.pts.size());
        r.closed.push_back(0);
        cur_pts.clear();
        cur_flags.clear();
    };
    float total = 0.0f;
    for (uint32_t i = 0; i < nd; i++) total += dashes[i];
    float offset = std::fmod(offset0, total);
    uint32_t idx = 0;
    while (idx < nd) {
        if (offset < dashes[idx]) break;
        offset -= dashes[idx];
        idx++;
    }
    float left = offset;
    uint32_t steps = 0;
    bool limited = false;
    for (uint32_t c = in->outline_starts[o]; c < in->outline_starts[o + 1] && !limited; c++) {
        const uint32_t a = in->contour_starts[c], b = in->contour_starts[c + 1];
        const std::vector<Seg> segs = contour_segments(in->points + a, in->point_flags + a, b - a,
                                                       in->contour_closed[c] != 0);
        size_t next = 0;
        Seg queued{};
        bool have = false;
        for (;;) {
            if (!have) {
                if (next == segs.size()) break;
                queued = segs[next++];
            }
            if (steps++ == kMaxDashSteps) { limited = true; break; }
            Seg cur = queued;
            have = false;
            float distance = left;
            const float t = distance / std::sqrt(vsqlen(lvec(cur.base)));
            if (t < 1.0f) {
                Seg a0, b0;
                seg_split(cur, t, &a0, &b0);
                cur = a0;
                queued = b0;
                have = true;
            } else {
                distance = std::sqrt(vsqlen(lvec(cur.base)));
            }
            const bool on = idx % 2 == 0;
            if (on) push_dash_segment(cur_pts, cur_flags, cur);
            left -= distance;
            if (left < kDashEpsilon) {
                if (on) push_contour();
                idx++;
                if (idx >= nd) idx = 0;  // the reference compares with ==; >= also wraps an offset past the end
                left = dashes[idx];
            }
        }
    }
    if (idx % 2 == 0) push_contour();
    r.limited = r.limited || limited;
}

}  // namespace

extern "C" {

// Dashes every outline of `in` (host memory) with the patterns of `dash`
// (an outline with an empty pattern is copied); returns a handle, or NULL for
// invalid input.
void* pfo_dash(const PFCUDAStrokeInput* in, const PFCUDADashInput* dash) {
    if (!in || !dash || in->memory != PF_MEMORY_HOST || !dash->dash_starts) return nullptr;
    if (in->outline_count && (!in->outline_starts || !dash->offsets)) return nullptr;
    if (in->contour_count && (!in->contour_starts || !in->contour_closed)) return nullptr;
    if (in->point_count && (!in->points || !in->point_flags)) return nullptr;
    DashResult* r = new DashResult();
    for (uint32_t o = 0; o < in->outline_count; o++) {
        const uint32_t c0 = in->outline_starts[o], c1 = in->outline_starts[o + 1];
        const uint32_t d0 = dash->dash_starts[o], d1 = dash->dash_starts[o + 1];
        if (c0 > c1 || c1 > in->contour_count || d0 > d1) { delete r; return nullptr; }
        for (uint32_t c = c0; c < c1; c++) {
            const uint32_t a = in->contour_starts[c], b = in->contour_starts[c + 1];
            if (a > b || b > in->point_count) { delete r; return nullptr; }
        }
        if (d0 == d1) {
            for (uint32_t c = c0; c < c1; c++) {
                const uint32_t a = in->contour_starts[c], b = in->contour_starts[c + 1];
                r->pts.insert(r->pts.end(), in->points + a, in->points + b);
                r->flags.insert(r->flags.end(), in->point_flags + a, in->point_flags + b);
                r->contour_starts.push_back((uint32_t)r->pts.size());
                r->closed.push_back(in->contour_closed[c] != 0 ? 1 : 0);
            }
        } else {
            dash_outline(*r, in, o, dash->dashes + d0, d1 - d0, dash->offsets[o]);
        }
        r->outline_starts.push_back((uint32_t)(r->contour_starts.size() - 1));
    }
    return r;
}

void pfo_dash_counts(void* h, uint64_t* out3) {
    const DashResult* r = (const DashResult*)h;
    out3[0] = r->pts.size();
    out3[1] = r->contour_starts.size() - 1;
    out3[2] = r->limited ? 1 : 0;
}

void pfo_dash_read(void* h, PFVector2F* pts, uint8_t* flags, uint32_t* contour_starts, uint8_t* closed,
                   uint32_t* outline_starts) {
    const DashResult* r = (const DashResult*)h;
    if (pts && !r->pts.empty()) std::memcpy(pts, r->pts.data(), r->pts.size() * sizeof(PFVector2F));
    if (flags && !r->flags.empty()) std::memcpy(flags, r->flags.data(), r->flags.size());
    if (contour_starts) std::memcpy(contour_starts, r->contour_starts.data(), r->contour_starts.size() * 4);
    if (closed && !r->closed.empty()) std::memcpy(closed, r->closed.data(), r->closed.size());
    if (outline_starts) std::memcpy(outline_starts, r->outline_starts.data(), r->outline_starts.size() * 4);
}

void pfo_dash_free(void* h) { delete (DashResult*)h; }

// Strokes every outline of `in` (host memory); returns a handle, or NULL for
// invalid input.
void* pfo_stroke(const PFCUDAStrokeInput* in) {
    if (!in || in->memory != PF_MEMORY_HOST) return nullptr;
    if (in->outline_count && (!in->outline_starts || !in->styles)) return nullptr;
    if (in->contour_count && (!in->contour_starts || !in->contour_closed)) return nullptr;
    if (in->point_count && (!in->points || !in->point_flags)) return nullptr;
    StrokeResult* r = new StrokeResult();
    for (uint32_t o = 0; o < in->outline_count; o++) {
        const PFCUDAStrokeStyle& s = in->styles[o];
        if (!(s.line_width >= 0.0f) || s.line_cap < 0 || s.line_cap > 2 || s.line_join < 0 || s.line_join > 2) {
            delete r;
            return nullptr;
        }
        const Style st{s.line_width, s.line_cap, s.line_join, s.miter_limit};
        const uint32_t c0 = in->outline_starts[o], c1 = in->outline_starts[o + 1];
        if (c0 > c1 || c1 > in->contour_count) { delete r; return nullptr; }
        for (uint32_t c = c0; c < c1; c++) {
            const uint32_t a = in->contour_starts[c], b = in->contour_starts[c + 1];
            if (a > b || b > in->point_count) { delete r; return nullptr; }
            stroke_contour(*r, st, in->points + a, in->point_flags + a, b - a, in->contour_closed[c] != 0);
        }
        r->outline_starts.push_back((uint32_t)(r->contour_starts.size() - 1));
    }
    return r;
}

void pfo_stroke_counts(void* h, uint64_t* out3) {
    const StrokeResult* r = (const StrokeResult*)h;
    out3[0] = r->pts.size();
    out3[1] = r->contour_starts.size() - 1;
    out3[2] = r->depth_limit ? 1 : 0;
}

void pfo_stroke_read(void* h, PFVector2F* pts, uint8_t* flags, uint32_t* contour_starts, uint32_t* outline_starts) {
    const StrokeResult* r = (const StrokeResult*)h;
    if (pts && !r->pts.empty()) std::memcpy(pts, r->pts.data(), r->pts.size() * sizeof(PFVector2F));
    if (flags && !r->flags.empty()) std::memcpy(flags, r->flags.data(), r->flags.size());
    if (contour_starts) std::memcpy(contour_starts, r->contour_starts.data(), r->contour_starts.size() * 4);
    if (outline_starts) std::memcpy(outline_starts, r->outline_starts.data(), r->outline_starts.size() * 4);
}

void pfo_stroke_free(void* h) { delete (StrokeResult*)h; }

}  // extern "C"

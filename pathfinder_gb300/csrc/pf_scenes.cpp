// pf_scenes.cpp — seeded synthetic scenes (host code).
//
// Builds outlines the way the reference's front-ends do through
// Contour::push_endpoint / push_quadratic / push_cubic + close
// (content/src/outline.rs:531-557): one point per on-curve position, control
// points flagged CONTROL_POINT_0 / CONTROL_POINT_1.

#include "../../include/pathfinder_cuda_scenes.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

namespace {

const double kPi = 3.14159265358979323846;

// Deterministic transforms of mt19937_64 output (independent of the C++
// library's distribution implementations).
struct Rng {
    std::mt19937_64 g;
    explicit Rng(uint64_t seed) : g(seed) {}
    double uniform() { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
    int64_t integer(int64_t lo, int64_t hi) {  // inclusive
        return lo + (int64_t)(uniform() * (double)(hi - lo + 1));
    }
    double normal() {  // Box-Muller
        double u1 = uniform(), u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * kPi * u2);
    }
};

struct Builder {
    std::vector<PFVector2F> points;
    std::vector<uint8_t> flags;
    std::vector<uint32_t> contour_starts{0};
    std::vector<PFCUDAPath> clip_paths, draw_paths;
    std::vector<PFRectI> cells;

    void begin_contour(double x, double y) { push(x, y, 0); }
    void line_to(double x, double y) { push(x, y, 0); }
    void quad_to(double cx, double cy, double x, double y) {
        push(cx, cy, PF_POINT_FLAG_CONTROL_POINT_0);
        push(x, y, 0);
    }
    void cubic_to(double c0x, double c0y, double c1x, double c1y, double x, double y) {
        push(c0x, c0y, PF_POINT_FLAG_CONTROL_POINT_0);
        push(c1x, c1y, PF_POINT_FLAG_CONTROL_POINT_1);
        push(x, y, 0);
    }
    void end_contour() { contour_starts.push_back((uint32_t)points.size()); }
    uint32_t contour_count() const { return (uint32_t)contour_starts.size() - 1; }
    void push(double x, double y, uint8_t f) {
        points.push_back(PFVector2F{(float)x, (float)y});
        flags.push_back(f);
    }
};

PFCUDAPath make_path(uint32_t first_contour, uint32_t count, PFColorU paint, int32_t clip, uint8_t rule) {
    PFCUDAPath p;
    p.first_contour = first_contour;
    p.contour_count = count;
    p.paint = paint;
    p.clip_path = clip;
    p.fill_rule = rule;
    p.blend_mode = PF_BLEND_MODE_SRC_OVER;
    p.overlay = 0;
    return p;
}

// A closed star-like contour around (cx, cy): k vertices at alternating /
// jittered radii, each edge a line, quadratic or cubic with control points
// placed near the edge and jittered.
void star_contour(Builder& b, Rng& r, double cx, double cy, double r_out, double r_in, int k,
                  double p_line, double p_quad, double lo, double hi, bool reverse) {
    std::vector<double> vx(k), vy(k);
    double phase = r.uniform(0.0, 2.0 * kPi);
    for (int i = 0; i < k; i++) {
        double a = phase + 2.0 * kPi * i / k * (reverse ? -1.0 : 1.0);
        double rad = (i % 2 == 0) ? r_out : r_in;
        vx[i] = std::min(hi, std::max(lo, cx + rad * std::cos(a)));
        vy[i] = std::min(hi, std::max(lo, cy + rad * std::sin(a)));
    }
    auto clampc = [&](double v) { return std::min(hi, std::max(lo, v)); };
    double jit = 0.25 * r_out * 2.0 * kPi / k;
    b.begin_contour(vx[0], vy[0]);
    for (int i = 0; i < k; i++) {
        int j = (i + 1) % k;
        double ax = vx[i], ay = vy[i], bx = vx[j], by = vy[j];
        double u = r.uniform();
        if (u < p_line) {
            if (j != 0) b.line_to(bx, by);
            else b.line_to(vx[0], vy[0]);
        } else if (u < p_line + p_quad) {
            double mx = 0.5 * (ax + bx) + jit * r.normal(), my = 0.5 * (ay + by) + jit * r.normal();
            b.quad_to(clampc(mx), clampc(my), bx, by);
        } else {
            double c0x = ax + (bx - ax) / 3.0 + jit * r.normal(), c0y = ay + (by - ay) / 3.0 + jit * r.normal();
            double c1x = ax + 2.0 * (bx - ax) / 3.0 + jit * r.normal(), c1y = ay + 2.0 * (by - ay) / 3.0 + jit * r.normal();
            b.cubic_to(clampc(c0x), clampc(c0y), clampc(c1x), clampc(c1y), bx, by);
        }
    }
    b.end_contour();
}

void gen_stars_512(Builder& b, Rng& r, double scale, int W, int H) {
    int n = std::max(1, (int)std::lround(64 * scale));
    for (int p = 0; p < n; p++) {
        double cx = r.uniform(0, W), cy = r.uniform(0, H);
        double ro = r.uniform(16.0, 160.0), ri = ro * r.uniform(0.3, 0.7);
        int k = (int)r.integer(8, 32);
        uint32_t c0 = b.contour_count();
        // 50% quadratic, 50% cubic edges; all points inside the viewport.
        star_contour(b, r, cx, cy, ro, ri, k, 0.0, 0.5, 0.0, (double)std::min(W, H), false);
        PFColorU paint{(uint8_t)r.integer(0, 255), (uint8_t)r.integer(0, 255), (uint8_t)r.integer(0, 255), 255};
        b.draw_paths.push_back(make_path(c0, 1, paint, -1, PF_FILL_RULE_WINDING));
    }
}

void gen_svg_4k(Builder& b, Rng& r, double scale, int W, int H) {
    int n = std::max(1, (int)std::lround(20000 * scale));
    for (int p = 0; p < n; p++) {
        double cx = r.uniform(0, W), cy = r.uniform(0, H);
        double radius = 20.0 * std::exp(r.normal());  // log-normal, median 20 px, sigma 1
        int k = (int)r.integer(70, 140);               // ~105 segments per path
        double ri = radius * r.uniform(0.5, 0.95);
        uint32_t c0 = b.contour_count();
        star_contour(b, r, cx, cy, radius, ri, k, 0.4, 0.3, -4096.0, 8192.0, false);
        uint8_t rule = r.uniform() < 0.3 ? PF_FILL_RULE_EVEN_ODD : PF_FILL_RULE_WINDING;
        uint8_t alpha = 255;
        if (r.uniform() < 0.5) alpha = (uint8_t)std::lround(255.0 * r.uniform(0.2, 1.0));
        PFColorU paint{(uint8_t)r.integer(0, 255), (uint8_t)r.integer(0, 255), (uint8_t)r.integer(0, 255), alpha};
        int32_t clip = -1;
        if (r.uniform() < 0.1) {
            // A random axis-aligned rect clip path around the path's centre.
            double hw = radius * r.uniform(0.3, 1.2), hh = radius * r.uniform(0.3, 1.2);
            double ox = cx + radius * r.uniform(-0.5, 0.5), oy = cy + radius * r.uniform(-0.5, 0.5);
            uint32_t cc = b.contour_count();
            b.begin_contour(ox - hw, oy - hh);
            b.line_to(ox + hw, oy - hh);
            b.line_to(ox + hw, oy + hh);
            b.line_to(ox - hw, oy + hh);
            b.end_contour();
            clip = (int32_t)b.clip_paths.size();
            b.clip_paths.push_back(make_path(cc, 1, PFColorU{0, 0, 0, 0}, -1, PF_FILL_RULE_WINDING));
        }
        b.draw_paths.push_back(make_path(c0, 1, paint, clip, rule));
    }
}

// Perturbed ellipse or rounded rect of quadratic segments inside a box.
void glyph_contour(Builder& b, Rng& r, double x0, double y0, double x1, double y1, int nseg, bool hole) {
    double cx = 0.5 * (x0 + x1), cy = 0.5 * (y0 + y1);
    double rx = 0.5 * (x1 - x0), ry = 0.5 * (y1 - y0);
    bool rect = r.uniform() < 0.5;
    std::vector<double> px(nseg), py(nseg);
    double phase = r.uniform(0.0, 2.0 * kPi);
    for (int i = 0; i < nseg; i++) {
        double a = phase + 2.0 * kPi * i / nseg * (hole ? -1.0 : 1.0);
        double c = std::cos(a), s = std::sin(a);
        double rr = 1.0 + 0.08 * r.normal();
        rr = std::min(1.0, std::max(0.6, rr));
        if (rect) {  // superellipse ~ rounded rect
            double e = 0.25;
            c = (c < 0 ? -1 : 1) * std::pow(std::fabs(c), e);
            s = (s < 0 ? -1 : 1) * std::pow(std::fabs(s), e);
        }
        px[i] = cx + rx * rr * c;
        py[i] = cy + ry * rr * s;
    }
    b.begin_contour(px[0], py[0]);
    for (int i = 0; i < nseg; i++) {
        int j = (i + 1) % nseg;
        double mx = 0.5 * (px[i] + px[j]), my = 0.5 * (py[i] + py[j]);
        // push the control point outward a little
        double ox = mx - cx, oy = my - cy;
        mx += 0.05 * ox; my += 0.05 * oy;
        mx = std::min(x1, std::max(x0, mx)); my = std::min(y1, std::max(y0, my));
        b.quad_to(mx, my, px[j], py[j]);
    }
    b.end_contour();
}

void gen_glyph_atlas(Builder& b, Rng& r, double scale, int W, int H) {
    int n = std::max(1, (int)std::lround(16384 * scale));
    struct G { double em; int w, h; };
    std::vector<G> gs(n);
    for (int i = 0; i < n; i++) {
        double em = r.uniform(8.0, 128.0);
        // ink box of 0.34 em per side so that 16,384 glyphs fit one 4096^2 atlas
        int side = std::max(3, (int)std::ceil(0.34 * em)) + 2;  // + 1 px padding each side
        gs[i] = G{em, side, side};
    }
    // Shelf packing, tallest first (glyph order itself is unchanged).
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return gs[a].h > gs[c].h; });
    int x = 0, y = 0, shelf_h = 0;
    b.cells.resize(n);
    for (int oi = 0; oi < n; oi++) {
        int i = order[oi];
        if (x + gs[i].w > W) { x = 0; y += shelf_h; shelf_h = 0; }
        if (y + gs[i].h > H) y = 0;  // atlas full: only reachable for scales above 1
        b.cells[i] = PFRectI{{x, y}, {x + gs[i].w, y + gs[i].h}};
        x += gs[i].w;
        shelf_h = std::max(shelf_h, gs[i].h);
    }
    for (int i = 0; i < n; i++) {
        const PFRectI& c = b.cells[i];
        double x0 = c.origin.x + 1.0, y0 = c.origin.y + 1.0;
        double x1 = c.lower_right.x - 1.0, y1 = c.lower_right.y - 1.0;
        int ncont = (int)r.integer(1, 4);
        uint32_t c0 = b.contour_count();
        glyph_contour(b, r, x0, y0, x1, y1, (int)r.integer(10, 60), false);
        for (int k = 1; k < ncont; k++) {
            // holes: smaller boxes inside the outer contour, opposite winding
            double fx = r.uniform(0.2, 0.45), fy = r.uniform(0.2, 0.45);
            double hx = r.uniform(x0 + (x1 - x0) * 0.25, x1 - (x1 - x0) * 0.25);
            double hy = r.uniform(y0 + (y1 - y0) * 0.25, y1 - (y1 - y0) * 0.25);
            double hw = (x1 - x0) * fx * 0.5, hh = (y1 - y0) * fy * 0.5;
            glyph_contour(b, r, hx - hw, hy - hh, hx + hw, hy + hh, (int)r.integer(10, 60), true);
        }
        b.draw_paths.push_back(make_path(c0, (uint32_t)ncont, PFColorU{255, 255, 255, 255}, -1,
                                         PF_FILL_RULE_WINDING));
    }
}

void gen_cubic_1k(Builder& b, Rng& r, double scale, int W, int H) {
    int n = std::max(1, (int)std::lround(256 * scale));
    // 4,096 control points over 256 paths: 16 points each = 5 cubics + start.
    for (int p = 0; p < n; p++) {
        double cx = r.uniform(0.1 * W, 0.9 * W), cy = r.uniform(0.1 * H, 0.9 * H);
        double rad = r.uniform(20.0, 120.0);
        uint32_t c0 = b.contour_count();
        const int k = 5;
        double phase = r.uniform(0.0, 2.0 * kPi);
        std::vector<double> vx(k), vy(k);
        for (int i = 0; i < k; i++) {
            double a = phase + 2.0 * kPi * i / k;
            double rr = rad * r.uniform(0.6, 1.0);
            vx[i] = cx + rr * std::cos(a);
            vy[i] = cy + rr * std::sin(a);
        }
        b.begin_contour(vx[0], vy[0]);
        for (int i = 0; i < k; i++) {
            int j = (i + 1) % k;
            double dx = vx[j] - vx[i], dy = vy[j] - vy[i];
            double c0x = vx[i] + dx / 3.0 + 0.3 * rad * r.normal() * 0.3;
            double c0y = vy[i] + dy / 3.0 + 0.3 * rad * r.normal() * 0.3;
            double c1x = vx[i] + 2.0 * dx / 3.0 + 0.3 * rad * r.normal() * 0.3;
            double c1y = vy[i] + 2.0 * dy / 3.0 + 0.3 * rad * r.normal() * 0.3;
            b.cubic_to(c0x, c0y, c1x, c1y, vx[j], vy[j]);
        }
        b.end_contour();
        uint8_t alpha = (uint8_t)std::lround(255.0 * r.uniform(0.3, 0.9));
        PFColorU paint{255, 255, 255, alpha};
        b.draw_paths.push_back(make_path(c0, 1, paint, -1, PF_FILL_RULE_WINDING));
    }
}

// Hand-built edge cases (64x64 canvas):
void gen_edge_cases(Builder& b, Rng& r, double, int W, int H) {
    (void)r; (void)W; (void)H;
    PFColorU opaque{200, 100, 50, 255}, half{20, 200, 120, 128};
    auto add = [&](PFColorU c, uint8_t rule, int32_t clip) {
        b.draw_paths.push_back(make_path(b.contour_count() - 1, 1, c, clip, rule));
    };
    // 0: full-tile square on the tile grid (solid interior, exact edges)
    b.begin_contour(16, 16); b.line_to(48, 16); b.line_to(48, 48); b.line_to(16, 48); b.end_contour();
    add(opaque, PF_FILL_RULE_WINDING, -1);
    // 1: a triangle whose edges pass exactly through tile corners
    b.begin_contour(0, 0); b.line_to(32, 32); b.line_to(0, 64); b.end_contour();
    add(half, PF_FILL_RULE_WINDING, -1);
    // 2: a path reaching far above the view box (backdrop-only columns above)
    b.begin_contour(20, -200); b.line_to(40, -180); b.line_to(44, 30); b.line_to(10, 40); b.end_contour();
    add(half, PF_FILL_RULE_EVEN_ODD, -1);
    // 3: horizontal and vertical lines only, partly left of the view box
    b.begin_contour(-10, 5.5f); b.line_to(30.25f, 5.5f); b.line_to(30.25f, 9.75f); b.line_to(-10, 9.75f); b.end_contour();
    add(opaque, PF_FILL_RULE_WINDING, -1);
    // 4: a self-overlapping star (winding 2 in the middle), even-odd
    b.begin_contour(32, 2); b.line_to(50, 60); b.line_to(2, 22); b.line_to(62, 22); b.line_to(14, 60); b.end_contour();
    add(half, PF_FILL_RULE_EVEN_ODD, -1);
    // 5: same star, nonzero
    b.begin_contour(32, 2); b.line_to(50, 60); b.line_to(2, 22); b.line_to(62, 22); b.line_to(14, 60); b.end_contour();
    add(half, PF_FILL_RULE_WINDING, -1);
    // 6: a degenerate contour (single point) and a zero-area line pair
    b.begin_contour(7, 7); b.end_contour();
    add(opaque, PF_FILL_RULE_WINDING, -1);
    // 7: a big cubic loop crossing the right edge of the view box
    b.begin_contour(40, 10); b.cubic_to(120, -20, 120, 90, 30, 50); b.end_contour();
    add(half, PF_FILL_RULE_WINDING, -1);
    // clip path 0: rect; 8: a circle-ish quad path clipped by it
    uint32_t cc = b.contour_count();
    b.begin_contour(8, 8); b.line_to(40.5, 8); b.line_to(40.5, 40.5); b.line_to(8, 40.5); b.end_contour();
    b.clip_paths.push_back(make_path(cc, 1, PFColorU{0, 0, 0, 0}, -1, PF_FILL_RULE_WINDING));
    b.begin_contour(32, 4); b.quad_to(60, 4, 60, 32); b.quad_to(60, 60, 32, 60); b.quad_to(4, 60, 4, 32);
    b.quad_to(4, 4, 32, 4); b.end_contour();
    add(opaque, PF_FILL_RULE_WINDING, 0);
    // 9: a path entirely outside the view box
    b.begin_contour(100, 100); b.line_to(120, 100); b.line_to(110, 120); b.end_contour();
    add(opaque, PF_FILL_RULE_WINDING, -1);
}

}  // namespace

struct PFCUDASceneBuffers {
    Builder b;
    int32_t width = 0, height = 0;
    PFRectF view_box{};
};

extern "C" {

int32_t PFCUDASceneGenerate(const PFCUDASceneParams* params, PFCUDASceneBuffersRef* out) {
    if (!params || !out) return PF_CUDA_ERR_INVALID;
    double scale = params->scale > 0 ? params->scale : 1.0;
    PFCUDASceneBuffers* s = new PFCUDASceneBuffers();
    Rng r(params->seed);
    int W = params->width, H = params->height;
    switch (params->workload) {
        case PF_SCENE_STARS_512: if (!W) W = 512; if (!H) H = 512; gen_stars_512(s->b, r, scale, W, H); break;
        case PF_SCENE_SVG_4K: if (!W) W = 3840; if (!H) H = 2160; gen_svg_4k(s->b, r, scale, W, H); break;
        case PF_SCENE_GLYPH_ATLAS: if (!W) W = 4096; if (!H) H = 4096; gen_glyph_atlas(s->b, r, scale, W, H); break;
        case PF_SCENE_CUBIC_1K: if (!W) W = 1024; if (!H) H = 1024; gen_cubic_1k(s->b, r, scale, W, H); break;
        case PF_SCENE_EDGE_CASES: if (!W) W = 64; if (!H) H = 64; gen_edge_cases(s->b, r, scale, W, H); break;
        default: delete s; return PF_CUDA_ERR_INVALID;
    }
    if (params->jitter_sigma > 0) {
        Rng jr(params->jitter_seed);
        for (PFVector2F& p : s->b.points) {
            p.x = (float)(p.x + params->jitter_sigma * jr.normal());
            p.y = (float)(p.y + params->jitter_sigma * jr.normal());
        }
    }
    s->width = W;
    s->height = H;
    s->view_box = PFRectF{{0.0f, 0.0f}, {(float)W, (float)H}};
    *out = s;
    return PF_CUDA_OK;
}

int32_t PFCUDASceneGetDesc(PFCUDASceneBuffersRef s, PFCUDASceneDesc* d, int32_t* w, int32_t* h) {
    if (!s || !d) return PF_CUDA_ERR_INVALID;
    d->points = s->b.points.data();
    d->point_flags = s->b.flags.data();
    d->contour_starts = s->b.contour_starts.data();
    d->clip_paths = s->b.clip_paths.data();
    d->draw_paths = s->b.draw_paths.data();
    d->point_count = (uint32_t)s->b.points.size();
    d->contour_count = s->b.contour_count();
    d->clip_path_count = (uint32_t)s->b.clip_paths.size();
    d->draw_path_count = (uint32_t)s->b.draw_paths.size();
    d->view_box = s->view_box;
    d->memory = PF_MEMORY_HOST;
    d->gradients = nullptr;  // generated scenes have solid paint
    d->gradient_count = 0;
    d->patterns = nullptr;
    d->pattern_count = 0;
    if (w) *w = s->width;
    if (h) *h = s->height;
    return PF_CUDA_OK;
}

int32_t PFCUDASceneGetCells(PFCUDASceneBuffersRef s, PFRectI* cells, uint32_t capacity) {
    if (!s) return PF_CUDA_ERR_INVALID;
    if (cells) {
        uint32_t n = std::min<uint32_t>(capacity, (uint32_t)s->b.cells.size());
        for (uint32_t i = 0; i < n; i++) cells[i] = s->b.cells[i];
    }
    return PF_CUDA_OK;
}

int32_t PFCUDASceneDestroy(PFCUDASceneBuffersRef s) {
    delete s;
    return PF_CUDA_OK;
}

}  // extern "C"

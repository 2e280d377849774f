// pf_renderer.cu — host side of the CUDA renderer level and its C ABI.
//
// The frame replaces RendererD3D11::prepare_tiles / draw_tiles
// (renderer/src/gpu/d3d11/renderer.rs:414-782).  The reference sizes its
// buffers with three blocking readbacks and a regrow-and-retry loop
// (:218-229, :338-353, :463-499, :634-648).  Here every kernel checks the
// device-side totals against the buffer capacities, the frame is enqueued
// without any mid-frame synchronisation, and the single status readback at
// the end triggers a regrow and one re-run only when a capacity was exceeded
// (in steady state: never).
#include "pf_kernels.cuh"
#include "../../include/pathfinder_cuda.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

using namespace pf;

namespace {

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t n) {
        if (n <= cap && p) return cudaSuccess;
        if (p) { cudaFree(p); p = nullptr; cap = 0; }
        size_t want = std::max<size_t>(n, 1);
        cudaError_t e = cudaMalloc((void**)&p, want * sizeof(T));
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; cap = 0; }
};

inline int32_t cvt_rne_host(float x) {
    if (!(x >= -2147483648.0f && x < 2147483648.0f)) return INT32_MIN;
    return (int32_t)std::nearbyint(x);
}

}  // namespace

struct PFCUDARenderer {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    PFCUDARendererOptions options{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    // scene (resident)
    bool has_scene = false;
    uint32_t P = 0, nclip = 0, ndraw = 0, NP = 0, NC = 0, nord = 0, S = 0;
    PFRectF view_box{};
    DevBuf<float2> pts, pts_t;
    DevBuf<uint8_t> flags;
    DevBuf<uint32_t> starts, ord_contour, ord_path, contour_segs, contour_seg_base;
    DevBuf<SegRec> segs;
    DevBuf<uint32_t> first_ord, paint, local_index, scene_of;
    DevBuf<int32_t> clip_gpath;
    DevBuf<uint8_t> rule, is_clip;
    DevBuf<SceneDev> scenes;
    std::vector<PFCUDAPath> host_paths;  // clip paths then draw paths

    // per-frame buffers
    DevBuf<int4> tile_rect;
    DevBuf<uint32_t> tile_offset, col_offset;
    DevBuf<uint32_t> seg_line_count, seg_line_base;
    DevBuf<float4> lines;
    DevBuf<uint32_t> line_path, line_fill_count, line_fill_base;
    DevBuf<uint32_t> tile_fill_count, tile_fill_base, tile_alpha, alpha_owner;
    DevBuf<int32_t> tile_delta, col_backdrop, zbuf;
    DevBuf<uint32_t> tile_delta_scan, path_tiles, path_cols;
    DevBuf<uint2> fills;
    DevBuf<uint32_t> fill_e;
    DevBuf<int4> tiles, clips;
    DevBuf<uint32_t> screen_cnt, screen_base, vis;
    DevBuf<uint32_t> scan_partials;
    DevBuf<Counters> counters;
    DevBuf<uint8_t> out_tmp;
    Counters* h_counters = nullptr;  // pinned

    uint32_t tile_cap = 0, col_cap = 0, fill_cap = 0, vis_cap = 0, line_cap = 0;
    uint32_t screen_count = 0;
    int4 screen_rect{0, 0, 0, 0};
    int32_t last_w = 0, last_h = 0;
    PFCUDARenderStats stats{};
    uint64_t last_needed = 0;
    uint32_t pending_status = 0;
    bool profiling = false;
    cudaEvent_t stage_ev[PF_CUDA_STAGE_COUNT + 1] = {};
    uint64_t launches = 0;
};

namespace {

int32_t cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return PF_CUDA_OK;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return PF_CUDA_ERR_NO_DEVICE;
    return PF_CUDA_ERR_LAUNCH;
}

#define PF_TRY(expr)                                      \
    do {                                                  \
        cudaError_t _e = (expr);                          \
        if (_e != cudaSuccess) return cuda_status(_e);    \
    } while (0)

int4 screen_rect_of(PFRectF v) {
    // round_rect_out_to_tile_bounds (renderer/src/tiles.rs:64-66)
    const float q = 1.0f / 16.0f;
    return make_int4(cvt_rne_host(std::floor(v.origin.x * q)), cvt_rne_host(std::floor(v.origin.y * q)),
                     cvt_rne_host(std::ceil(v.lower_right.x * q)), cvt_rne_host(std::ceil(v.lower_right.y * q)));
}

FrameDev frame_dev(PFCUDARenderer* r, bool transformed) {
    FrameDev f{};
    f.pts = transformed ? r->pts_t.p : r->pts.p;
    f.segs = r->segs.p;
    f.seg_count = r->S;
    f.path.first_ord_contour = r->first_ord.p;
    f.path.paint = r->paint.p;
    f.path.clip_gpath = r->clip_gpath.p;
    f.path.rule = r->rule.p;
    f.path.is_clip = r->is_clip.p;
    f.path.local_index = r->local_index.p;
    f.path.scene = r->scene_of.p;
    f.path.tile_rect = r->tile_rect.p;
    f.path.tile_offset = r->tile_offset.p;
    f.path.col_offset = r->col_offset.p;
    f.scenes = r->scenes.p;
    f.path_count = r->P;
    f.scene_count = 1;
    f.tile_cap = r->tile_cap;
    f.col_cap = r->col_cap;
    f.fill_cap = r->fill_cap;
    f.vis_cap = r->vis_cap;
    f.screen_count = r->screen_count;
    f.tile_fill_count = r->tile_fill_count.p;
    f.tile_fill_base = r->tile_fill_base.p;
    f.tile_alpha = r->tile_alpha.p;
    f.tile_delta = r->tile_delta.p;
    f.tile_delta_scan = r->tile_delta_scan.p;
    f.path_tiles = r->path_tiles.p;
    f.path_cols = r->path_cols.p;
    f.col_backdrop = r->col_backdrop.p;
    f.seg_line_count = r->seg_line_count.p;
    f.seg_line_base = r->seg_line_base.p;
    f.lines = r->lines.p;
    f.line_path = r->line_path.p;
    f.line_fill_count = r->line_fill_count.p;
    f.line_fill_base = r->line_fill_base.p;
    f.line_cap = r->line_cap;
    f.fills = r->fills.p;
    f.fill_e = r->fill_e.p;
    f.tiles = r->tiles.p;
    f.clips = r->clips.p;
    f.alpha_owner = r->alpha_owner.p;
    f.zbuf = r->zbuf.p;
    f.screen_cnt = r->screen_cnt.p;
    f.screen_base = r->screen_base.p;
    f.vis = r->vis.p;
    f.counters = r->counters.p;
    f.dda_limit = 1u << 24;
    return f;
}

cudaError_t ensure_frame_buffers(PFCUDARenderer* r) {
    cudaError_t e;
    if ((e = r->tile_fill_count.ensure((size_t)r->tile_cap + 1))) return e;
    if ((e = r->tile_fill_base.ensure((size_t)r->tile_cap + 1))) return e;
    if ((e = r->tile_alpha.ensure((size_t)r->tile_cap + 1))) return e;
    if ((e = r->alpha_owner.ensure((size_t)r->tile_cap + 1))) return e;
    if ((e = r->tile_delta.ensure((size_t)r->tile_cap + 1))) return e;
    if ((e = r->tile_delta_scan.ensure((size_t)r->tile_cap + 1))) return e;
    if ((e = r->path_tiles.ensure((size_t)r->P + 1))) return e;
    if ((e = r->path_cols.ensure((size_t)r->P + 1))) return e;
    if ((e = r->tiles.ensure((size_t)r->tile_cap + 1))) return e;
    if ((e = r->clips.ensure((size_t)r->tile_cap + 1))) return e;
    if ((e = r->col_backdrop.ensure((size_t)r->col_cap + 1))) return e;
    if ((e = r->fills.ensure((size_t)r->fill_cap + 1))) return e;
    if ((e = r->fill_e.ensure((size_t)r->fill_cap + 1))) return e;
    if ((e = r->lines.ensure((size_t)r->line_cap + 1))) return e;
    if ((e = r->line_path.ensure((size_t)r->line_cap + 1))) return e;
    if ((e = r->line_fill_count.ensure((size_t)r->line_cap + 1))) return e;
    if ((e = r->line_fill_base.ensure((size_t)r->line_cap + 1))) return e;
    if ((e = r->vis.ensure((size_t)r->vis_cap + 1))) return e;
    if ((e = r->zbuf.ensure((size_t)r->screen_count + 1))) return e;
    if ((e = r->screen_cnt.ensure((size_t)r->screen_count + 1))) return e;
    if ((e = r->screen_base.ensure((size_t)r->screen_count + 1))) return e;
    size_t nmax = std::max<size_t>({(size_t)r->tile_cap, (size_t)r->S, (size_t)r->screen_count, (size_t)r->nord,
                                    (size_t)r->line_cap, (size_t)r->P}) + 1;
    if ((e = r->scan_partials.ensure(nmax / 2048 + 2))) return e;
    return cudaSuccess;
}

bool is_identity(const PFCUDABuildOptions* o) {
    if (!o || !o->has_transform) return true;
    const PFTransform2F& t = o->transform;
    return t.m00 == 1.0f && t.m01 == 0.0f && t.m10 == 0.0f && t.m11 == 1.0f && t.vector.x == 0.0f &&
           t.vector.y == 0.0f;
}

// Enqueue one frame.  mode: 0 RGBA8, 1 R8, 2 FP32 single channel, -1 no composite.
cudaError_t enqueue_frame(PFCUDARenderer* r, const PFCUDABuildOptions* opts, int mode, void* out_dev) {
    cudaStream_t s = r->stream;
    bool transformed = !is_identity(opts);
    cudaError_t e;
    if (transformed) {
        if ((e = r->pts_t.ensure(r->NP))) return e;
        float m6[6] = {opts->transform.m00, opts->transform.m01, opts->transform.m10, opts->transform.m11,
                       opts->transform.vector.x, opts->transform.vector.y};
        launch_transform(r->pts.p, r->pts_t.p, r->NP, m6, s);
    }
    FrameDev f = frame_dev(r, transformed);
    ScanTemp tmp{r->scan_partials.p, (uint32_t)r->scan_partials.cap};
    Counters* c = r->counters.p;
    auto mark = [&](int stage) {
        if (r->profiling) cudaEventRecord(r->stage_ev[stage], s);
    };
    uint64_t before = launch_counter();
    if ((e = cudaMemsetAsync(c, 0, sizeof(Counters), s))) return e;
    mark(0);
    launch_bound(f, r->ord_contour.p, r->starts.p, s);
    launch_path_scan(f, tmp, s);
    mark(1);
    launch_flatten(f, tmp, s);
    mark(2);
    launch_bin_count(f, s);
    mark(3);
    launch_scan((const uint32_t*)r->tile_delta.p, r->tile_delta_scan.p, &c->tiles, 0, r->tile_cap, 0, nullptr, tmp, s);
    launch_scan(r->line_fill_count.p, r->line_fill_base.p, &c->lines, 0, r->line_cap, 0, &c->fills, tmp, s);
    launch_scan(r->tile_fill_count.p, r->tile_fill_base.p, &c->tiles, 0, r->tile_cap, 0, nullptr, tmp, s);
    launch_scan(r->tile_fill_count.p, r->tile_alpha.p, &c->tiles, 0, r->tile_cap, 1, &c->alpha_tiles, tmp, s);
    mark(4);
    launch_bin_emit(f, s);
    mark(5);
    if ((e = cudaMemsetAsync(r->zbuf.p, 0, sizeof(int32_t) * (r->screen_count + 1), s))) return e;
    // clip paths first: draw paths read their finished tiles
    launch_propagate(f, true, 0, r->nclip, 0, s);
    launch_propagate(f, false, r->nclip, r->ndraw, 0, s);
    mark(6);
    if ((e = cudaMemsetAsync(r->screen_cnt.p, 0, sizeof(uint32_t) * (r->screen_count + 1), s))) return e;
    launch_visible(f, false, s);
    launch_scan(r->screen_cnt.p, r->screen_base.p, nullptr, r->screen_count, r->screen_count, 0, &c->visible, tmp, s);
    launch_visible(f, true, s);
    mark(7);
    if (mode >= 0) {
        float4 bg = make_float4(0, 0, 0, 0);
        if (r->options.has_background_color)
            bg = make_float4(r->options.background_color.r, r->options.background_color.g,
                             r->options.background_color.b, r->options.background_color.a);
        launch_composite(f, mode, out_dev, bg, s);
    }
    mark(8);
    r->launches = launch_counter() - before;
    return cudaGetLastError();
}

// Grow capacities after an overflow report.
void grow(PFCUDARenderer* r, const Counters& h) {
    auto up = [](uint64_t need) { return (uint32_t)std::min<uint64_t>(0xfffffff0ull, need + need / 4 + 1024); };
    if (h.status & (kStatusTileCapacity | kStatusColumnCapacity)) {
        r->tile_cap = std::max(r->tile_cap, up(h.tiles));
        r->col_cap = std::max(r->col_cap, up(h.columns));
        r->vis_cap = std::max(r->vis_cap, r->tile_cap);
    }
    if (h.status & kStatusFillCapacity) r->fill_cap = std::max(r->fill_cap, up(h.fills));
    if (h.status & kStatusLineCapacity) r->line_cap = std::max(r->line_cap, up(h.lines));
    if (h.status & kStatusVisibleCapacity) r->vis_cap = std::max(r->vis_cap, up(h.visible));
}

const uint32_t kCapacityBits = kStatusTileCapacity | kStatusColumnCapacity | kStatusFillCapacity |
                               kStatusVisibleCapacity | kStatusAlphaCapacity | kStatusLineCapacity;

int32_t status_to_code(uint32_t st) {
    if (st & kCapacityBits) return PF_CUDA_ERR_CAPACITY;
    if (st & (kStatusDdaLimit | kStatusDepthLimit)) return PF_CUDA_ERR_LIMIT;
    if (st & kStatusMalformed) return PF_CUDA_ERR_INVALID;
    return PF_CUDA_OK;
}

void record_stats(PFCUDARenderer* r, const Counters& h, float ms) {
    r->stats.path_count = r->P;
    r->stats.segment_count = r->S;
    r->stats.line_count = h.lines;
    r->stats.fill_count = h.fills;
    r->stats.tile_count = h.tiles;
    r->stats.alpha_tile_count = h.alpha_tiles;
    r->stats.visible_tile_count = h.visible;
    r->stats.screen_tile_count = r->screen_count;
    r->stats.status = h.status;
    r->stats.gpu_time_ms = ms;
    r->stats.kernel_launches = r->launches;
}

int32_t prepare_size(PFCUDARenderer* r, int32_t width, int32_t height) {
    if (width <= 0 || height <= 0) return PF_CUDA_ERR_INVALID;
    SceneDev sd{};
    sd.view_box = make_float4(r->view_box.origin.x, r->view_box.origin.y, r->view_box.lower_right.x,
                              r->view_box.lower_right.y);
    sd.screen = r->screen_rect;
    sd.screen_offset = 0;
    sd.first_path = 0;
    sd.clip_count = r->nclip;
    sd.draw_count = r->ndraw;
    sd.width = width;
    sd.height = height;
    sd.out_offset = 0;
    PF_TRY(cudaMemcpyAsync(r->scenes.p, &sd, sizeof(SceneDev), cudaMemcpyHostToDevice, r->stream));
    r->last_w = width;
    r->last_h = height;
    return PF_CUDA_OK;
}

// Run one frame synchronously with regrow-and-retry.
int32_t run_frame(PFCUDARenderer* r, const PFCUDABuildOptions* opts, int mode, void* out_dev, int32_t w, int32_t h) {
    if (!r->has_scene) return PF_CUDA_ERR_NO_SCENE;
    int32_t rc = prepare_size(r, w, h);
    if (rc) return rc;
    for (int attempt = 0; attempt < 4; attempt++) {
        PF_TRY(ensure_frame_buffers(r));
        PF_TRY(cudaEventRecord(r->ev0, r->stream));
        PF_TRY(enqueue_frame(r, opts, mode, out_dev));
        PF_TRY(cudaEventRecord(r->ev1, r->stream));
        PF_TRY(cudaMemcpyAsync(r->h_counters, r->counters.p, sizeof(Counters), cudaMemcpyDeviceToHost, r->stream));
        PF_TRY(cudaStreamSynchronize(r->stream));
        float ms = 0;
        cudaEventElapsedTime(&ms, r->ev0, r->ev1);
        Counters h = *r->h_counters;
        record_stats(r, h, ms);
        if (h.status & kCapacityBits) {
            grow(r, h);
            continue;
        }
        return status_to_code(h.status);
    }
    return PF_CUDA_ERR_CAPACITY;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int32_t PFCUDARendererCreate(int32_t device_ordinal, const PFCUDARendererOptions* options,
                             PFCUDARendererRef* out_renderer) {
    if (!out_renderer) return PF_CUDA_ERR_INVALID;
    *out_renderer = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return PF_CUDA_ERR_NO_DEVICE;
    if (device_ordinal < 0 || device_ordinal >= count) return PF_CUDA_ERR_INVALID;
    PF_TRY(cudaSetDevice(device_ordinal));
    PFCUDARenderer* r = new PFCUDARenderer();
    r->device = device_ordinal;
    if (options) r->options = *options;
    if ((e = cudaStreamCreateWithFlags(&r->own_stream, cudaStreamNonBlocking)) ||
        (e = cudaEventCreate(&r->ev0)) || (e = cudaEventCreate(&r->ev1)) ||
        (e = cudaMallocHost((void**)&r->h_counters, sizeof(Counters))) || (e = r->counters.ensure(1)) ||
        (e = r->scenes.ensure(1))) {
        PFCUDARendererDestroy(r);
        return cuda_status(e);
    }
    r->stream = r->own_stream;
    *out_renderer = r;
    return PF_CUDA_OK;
}

int32_t PFCUDARendererDestroy(PFCUDARendererRef r) {
    if (!r) return PF_CUDA_OK;
    cudaSetDevice(r->device);
    if (r->stream) cudaStreamSynchronize(r->stream);
    r->pts.release(); r->pts_t.release(); r->flags.release(); r->starts.release();
    r->ord_contour.release(); r->ord_path.release(); r->contour_segs.release(); r->contour_seg_base.release();
    r->segs.release(); r->first_ord.release(); r->paint.release(); r->local_index.release();
    r->scene_of.release(); r->clip_gpath.release(); r->rule.release(); r->is_clip.release();
    r->scenes.release(); r->tile_rect.release(); r->tile_offset.release(); r->col_offset.release();
    r->seg_line_count.release(); r->seg_line_base.release(); r->lines.release(); r->line_path.release();
    r->line_fill_count.release(); r->line_fill_base.release(); r->tile_fill_count.release();
    r->tile_fill_base.release(); r->tile_alpha.release(); r->alpha_owner.release(); r->tile_delta.release();
    r->tile_delta_scan.release(); r->path_tiles.release(); r->path_cols.release();
    r->col_backdrop.release(); r->zbuf.release(); r->fills.release(); r->fill_e.release(); r->tiles.release();
    r->clips.release(); r->screen_cnt.release(); r->screen_base.release(); r->vis.release();
    r->scan_partials.release(); r->counters.release(); r->out_tmp.release();
    if (r->h_counters) cudaFreeHost(r->h_counters);
    if (r->ev0) cudaEventDestroy(r->ev0);
    if (r->ev1) cudaEventDestroy(r->ev1);
    for (int i = 0; i <= PF_CUDA_STAGE_COUNT; i++)
        if (r->stage_ev[i]) cudaEventDestroy(r->stage_ev[i]);
    if (r->own_stream) cudaStreamDestroy(r->own_stream);
    delete r;
    return PF_CUDA_OK;
}

int32_t PFCUDARendererSetStream(PFCUDARendererRef r, void* stream) {
    if (!r) return PF_CUDA_ERR_INVALID;
    r->stream = stream ? (cudaStream_t)stream : r->own_stream;
    return PF_CUDA_OK;
}

int32_t PFCUDARendererSetOptions(PFCUDARendererRef r, const PFCUDARendererOptions* options) {
    if (!r || !options) return PF_CUDA_ERR_INVALID;
    r->options = *options;
    return PF_CUDA_OK;
}

int32_t PFCUDASceneUpload(PFCUDARendererRef r, const PFCUDASceneDesc* sc) {
    if (!r || !sc) return PF_CUDA_ERR_INVALID;
    if (sc->memory != PF_MEMORY_HOST && sc->memory != PF_MEMORY_DEVICE) return PF_CUDA_ERR_INVALID;
    if ((sc->clip_path_count && !sc->clip_paths) || (sc->draw_path_count && !sc->draw_paths))
        return PF_CUDA_ERR_INVALID;
    if (sc->contour_count && !sc->contour_starts) return PF_CUDA_ERR_INVALID;
    if (sc->point_count && (!sc->points || !sc->point_flags)) return PF_CUDA_ERR_INVALID;
    PF_TRY(cudaSetDevice(r->device));
    cudaStream_t s = r->stream;
    r->has_scene = false;
    const cudaMemcpyKind kind = sc->memory == PF_MEMORY_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;

    // contour starts are needed on the host for validation and ordering
    std::vector<uint32_t> hstarts(sc->contour_count + 1, 0);
    if (sc->contour_count) {
        if (sc->memory == PF_MEMORY_HOST)
            std::memcpy(hstarts.data(), sc->contour_starts, sizeof(uint32_t) * (sc->contour_count + 1));
        else
            PF_TRY(cudaMemcpy(hstarts.data(), sc->contour_starts, sizeof(uint32_t) * (sc->contour_count + 1),
                              cudaMemcpyDeviceToHost));
    }
    for (uint32_t c = 0; c < sc->contour_count; c++)
        if (hstarts[c] > hstarts[c + 1] || hstarts[c + 1] > sc->point_count) return PF_CUDA_ERR_INVALID;

    uint32_t P = sc->clip_path_count + sc->draw_path_count;
    r->host_paths.assign(P, PFCUDAPath{});
    std::vector<uint32_t> first_ord(P + 1, 0), ord_contour, ord_path, paint(P), local(P), scene(P, 0);
    std::vector<int32_t> clip(P);
    std::vector<uint8_t> rule(P), isclip(P);
    for (uint32_t gp = 0; gp < P; gp++) {
        bool c = gp < sc->clip_path_count;
        const PFCUDAPath& p = c ? sc->clip_paths[gp] : sc->draw_paths[gp - sc->clip_path_count];
        r->host_paths[gp] = p;
        if ((uint64_t)p.first_contour + p.contour_count > sc->contour_count) return PF_CUDA_ERR_INVALID;
        if (p.fill_rule > 1 || p.blend_mode != PF_BLEND_MODE_SRC_OVER) return PF_CUDA_ERR_INVALID;
        if (!c && p.clip_path >= (int32_t)sc->clip_path_count) return PF_CUDA_ERR_INVALID;
        if (c && p.clip_path >= 0) return PF_CUDA_ERR_INVALID;  // nested clips: not on this path
        first_ord[gp] = (uint32_t)ord_contour.size();
        for (uint32_t k = 0; k < p.contour_count; k++) {
            ord_contour.push_back(p.first_contour + k);
            ord_path.push_back(gp);
        }
        paint[gp] = (uint32_t)p.paint.r | ((uint32_t)p.paint.g << 8) | ((uint32_t)p.paint.b << 16) |
                    ((uint32_t)p.paint.a << 24);
        local[gp] = c ? gp : gp - sc->clip_path_count;
        clip[gp] = (!c && p.clip_path >= 0) ? p.clip_path : -1;  // clip paths come first: gp == clip index
        rule[gp] = p.fill_rule;
        isclip[gp] = c ? 1 : 0;
    }
    first_ord[P] = (uint32_t)ord_contour.size();
    uint32_t nord = (uint32_t)ord_contour.size();

    cudaError_t e;
    if ((e = r->pts.ensure(sc->point_count)) || (e = r->flags.ensure(sc->point_count)) ||
        (e = r->starts.ensure(sc->contour_count + 1)) || (e = r->ord_contour.ensure(nord)) ||
        (e = r->ord_path.ensure(nord)) || (e = r->contour_segs.ensure(nord + 1)) ||
        (e = r->contour_seg_base.ensure(nord + 1)) || (e = r->first_ord.ensure(P + 1)) ||
        (e = r->paint.ensure(P)) || (e = r->local_index.ensure(P)) || (e = r->scene_of.ensure(P)) ||
        (e = r->clip_gpath.ensure(P)) || (e = r->rule.ensure(P)) || (e = r->is_clip.ensure(P)) ||
        (e = r->tile_rect.ensure(P)) || (e = r->tile_offset.ensure(P + 1)) || (e = r->col_offset.ensure(P + 1)) ||
        (e = r->scan_partials.ensure(nord / 2048 + 2)))
        return cuda_status(e);
    if (sc->point_count) {
        PF_TRY(cudaMemcpyAsync(r->pts.p, sc->points, sizeof(float2) * sc->point_count, kind, s));
        PF_TRY(cudaMemcpyAsync(r->flags.p, sc->point_flags, sc->point_count, kind, s));
    }
    PF_TRY(cudaMemcpyAsync(r->starts.p, hstarts.data(), sizeof(uint32_t) * (sc->contour_count + 1),
                           cudaMemcpyHostToDevice, s));
    if (nord) {
        PF_TRY(cudaMemcpyAsync(r->ord_contour.p, ord_contour.data(), sizeof(uint32_t) * nord, cudaMemcpyHostToDevice, s));
        PF_TRY(cudaMemcpyAsync(r->ord_path.p, ord_path.data(), sizeof(uint32_t) * nord, cudaMemcpyHostToDevice, s));
    }
    if (P) {
        PF_TRY(cudaMemcpyAsync(r->first_ord.p, first_ord.data(), sizeof(uint32_t) * (P + 1), cudaMemcpyHostToDevice, s));
        PF_TRY(cudaMemcpyAsync(r->paint.p, paint.data(), sizeof(uint32_t) * P, cudaMemcpyHostToDevice, s));
        PF_TRY(cudaMemcpyAsync(r->local_index.p, local.data(), sizeof(uint32_t) * P, cudaMemcpyHostToDevice, s));
        PF_TRY(cudaMemcpyAsync(r->scene_of.p, scene.data(), sizeof(uint32_t) * P, cudaMemcpyHostToDevice, s));
        PF_TRY(cudaMemcpyAsync(r->clip_gpath.p, clip.data(), sizeof(int32_t) * P, cudaMemcpyHostToDevice, s));
        PF_TRY(cudaMemcpyAsync(r->rule.p, rule.data(), P, cudaMemcpyHostToDevice, s));
        PF_TRY(cudaMemcpyAsync(r->is_clip.p, isclip.data(), P, cudaMemcpyHostToDevice, s));
    }
    // Segment packing on the GPU (SegmentsD3D11::add_path): count, scan, emit.
    PF_TRY(cudaMemsetAsync(r->counters.p, 0, sizeof(Counters), s));
    launch_contour_segcount(r->ord_contour.p, nord, r->starts.p, r->flags.p, r->contour_segs.p,
                            &r->counters.p->status, s);
    ScanTemp tmp{r->scan_partials.p, (uint32_t)r->scan_partials.cap};
    launch_scan(r->contour_segs.p, r->contour_seg_base.p, nullptr, nord, nord, 0, &r->counters.p->lines, tmp, s);
    PF_TRY(cudaMemcpyAsync(r->h_counters, r->counters.p, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    PF_TRY(cudaStreamSynchronize(s));
    if (r->h_counters->status & kStatusMalformed) return PF_CUDA_ERR_INVALID;
    uint32_t S = (uint32_t)r->h_counters->lines;
    if ((e = r->segs.ensure(S + 1)) || (e = r->seg_line_count.ensure(S + 1)) || (e = r->seg_line_base.ensure(S + 1)))
        return cuda_status(e);
    launch_contour_segemit(r->ord_contour.p, r->ord_path.p, nord, r->starts.p, r->flags.p, r->contour_seg_base.p,
                           r->segs.p, s);
    PF_TRY(cudaGetLastError());

    r->P = P;
    r->nclip = sc->clip_path_count;
    r->ndraw = sc->draw_path_count;
    r->NP = sc->point_count;
    r->NC = sc->contour_count;
    r->nord = nord;
    r->S = S;
    r->view_box = sc->view_box;
    r->screen_rect = screen_rect_of(sc->view_box);
    int32_t sw = std::max(0, r->screen_rect.z - r->screen_rect.x), sh = std::max(0, r->screen_rect.w - r->screen_rect.y);
    r->screen_count = (uint32_t)sw * (uint32_t)sh;
    // first-frame capacity guesses; grown on overflow and kept across frames
    r->tile_cap = std::max<uint32_t>(r->tile_cap, std::max<uint32_t>(1u << 16, 4 * r->screen_count));
    r->col_cap = std::max<uint32_t>(r->col_cap, std::max<uint32_t>(1u << 16, 16 * P));
    r->fill_cap = std::max<uint32_t>(r->fill_cap, std::max<uint32_t>(1u << 18, 4 * S));
    r->line_cap = std::max<uint32_t>(r->line_cap, std::max<uint32_t>(1u << 16, 2 * S));
    r->vis_cap = std::max<uint32_t>(r->vis_cap, r->tile_cap);
    r->has_scene = true;
    PF_TRY(cudaStreamSynchronize(s));
    return PF_CUDA_OK;
}

int32_t PFCUDARenderScene(PFCUDARendererRef r, const PFCUDABuildOptions* options, int32_t width, int32_t height,
                          uint8_t* out, int32_t out_memory) {
    if (!r || !out) return PF_CUDA_ERR_INVALID;
    PF_TRY(cudaSetDevice(r->device));
    void* dst = out;
    size_t bytes = (size_t)width * (size_t)height * 4;
    if (out_memory == PF_MEMORY_HOST) {
        PF_TRY(r->out_tmp.ensure(bytes));
        dst = r->out_tmp.p;
    } else if (out_memory != PF_MEMORY_DEVICE) {
        return PF_CUDA_ERR_INVALID;
    }
    int32_t rc = run_frame(r, options, 0, dst, width, height);
    if (rc == PF_CUDA_OK && out_memory == PF_MEMORY_HOST) {
        PF_TRY(cudaMemcpyAsync(out, dst, bytes, cudaMemcpyDeviceToHost, r->stream));
        PF_TRY(cudaStreamSynchronize(r->stream));
    }
    return rc;
}

int32_t PFCUDARenderSceneAsync(PFCUDARendererRef r, const PFCUDABuildOptions* options, int32_t width,
                               int32_t height, uint8_t* out_rgba8_device) {
    if (!r || !out_rgba8_device) return PF_CUDA_ERR_INVALID;
    if (!r->has_scene) return PF_CUDA_ERR_NO_SCENE;
    if (width != r->last_w || height != r->last_h) {
        int32_t rc = prepare_size(r, width, height);
        if (rc) return rc;
    }
    PF_TRY(ensure_frame_buffers(r));
    PF_TRY(enqueue_frame(r, options, 0, out_rgba8_device));
    return PF_CUDA_OK;
}

int32_t PFCUDARenderStatus(PFCUDARendererRef r, uint64_t* out_needed) {
    if (!r) return PF_CUDA_ERR_INVALID;
    PF_TRY(cudaMemcpyAsync(r->h_counters, r->counters.p, sizeof(Counters), cudaMemcpyDeviceToHost, r->stream));
    PF_TRY(cudaStreamSynchronize(r->stream));
    Counters h = *r->h_counters;
    record_stats(r, h, 0.0f);
    if (out_needed) *out_needed = std::max({h.needed_fills, h.needed_tiles, h.needed_visible});
    if (h.status & kCapacityBits) grow(r, h);
    return status_to_code(h.status);
}

int32_t PFCUDARenderCoverage(PFCUDARendererRef r, const PFCUDABuildOptions* options, int32_t width, int32_t height,
                             float* out, int32_t out_memory) {
    if (!r || !out) return PF_CUDA_ERR_INVALID;
    PF_TRY(cudaSetDevice(r->device));
    void* dst = out;
    size_t bytes = (size_t)width * (size_t)height * sizeof(float);
    if (out_memory == PF_MEMORY_HOST) {
        PF_TRY(r->out_tmp.ensure(bytes));
        dst = r->out_tmp.p;
    } else if (out_memory != PF_MEMORY_DEVICE) {
        return PF_CUDA_ERR_INVALID;
    }
    int32_t rc = run_frame(r, options, 2, dst, width, height);
    if (rc == PF_CUDA_OK && out_memory == PF_MEMORY_HOST) {
        PF_TRY(cudaMemcpyAsync(out, dst, bytes, cudaMemcpyDeviceToHost, r->stream));
        PF_TRY(cudaStreamSynchronize(r->stream));
    }
    return rc;
}

int32_t PFCUDAReadMasks(PFCUDARendererRef r, float* out_alpha, uint64_t alpha_cap, float* out_tile,
                        uint64_t tile_cap) {
    if (!r || !r->has_scene) return PF_CUDA_ERR_NO_SCENE;
    PF_TRY(cudaSetDevice(r->device));
    uint64_t A = r->stats.alpha_tile_count, T = r->stats.tile_count;
    if ((out_alpha && alpha_cap < A) || (out_tile && tile_cap < T)) return PF_CUDA_ERR_CAPACITY;
    FrameDev f = frame_dev(r, false);
    DevBuf<float> a, t;
    if (out_alpha) PF_TRY(a.ensure(A * 256 + 1));
    if (out_tile) PF_TRY(t.ensure(T * 256 + 1));
    launch_masks(f, out_alpha ? a.p : nullptr, out_tile ? t.p : nullptr, r->stream);
    PF_TRY(cudaGetLastError());
    if (out_alpha && A) PF_TRY(cudaMemcpyAsync(out_alpha, a.p, A * 256 * sizeof(float), cudaMemcpyDeviceToHost, r->stream));
    if (out_tile && T) PF_TRY(cudaMemcpyAsync(out_tile, t.p, T * 256 * sizeof(float), cudaMemcpyDeviceToHost, r->stream));
    PF_TRY(cudaStreamSynchronize(r->stream));
    a.release();
    t.release();
    return PF_CUDA_OK;
}

int32_t PFCUDAReadRecords(PFCUDARendererRef r, PFCUDAFill* fills, uint32_t* fill_tile, uint64_t fill_capacity,
                          PFCUDATile* tiles, uint64_t tile_capacity, uint32_t* path_tile_offsets,
                          PFRectI* path_tile_rects, uint64_t path_capacity, PFCUDAClip* clips, int32_t* z_buffer,
                          uint64_t z_capacity) {
    if (!r || !r->has_scene) return PF_CUDA_ERR_NO_SCENE;
    PF_TRY(cudaSetDevice(r->device));
    cudaStream_t s = r->stream;
    uint64_t F = r->stats.fill_count, T = r->stats.tile_count;
    if ((fills || fill_tile) && fill_capacity < F) return PF_CUDA_ERR_CAPACITY;
    if ((tiles || clips) && tile_capacity < T) return PF_CUDA_ERR_CAPACITY;
    if ((path_tile_offsets || path_tile_rects) && path_capacity < (uint64_t)r->P + 1) return PF_CUDA_ERR_CAPACITY;
    if (z_buffer && z_capacity < r->screen_count) return PF_CUDA_ERR_CAPACITY;
    if (fills && F) {
        std::vector<uint2> seg(F);
        std::vector<uint32_t> e(F);
        PF_TRY(cudaMemcpyAsync(seg.data(), r->fills.p, F * sizeof(uint2), cudaMemcpyDeviceToHost, s));
        PF_TRY(cudaMemcpyAsync(e.data(), r->fill_e.p, F * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        PF_TRY(cudaStreamSynchronize(s));
        for (uint64_t i = 0; i < F; i++)
            fills[i] = PFCUDAFill{(uint16_t)(seg[i].x & 0xffff), (uint16_t)(seg[i].x >> 16),
                                  (uint16_t)(seg[i].y & 0xffff), (uint16_t)(seg[i].y >> 16), e[i]};
    }
    if (fill_tile && F) {
        std::vector<uint32_t> base(T + 1);
        PF_TRY(cudaMemcpyAsync(base.data(), r->tile_fill_base.p, (T + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        PF_TRY(cudaStreamSynchronize(s));
        uint64_t g = 0;
        for (uint64_t i = 0; i < F; i++) {
            while (g + 1 <= T && base[g + 1] <= i) g++;
            fill_tile[i] = (uint32_t)g;
        }
    }
    if (tiles && T) {
        PF_TRY(cudaMemcpyAsync(tiles, r->tiles.p, T * sizeof(PFCUDATile), cudaMemcpyDeviceToHost, s));
        PF_TRY(cudaStreamSynchronize(s));
        // device records carry the global path index; report the index within
        // the clip paths or the draw paths, as TileObjectPrimitive::path_id
        for (uint64_t i = 0; i < T; i++)
            if (tiles[i].path_id >= r->nclip) tiles[i].path_id -= r->nclip;
    }
    if (clips && T) {
        PF_TRY(cudaMemcpyAsync(clips, r->clips.p, T * sizeof(PFCUDAClip), cudaMemcpyDeviceToHost, s));
        PF_TRY(cudaStreamSynchronize(s));
        // tiles of clip paths carry no clip record
        std::vector<uint32_t> off(r->P + 1);
        PF_TRY(cudaMemcpy(off.data(), r->tile_offset.p, (r->P + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        for (uint32_t gp = 0; gp < r->nclip; gp++)
            for (uint32_t g = off[gp]; g < off[gp + 1]; g++) clips[g] = PFCUDAClip{0xffffffffu, 0, 0xffffffffu, 0};
    }
    if (path_tile_offsets)
        PF_TRY(cudaMemcpyAsync(path_tile_offsets, r->tile_offset.p, (r->P + 1) * sizeof(uint32_t),
                               cudaMemcpyDeviceToHost, s));
    if (path_tile_rects && r->P)
        PF_TRY(cudaMemcpyAsync(path_tile_rects, r->tile_rect.p, r->P * sizeof(PFRectI), cudaMemcpyDeviceToHost, s));
    if (z_buffer && r->screen_count)
        PF_TRY(cudaMemcpyAsync(z_buffer, r->zbuf.p, r->screen_count * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    PF_TRY(cudaStreamSynchronize(s));
    return PF_CUDA_OK;
}

int32_t PFCUDASetProfiling(PFCUDARendererRef r, int32_t enable) {
    if (!r) return PF_CUDA_ERR_INVALID;
    PF_TRY(cudaSetDevice(r->device));
    if (enable && !r->stage_ev[0])
        for (int i = 0; i <= PF_CUDA_STAGE_COUNT; i++) PF_TRY(cudaEventCreate(&r->stage_ev[i]));
    r->profiling = enable != 0;
    return PF_CUDA_OK;
}

int32_t PFCUDAGetStageTimes(PFCUDARendererRef r, float* out_ms, int32_t capacity) {
    if (!r || !out_ms || capacity < PF_CUDA_STAGE_COUNT) return PF_CUDA_ERR_INVALID;
    if (!r->profiling) return PF_CUDA_ERR_INVALID;
    PF_TRY(cudaEventSynchronize(r->stage_ev[PF_CUDA_STAGE_COUNT]));
    for (int i = 0; i < PF_CUDA_STAGE_COUNT; i++) {
        float ms = 0;
        PF_TRY(cudaEventElapsedTime(&ms, r->stage_ev[i], r->stage_ev[i + 1]));
        out_ms[i] = ms;
    }
    return PF_CUDA_OK;
}

int32_t PFCUDAExclusiveScan(PFCUDARendererRef r, const uint32_t* in, uint32_t* out, uint32_t n) {
    if (!r || !out || (!in && n) || n >= 0x80000000u) return PF_CUDA_ERR_INVALID;
    PF_TRY(cudaSetDevice(r->device));
    PF_TRY(r->scan_partials.ensure((size_t)n / 2048 + 2));
    ScanTemp tmp{r->scan_partials.p, (uint32_t)r->scan_partials.cap};
    launch_scan(in, out, nullptr, n, n, 0, nullptr, tmp, r->stream);
    PF_TRY(cudaGetLastError());
    PF_TRY(cudaStreamSynchronize(r->stream));
    return PF_CUDA_OK;
}

int32_t PFCUDAGetStats(PFCUDARendererRef r, PFCUDARenderStats* out) {
    if (!r || !out) return PF_CUDA_ERR_INVALID;
    *out = r->stats;
    return PF_CUDA_OK;
}

const char* PFCUDAStatusString(int32_t status) {
    switch (status) {
        case PF_CUDA_OK: return "ok";
        case PF_CUDA_ERR_INVALID: return "invalid argument or malformed scene";
        case PF_CUDA_ERR_CAPACITY: return "device buffer capacity exceeded";
        case PF_CUDA_ERR_LAUNCH: return "CUDA call failed";
        case PF_CUDA_ERR_NO_DEVICE: return "no CUDA device";
        case PF_CUDA_ERR_LIMIT: return "a bounded device loop hit its limit";
        case PF_CUDA_ERR_NO_SCENE: return "no scene uploaded";
        default: return "unknown status";
    }
}

}  // extern "C"

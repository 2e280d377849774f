// pf_renderer.cu — host side of the CUDA renderer level and its C ABI.
//
// A frame replaces RendererD3D11::prepare_tiles / draw_tiles
// (renderer/src/gpu/d3d11/renderer.rs:414-782).  The reference sizes its
// buffers with three blocking readbacks and a regrow-and-retry loop
// (:218-229, :338-353, :463-499, :634-648).  Here every kernel checks the
// device-side totals against the buffer capacities, the frame is enqueued
// without any mid-frame synchronisation, and the single status readback at
// the end triggers a regrow and one re-run only when a capacity was exceeded
// (in steady state: never).
//
// The renderer holds a batch of scenes (one for the plain API).  Global path
// order is scene-major, each scene's clip paths before its draw paths, so the
// paths, segments and screen tiles of any contiguous range of scenes are
// contiguous and one frame covers such a range.
#include "pf_kernels.cuh"
#include <cuda.h>
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

// Pinned host staging for the scene tables built at upload. A copy from
// pageable memory waits for the driver's bounce buffer, so a dozen small
// tables cost a dozen round trips; from here each copy is one async enqueue.
// `done` is recorded after the last copy that reads the staging, and the next
// upload waits on it before writing.
struct HostStage {
    uint8_t* p = nullptr;
    size_t cap = 0, used = 0;
    cudaEvent_t done = nullptr;
    bool pending = false;
    cudaError_t begin(size_t n) {
        cudaError_t e = cudaSuccess;
        if (pending && (e = cudaEventSynchronize(done))) return e;
        pending = false;
        used = 0;
        if (n <= cap && p) return cudaSuccess;
        if (p) { cudaFreeHost(p); p = nullptr; cap = 0; }
        const size_t want = std::max<size_t>(n, 1u << 16);
        if ((e = cudaHostAlloc((void**)&p, want, cudaHostAllocDefault))) return e;
        cap = want;
        return cudaSuccess;
    }
    static size_t room(size_t bytes) { return (bytes + 15) & ~size_t(15); }
    template <typename T>
    T* take(size_t n) {
        T* q = (T*)(p + used);
        used += room(n * sizeof(T));
        return q;
    }
    template <typename T>
    const T* put(const std::vector<T>& v) {
        T* q = take<T>(v.size());
        if (!v.empty()) std::memcpy(q, v.data(), v.size() * sizeof(T));
        return q;
    }
    cudaError_t mark(cudaStream_t s) {
        if (!done) {
            cudaError_t e = cudaEventCreateWithFlags(&done, cudaEventDisableTiming);
            if (e) return e;
        }
        pending = true;
        return cudaEventRecord(done, s);
    }
    void release() {
        if (pending && done) cudaEventSynchronize(done);
        if (p) cudaFreeHost(p);
        if (done) cudaEventDestroy(done);
        p = nullptr; cap = 0; done = nullptr; pending = false;
    }
};

inline int32_t cvt_rne_host(float x) {
    if (!(x >= -2147483648.0f && x < 2147483648.0f)) return INT32_MIN;
    return (int32_t)std::nearbyint(x);
}

struct SceneInfo {
    uint32_t first_path = 0, nclip = 0, ndraw = 0;
    uint32_t seg_begin = 0, seg_end = 0;
    uint32_t screen_offset = 0, screen_count = 0;
    PFRectF view_box{};
    int4 screen{0, 0, 0, 0};
    bool has_target = false;
    bool explicit_target = false;  // given at upload: plain renders keep it
    PFCUDASceneTarget target{};
};

struct Range {
    uint32_t s0 = 0, s1 = 0;     // scenes
    uint32_t p0 = 0, p1 = 0;     // paths
    uint32_t g0 = 0, g1 = 0;     // segments
    uint32_t st0 = 0, st1 = 0;   // screen tiles
};

const TuneParams kDefaultTune{128, 256, 32, 4, 2, 0};

}  // namespace

struct PFCUDARenderer {
    int device = 0;
    uint32_t sms = 1;                  // multiprocessors of the device (grid sizes)
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    // Uploads copy the points on their own stream, beside the packing
    // kernels (which read only the point flags); the frame stream waits on
    // points_done before anything that reads points.
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t points_done = nullptr, prior_done = nullptr;
    // A frame runs two pairs of independent stages side by side: flattening
    // beside the bounds and path scans, and the fill emission beside
    // propagation and visibility.  The second branch of each pair runs on
    // branch_stream, forked from and joined back to the frame's stream.
    cudaStream_t branch_stream = nullptr;
    cudaStream_t column_stream = nullptr;  // the column backdrops, beside the tile scan
    cudaEvent_t fork_ev[3] = {}, join_ev[3] = {};
    PFCUDARendererOptions options{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    // scenes (resident)
    bool has_scene = false;
    uint32_t P = 0, NP = 0, NC = 0, nord = 0, S = 0, screen_total = 0;
    std::vector<SceneInfo> scenes;
    DevBuf<float2> pts, pts_t;
    DevBuf<uint8_t> flags;
    DevBuf<uint32_t> starts, ord_contour, ord_path, contour_segs, contour_seg_base;
    uint32_t ord_cap = 0;               // contour references the order buffers hold
    // upload staging on the device: the caller's records and the packing results
    DevBuf<uint32_t> starts_raw, path_ncont, scene_ranges;
    DevBuf<PFCUDAPath> path_in;
    DevBuf<ScenePackDev> scene_pack;
    DevBuf<PackInfo> pack_info;
    DevBuf<uint8_t> overlay_opaque;
    DevBuf<float> alpha_default;        // paint alpha / 255 per draw path (the default alpha)
    DevBuf<SegRec> segs;
    DevBuf<uint32_t> first_ord, paint, local_index, scene_of;
    DevBuf<int32_t> clip_gpath;
    DevBuf<uint8_t> rule, is_clip, blend, occludes;
    DevBuf<uint32_t> overlay, texels;
    DevBuf<OverlayDev> overlays;
    DevBuf<SceneDev> scenes_dev;
    std::vector<SceneDev> scenes_host;
    DevBuf<uint32_t> scene_st;             // each scene's first global screen tile
    std::vector<uint32_t> scene_st_host;

    // per-frame buffers
    DevBuf<int4> tile_rect;
    DevBuf<PathCtx> path_bin;
    DevBuf<uint32_t> tile_offset, col_offset;
    DevBuf<uint32_t> seg_line_count, seg_line_base, seg_warp;
    DevBuf<unsigned long long> seg_leaves;
    DevBuf<float4> lines;
    DevBuf<uint32_t> line_path, line_fill_count, line_fill_base;
    DevBuf<uint32_t> tile_fill_count, tile_fill_base, tile_alpha, alpha_owner;
    DevBuf<int32_t> tile_delta, col_backdrop, zbuf;
    DevBuf<uint32_t> tile_delta_scan, path_tiles, path_cols;
    DevBuf<uint2> fills;
    DevBuf<uint32_t> fill_e;
    DevBuf<int4> tiles, clips;
    DevBuf<uint32_t> screen_cnt, screen_base, vis;
    DevBuf<int4> vis_info;
    DevBuf<unsigned long long> vis_key;
    DevBuf<uint4> vis_mask;
    DevBuf<int4> mask_items;
    DevBuf<uint32_t> scan_partials, scan_partials_branch;
    // look-back words of the frame's single-pass scans: one half for the
    // frame's stream, one for its branch stream; cleared at the frame's start
    DevBuf<unsigned long long> scan_lookback;
    DevBuf<Counters> counters;
    DevBuf<uint8_t> out_tmp;
    Counters* h_counters = nullptr;  // pinned
    HostStage stage;                 // pinned scene tables

    uint32_t tile_cap = 0, col_cap = 0, fill_cap = 0, vis_cap = 0, line_cap = 0;
    Range last;
    PFCUDARenderStats stats{};
    bool profiling = false;
    cudaEvent_t stage_ev[PF_CUDA_STAGE_COUNT + 1] = {};
    uint64_t launches = 0;
    TuneParams tune = kDefaultTune;

    // captured frame, and the launch key it was captured with: every pointer,
    // size and option its kernels read (a buffer regrown since makes the
    // graph stale, and PFCUDAGraphLaunch refuses it)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    std::vector<uint8_t> graph_key;
    PFCUDABuildOptions graph_opts{};
    bool graph_has_opts = false;
    int graph_format = 0;
    void* graph_out = nullptr;
    Range graph_range;

    // plain frames replayed from a graph while their key (every pointer, size
    // and option that a launch of the frame reads) repeats
    std::vector<uint8_t> replay_key;
    cudaGraphExec_t replay_exec = nullptr;

    // clip chains
    uint32_t clip_chain_max = 0;       // longest chain of clip paths behind a path
    bool nested_clips = false;         // some clip path is itself clipped
    bool paint_effects = false;        // some path has a gradient or a blend mode other than SrcOver
    StrokeWork* stroke = nullptr;      // stroke-to-fill work buffers, made on first use

    // differentiable frames
    uint32_t ND = 0;                   // draw paths of the batch
    DevBuf<uint32_t> draw_index;       // [P] path -> draw path index (kInvalid for clip paths)
    DevBuf<float> alpha_in;            // [ND] alpha of the current differentiable frame
    DevBuf<float4> fills_f;
    DevBuf<uint32_t> line_seg;
    DevBuf<float2> line_t;
    DevBuf<uint32_t> tape;
    DevBuf<float> grad_mask, grad_alpha_tmp;
    bool diff_buffers = false;         // allocate the buffers above with the frame's
    bool last_diff = false;            // the last enqueued frame was differentiable
    // Fill emission indices are written only by a frame that PFCUDAReadRecords
    // runs for them (fill_order); last_opts is the options of the last frame.
    bool fill_order = false, last_fill_order = false;
    PFCUDABuildOptions last_opts{};
    bool diff_valid = false;           // PFCUDABackward may run on the last frame
    Range diff_range;
    bool diff_transformed = false;
    float diff_m4[4] = {1, 0, 0, 1};
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

// Makes the renderer's device current for the duration of an entry point and
// restores the caller's device afterwards.
struct DeviceGuard {
    int prev = -1;
    cudaError_t status = cudaSuccess;
    explicit DeviceGuard(int device) {
        if ((status = cudaGetDevice(&prev)) != cudaSuccess) { prev = -1; return; }
        if (prev != device) status = cudaSetDevice(device);
        else prev = -1;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int4 screen_rect_of(PFRectF v) {
    // round_rect_out_to_tile_bounds (renderer/src/tiles.rs:64-66)
    const float q = 1.0f / 16.0f;
    return make_int4(cvt_rne_host(std::floor(v.origin.x * q)), cvt_rne_host(std::floor(v.origin.y * q)),
                     cvt_rne_host(std::ceil(v.lower_right.x * q)), cvt_rne_host(std::ceil(v.lower_right.y * q)));
}

Range make_range(const PFCUDARenderer* r, uint32_t s0, uint32_t count) {
    Range g;
    g.s0 = s0;
    g.s1 = s0 + count;
    const SceneInfo& a = r->scenes[s0];
    const SceneInfo& b = r->scenes[g.s1 - 1];
    g.p0 = a.first_path;
    g.p1 = b.first_path + b.nclip + b.ndraw;
    g.g0 = a.seg_begin;
    g.g1 = b.seg_end;
    g.st0 = a.screen_offset;
    g.st1 = b.screen_offset + b.screen_count;
    return g;
}

FrameDev frame_dev(PFCUDARenderer* r, bool transformed, const Range& g, bool diff = false) {
    FrameDev f{};
    f.diff = diff ? 1 : 0;
    f.d3d11 = (!diff && (r->options.flags & PF_CUDA_RENDERER_D3D11_SEMANTICS)) ? 1 : 0;
    f.path.alpha_f = diff ? r->alpha_in.p : nullptr;
    f.path.draw_index = r->draw_index.p;
    f.fills_f = r->fills_f.p;
    f.line_seg = r->line_seg.p;
    f.line_t = r->line_t.p;
    f.tape = r->tape.p;
    f.pts = transformed ? r->pts_t.p : r->pts.p;
    f.segs = r->segs.p;
    f.seg_begin = g.g0;
    f.seg_count = g.g1 - g.g0;
    f.path.first_ord_contour = r->first_ord.p;
    f.path.paint = r->paint.p;
    f.path.clip_gpath = r->clip_gpath.p;
    f.path.rule = r->rule.p;
    f.path.is_clip = r->is_clip.p;
    f.path.blend = r->blend.p;
    f.path.overlay = r->overlay.p;
    f.path.occludes = r->occludes.p;
    f.overlays = r->overlays.p;
    f.texels = r->texels.p;
    f.inv_m[0] = 1.0f; f.inv_m[4] = 1.0f;
    f.path.local_index = r->local_index.p;
    f.path.scene = r->scene_of.p;
    f.path.tile_rect = r->tile_rect.p;
    f.path_bin = r->path_bin.p;
    f.path.tile_offset = r->tile_offset.p;
    f.path.col_offset = r->col_offset.p;
    f.scenes = r->scenes_dev.p;
    f.scene_st = r->scene_st.p;
    f.path_begin = g.p0;
    f.path_count = g.p1 - g.p0;
    f.scene_begin = g.s0;
    f.scene_count = g.s1 - g.s0;
    f.screen_begin = g.st0;
    f.tune = r->tune;
    f.sms = r->sms;
    f.tile_cap = r->tile_cap;
    f.col_cap = r->col_cap;
    f.fill_cap = r->fill_cap;
    f.vis_cap = r->vis_cap;
    f.screen_count = g.st1 - g.st0;
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
    // two arrays of one value per warp of 32 segments (+ the scan total)
    f.seg_warp_lines = r->seg_warp.p;
    f.seg_warp_base = r->seg_warp.p ? r->seg_warp.p + ((size_t)r->S + 31) / 32 + 2 : nullptr;
    f.seg_leaves = r->seg_leaves.p;
    f.lines = r->lines.p;
    f.line_path = r->line_path.p;
    f.line_fill_count = r->line_fill_count.p;
    f.line_fill_base = r->line_fill_base.p;
    f.line_cap = r->line_cap;
    f.fills = r->fills.p;
    f.fill_e = r->fill_order ? r->fill_e.p : nullptr;
    f.tiles = r->tiles.p;
    f.clips = r->clips.p;
    f.alpha_owner = r->alpha_owner.p;
    f.zbuf = r->zbuf.p;
    f.screen_cnt = r->screen_cnt.p;
    f.screen_base = r->screen_base.p;
    f.vis = r->vis.p;
    f.vis_info = r->vis_info.p;
    f.vis_key = r->vis_key.p;
    f.vis_mask = r->vis_mask.p;
    f.mask_items = r->mask_items.p;
    f.counters = r->counters.p;
    f.dda_limit = 1u << 24;
    f.clip_chain_max = r->clip_chain_max;
    f.paint_effects = r->paint_effects ? 1u : 0u;
    return f;
}

cudaError_t ensure_frame_buffers(PFCUDARenderer* r) {
    cudaError_t e;
    const size_t T = (size_t)r->tile_cap + 1, L = (size_t)r->line_cap + 1, F = (size_t)r->fill_cap + 1;
    const size_t ST = (size_t)r->screen_total + 1, P = (size_t)r->P + 1;
    if ((e = r->tile_fill_count.ensure(T)) || (e = r->tile_fill_base.ensure(T)) || (e = r->tile_alpha.ensure(T)) ||
        (e = r->alpha_owner.ensure(T)) || (e = r->tile_delta.ensure(T)) || (e = r->tile_delta_scan.ensure(T)) ||
        (e = r->tiles.ensure(T)) || (e = r->clips.ensure(T)) || (e = r->col_backdrop.ensure((size_t)r->col_cap + 1)) ||
        (e = r->fills.ensure(F)) || (e = r->fill_e.ensure(F)) || (e = r->lines.ensure(L)) ||
        (e = r->line_path.ensure(L)) || (e = r->line_fill_count.ensure(L)) || (e = r->line_fill_base.ensure(L)) ||
        (e = r->vis.ensure((size_t)r->vis_cap + 1)) || (e = r->vis_info.ensure((size_t)r->vis_cap + 1)) ||
        (e = r->vis_key.ensure((size_t)r->vis_cap + 1)) || (e = r->vis_mask.ensure(((size_t)r->vis_cap + 1) * 32)) ||
        (e = r->mask_items.ensure((size_t)r->vis_cap + 1)) || (e = r->zbuf.ensure(ST)) || (e = r->screen_cnt.ensure(ST)) ||
        (e = r->screen_base.ensure(ST)) || (e = r->path_tiles.ensure(P)) || (e = r->path_cols.ensure(P)))
        return e;
    if (r->diff_buffers) {
        const size_t V = ((size_t)r->vis_cap + 1) * 256;
        if ((e = r->fills_f.ensure(F)) || (e = r->line_seg.ensure(L)) || (e = r->line_t.ensure(L)) ||
            (e = r->tape.ensure(V)))
            return e;
    }
    size_t nmax = std::max<size_t>({(size_t)r->tile_cap, (size_t)r->S, (size_t)r->screen_total, (size_t)r->nord,
                                    (size_t)r->line_cap, (size_t)r->P}) + 1;
    if ((e = r->scan_partials_branch.ensure(kMaxScanLanes * ((size_t)r->S + 1) / 2048 + 2 * kMaxScanLanes)))
        return e;
    // per half: a ticket and one word per tile and lane for each of the frame's scans
    if ((e = r->scan_lookback.ensure(2 * (16 + 3 * kMaxScanLanes * (nmax / 2048 + 2))))) return e;
    return r->scan_partials.ensure(kMaxScanLanes * (nmax / 2048 + 2));
}

float4 background_of(const PFCUDARenderer* r) {
    if (!r->options.has_background_color) return make_float4(0, 0, 0, 0);
    return make_float4(r->options.background_color.r, r->options.background_color.g, r->options.background_color.b,
                       r->options.background_color.a);
}

bool is_identity(const PFCUDABuildOptions* o) {
    if (!o || !o->has_transform) return true;
    const PFTransform2F& t = o->transform;
    return t.m00 == 1.0f && t.m01 == 0.0f && t.m10 == 0.0f && t.m11 == 1.0f && t.vector.x == 0.0f &&
           t.vector.y == 0.0f;
}

// Enqueue one frame over range g.  mode: PF_CUDA_FORMAT_*, or -1 for no
// composite.  diff: a differentiable frame (FP32 fills, FP32 output and the
// adjoint's tape; mode is ignored).
cudaError_t enqueue_frame(PFCUDARenderer* r, const PFCUDABuildOptions* opts, int mode, void* out_dev, const Range& g,
                          bool diff = false) {
    cudaStream_t s = r->stream;
    bool transformed = !is_identity(opts);
    cudaError_t e;
    // each frame kernel may start while its predecessor on its stream drains
    PdlScope pdl(true);
    if (transformed) {
        if ((e = r->pts_t.ensure(r->NP))) return e;
        float m6[6] = {opts->transform.m00, opts->transform.m01, opts->transform.m10, opts->transform.m11,
                       opts->transform.vector.x, opts->transform.vector.y};
        launch_transform(r->pts.p, r->pts_t.p, r->NP, m6, s);
    }
    r->last_diff = diff;
    r->last_fill_order = r->fill_order;
    if (opts != &r->last_opts) r->last_opts = opts ? *opts : PFCUDABuildOptions{};
    if (!diff) r->diff_valid = false;
    FrameDev f = frame_dev(r, transformed, g, diff);
    if (transformed) {  // gradients are evaluated at pixel centres mapped back to scene space
        const PFTransform2F& t = opts->transform;
        const float det = t.m00 * t.m11 - t.m01 * t.m10;
        if (det != 0.0f) {
            const float inv = 1.0f / det;
            const float a = t.m11 * inv, b = -t.m01 * inv, c = -t.m10 * inv, d = t.m00 * inv;
            f.inv_m[0] = a; f.inv_m[1] = b; f.inv_m[2] = -(a * t.vector.x + b * t.vector.y);
            f.inv_m[3] = c; f.inv_m[4] = d; f.inv_m[5] = -(c * t.vector.x + d * t.vector.y);
        }
    }
    Counters* c = r->counters.p;
    const uint32_t half = (uint32_t)(r->scan_lookback.cap / 2);
    ScanTemp tmp{r->scan_partials.p, (uint32_t)r->scan_partials.cap, r->scan_lookback.p, half, 0, &c->status};
    ScanTemp tmp_branch{r->scan_partials_branch.p, (uint32_t)r->scan_partials_branch.cap, r->scan_lookback.p + half,
                        half, 0, &c->status};
    auto mark = [&](int stage) {
        if (r->profiling) cudaEventRecord(r->stage_ev[stage], s);
    };
    // Stage-timed frames run every kernel on the frame's stream, in order.
    const bool branches = !r->profiling;
    cudaStream_t b = branches ? r->branch_stream : s;
    cudaStream_t bc = branches ? r->column_stream : s;
    auto fork = [&](int k, cudaStream_t to) -> cudaError_t {
        if (!branches) return cudaSuccess;
        cudaError_t e1 = cudaEventRecord(r->fork_ev[k], s);
        return e1 ? e1 : cudaStreamWaitEvent(to, r->fork_ev[k], 0);
    };
    auto join = [&](int k, cudaStream_t from) -> cudaError_t {
        if (!branches) return cudaSuccess;
        cudaError_t e1 = cudaEventRecord(r->join_ev[k], from);
        return e1 ? e1 : cudaStreamWaitEvent(s, r->join_ev[k], 0);
    };
    const size_t nst = (size_t)(g.st1 - g.st0) + 1;
    uint64_t before = launch_counter();
    if ((e = cudaMemsetAsync(c, 0, sizeof(Counters), s))) return e;
    if ((e = cudaMemsetAsync(r->scan_lookback.p, 0, r->scan_lookback.cap * sizeof(unsigned long long), s))) return e;
    mark(0);
    // flattening needs no tile rects: it runs beside the bounds and path scans
    if ((e = fork(0, b))) return e;
    launch_bound(f, r->ord_contour.p, r->starts.p, s);
    launch_path_scan(f, tmp, s);
    mark(1);
    launch_flatten(f, branches ? tmp_branch : tmp, b);
    if ((e = join(0, b))) return e;
    mark(2);
    launch_bin_count(f, s);
    mark(3);
    // the column backdrops need only the count pass: they run beside the
    // scans (in stage-timed frames, in the scans' stage)
    if ((e = fork(2, bc))) return e;
    launch_column_backdrops(f, bc);
    // the first fill of each line in emission order: only frames run for
    // record read-back write emission indices
    if (r->fill_order)
        launch_scan(r->line_fill_count.p, r->line_fill_base.p, &c->lines, 0, r->line_cap, 0, &c->fills, tmp, s);
    {
        // per tile: alpha-tile ids, fill offsets (their total is the frame's
        // fill count) and, over the counts, each tile's fill end: the emit
        // pass's cursor, counted down to the tile's offset
        ScanLanes lanes{};
        lanes.count = 2;
        lanes.in[0] = r->tile_fill_count.p; lanes.out[0] = r->tile_alpha.p; lanes.mode[0] = 1;
        lanes.total[0] = &c->alpha_tiles;
        lanes.in[1] = r->tile_fill_count.p; lanes.out[1] = r->tile_fill_base.p; lanes.mode[1] = 0;
        lanes.total[1] = &c->fills;
        lanes.incl[1] = r->tile_fill_count.p;
        launch_scan_multi(lanes, &c->tiles, r->tile_cap, tmp, s);
    }
    mark(4);
    // propagation and visibility read the tile scans, not the fills: the fill
    // emission runs beside them
    if ((e = fork(1, b))) return e;
    launch_bin_emit(f, b);
    mark(5);
    // clip paths first: draw tiles of clipped paths read their clip's finished tiles
    if ((e = join(2, bc))) return e;
    launch_propagate(f, true, s);
    launch_propagate(f, false, s);
    mark(6);
    launch_visible(f, false, s);
    launch_scan(r->screen_cnt.p, r->screen_base.p, nullptr, (uint32_t)(nst - 1), (uint32_t)(nst - 1), 0, &c->visible,
                tmp, s);
    launch_visible(f, true, s);
    if ((e = join(1, b))) return e;
    mark(7);
    if (mode >= 0 && !diff) launch_mask(f, s);
    mark(8);
    if (mode >= 0 || diff) {
        const float4 bg = background_of(r);
        if (diff) launch_composite_diff(f, (float*)out_dev, bg, s);
        else launch_composite(f, mode, out_dev, bg, s);
    }
    mark(9);
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
    if (h.status & kStatusLineCapacity) r->line_cap = std::max(r->line_cap, up(h.lines + h.lines_back));
    if (h.status & kStatusVisibleCapacity) r->vis_cap = std::max(r->vis_cap, up(h.visible));
}

const uint32_t kCapacityBits = kStatusTileCapacity | kStatusColumnCapacity | kStatusFillCapacity |
                               kStatusVisibleCapacity | kStatusAlphaCapacity | kStatusLineCapacity;

int32_t status_to_code(uint32_t st) {
    if (st & kCapacityBits) return PF_CUDA_ERR_CAPACITY;
    if (st & (kStatusDdaLimit | kStatusDepthLimit)) return PF_CUDA_ERR_LIMIT;
    if (st & kStatusMalformed) return PF_CUDA_ERR_INVALID;
    if (st & kStatusScanStall) return PF_CUDA_ERR_LAUNCH;
    return PF_CUDA_OK;
}

void record_stats(PFCUDARenderer* r, const Counters& h, float ms) {
    r->stats.path_count = r->last.p1 - r->last.p0;
    r->stats.segment_count = r->last.g1 - r->last.g0;
    r->stats.line_count = h.lines + h.lines_back;
    r->stats.fill_count = h.fills;
    r->stats.tile_count = h.tiles;
    r->stats.alpha_tile_count = h.alpha_tiles;
    r->stats.visible_tile_count = h.visible;
    r->stats.screen_tile_count = r->last.st1 - r->last.st0;
    r->stats.status = h.status;
    r->stats.gpu_time_ms = ms;
    r->stats.kernel_launches = r->launches;
    r->stats.mask_tile_count = h.mask_items;
    r->stats.mask_fill_count = h.mask_fills;
}

cudaError_t upload_scene_records(PFCUDARenderer* r) {
    cudaError_t e = cudaMemcpyAsync(r->scenes_dev.p, r->scenes_host.data(), sizeof(SceneDev) * r->scenes_host.size(),
                                    cudaMemcpyHostToDevice, r->stream);
    if (e) return e;
    // each scene's first screen tile, packed: the composite's screen-tile ->
    // scene search reads these 4-byte words instead of the scene records
    r->scene_st_host.resize(r->scenes_host.size());
    for (size_t k = 0; k < r->scenes_host.size(); k++) r->scene_st_host[k] = r->scenes_host[k].screen_offset;
    if ((e = r->scene_st.ensure(r->scene_st_host.size() + 1))) return e;
    return cudaMemcpyAsync(r->scene_st.p, r->scene_st_host.data(), sizeof(uint32_t) * r->scene_st_host.size(),
                           cudaMemcpyHostToDevice, r->stream);
}

void set_target(PFCUDARenderer* r, uint32_t k, const PFCUDASceneTarget& t) {
    r->scenes[k].target = t;
    r->scenes[k].has_target = true;
    SceneDev& d = r->scenes_host[k];
    d.clip = make_int4(t.clip.origin.x, t.clip.origin.y, t.clip.lower_right.x, t.clip.lower_right.y);
    d.origin_x = t.origin_x;
    d.origin_y = t.origin_y;
    d.pitch = t.pitch;
    d.out_offset = t.out_offset;
}

// The scene of global path gp (the last scene starting at or before it).
const SceneInfo& scene_of_path(const PFCUDARenderer* r, uint32_t gp) {
    auto it = std::upper_bound(r->scenes.begin(), r->scenes.end(), gp,
                               [](uint32_t v, const SceneInfo& si) { return v < si.first_path; });
    return it == r->scenes.begin() ? r->scenes.front() : *(it - 1);
}

bool path_is_clip_of(const PFCUDARenderer* r, uint32_t gp) {
    const SceneInfo& si = scene_of_path(r, gp);
    return gp - si.first_path < si.nclip;
}

// Index of global path gp within its scene's clip paths or draw paths.
uint32_t path_local_of(const PFCUDARenderer* r, uint32_t gp, bool* is_clip) {
    const SceneInfo& si = scene_of_path(r, gp);
    const uint32_t i = gp - si.first_path;
    if (is_clip) *is_clip = i < si.nclip;
    return i < si.nclip ? i : i - si.nclip;
}

bool valid_range(const PFCUDARenderer* r, uint32_t first, uint32_t count) {
    return r->has_scene && count > 0 && first < r->scenes.size() && count <= r->scenes.size() - first;
}

// Everything the launches of a plain frame read on the host: two frames with
// equal keys enqueue the same kernels with the same arguments. Scene contents
// stay out of it: they are read on the device, so a graph of the frame
// replays correctly after an upload that kept every buffer and size.
std::vector<uint8_t> frame_key(PFCUDARenderer* r, const PFCUDABuildOptions* opts, int mode, void* out_dev,
                               const Range& g) {
    const bool transformed = !is_identity(opts);
    const FrameDev f = frame_dev(r, transformed, g, false);
    std::vector<uint8_t> k;
    auto put = [&k](const void* p, size_t n) { k.insert(k.end(), (const uint8_t*)p, (const uint8_t*)p + n); };
    put(&f, sizeof f);
    const void* ptrs[] = {r->pts.p, r->ord_contour.p, r->starts.p, r->scan_partials.p, r->scan_partials_branch.p,
                          r->scan_lookback.p, out_dev};
    put(ptrs, sizeof ptrs);
    const uint64_t vals[] = {r->scan_partials.cap, r->scan_partials_branch.cap, r->scan_lookback.cap, r->NP,
                             (uint64_t)(int64_t)mode, transformed ? 1u : 0u};
    put(vals, sizeof vals);
    const float4 bg = background_of(r);
    put(&bg, sizeof bg);
    if (transformed) put(&opts->transform, sizeof opts->transform);
    return k;
}

void drop_replay(PFCUDARenderer* r) {
    if (r->replay_exec) cudaGraphExecDestroy(r->replay_exec);
    r->replay_exec = nullptr;
    r->replay_key.clear();
}

// A plain frame whose key repeats the previous one's runs as one graph
// launch, captured at the key's second frame (a key seen once is not worth a
// capture); any other frame is enqueued kernel by kernel.
cudaError_t enqueue_plain(PFCUDARenderer* r, const PFCUDABuildOptions* opts, int mode, void* out_dev, const Range& g) {
    std::vector<uint8_t> key = frame_key(r, opts, mode, out_dev, g);
    if (key != r->replay_key) {
        drop_replay(r);
        r->replay_key.swap(key);
        return enqueue_frame(r, opts, mode, out_dev, g);
    }
    if (!r->replay_exec) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(r->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
            (void)cudaGetLastError();
            return enqueue_frame(r, opts, mode, out_dev, g);
        }
        cudaError_t e = cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            return enqueue_frame(r, opts, mode, out_dev, g);
        }
        cudaGraph_t graph = nullptr;
        const cudaError_t e1 = enqueue_frame(r, opts, mode, out_dev, g);
        const cudaError_t e2 = cudaStreamEndCapture(r->stream, &graph);
        if (e1 != cudaSuccess || e2 != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return e1 != cudaSuccess ? e1 : e2;
        }
        e = cudaGraphInstantiate(&r->replay_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            r->replay_exec = nullptr;
            return e;
        }
    }
    r->last_diff = false;
    r->last_fill_order = r->fill_order;  // part of the key
    if (opts != &r->last_opts) r->last_opts = opts ? *opts : PFCUDABuildOptions{};
    r->diff_valid = false;
    return cudaGraphLaunch(r->replay_exec, r->stream);
}

// A device-to-host copy enqueued after a frame and before its status read.
struct ImageCopy {
    void* dst;
    const void* src;
    size_t bytes;
};

// Run one frame synchronously with regrow-and-retry; `copy` (optional) is
// enqueued behind each attempt, so the one synchronisation covers it.
int32_t run_frame(PFCUDARenderer* r, const PFCUDABuildOptions* opts, int mode, void* out_dev, const Range& g,
                  bool diff = false, const ImageCopy* copy = nullptr) {
    if (!r->has_scene) return PF_CUDA_ERR_NO_SCENE;
    r->last = g;
    for (int attempt = 0; attempt < 4; attempt++) {
        PF_TRY(ensure_frame_buffers(r));
        PF_TRY(cudaEventRecord(r->ev0, r->stream));
        if (diff || r->profiling) PF_TRY(enqueue_frame(r, opts, mode, out_dev, g, diff));
        else PF_TRY(enqueue_plain(r, opts, mode, out_dev, g));
        PF_TRY(cudaEventRecord(r->ev1, r->stream));
        if (copy) PF_TRY(cudaMemcpyAsync(copy->dst, copy->src, copy->bytes, cudaMemcpyDeviceToHost, r->stream));
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

void release_graph(PFCUDARenderer* r) {
    if (r->graph_exec) cudaGraphExecDestroy(r->graph_exec);
    if (r->graph) cudaGraphDestroy(r->graph);
    r->graph_exec = nullptr;
    r->graph = nullptr;
    r->graph_key.clear();
}

// Single-image rendering: scenes uploaded without targets draw into the
// width x height image (row 0 = top of the view box's pixel grid).
int32_t prepare_plain_targets(PFCUDARenderer* r, int32_t width, int32_t height, bool* changed) {
    if (width <= 0 || height <= 0) return PF_CUDA_ERR_INVALID;
    *changed = false;
    for (uint32_t k = 0; k < r->scenes.size(); k++) {
        if (r->scenes[k].explicit_target) continue;
        if (r->scenes[k].has_target) {
            const PFCUDASceneTarget& t = r->scenes[k].target;
            if (t.out_offset == 0 && t.origin_x == 0 && t.origin_y == 0 && t.pitch == width &&
                t.clip.lower_right.x == width && t.clip.lower_right.y == height && t.clip.origin.x == 0 &&
                t.clip.origin.y == 0)
                continue;
        }
        PFCUDASceneTarget t{};
        t.pitch = width;
        t.clip = PFRectI{{0, 0}, {width, height}};
        set_target(r, k, t);
        *changed = true;
    }
    return PF_CUDA_OK;
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
    if (options && (options->flags & ~PF_CUDA_RENDERER_D3D11_SEMANTICS)) return PF_CUDA_ERR_INVALID;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return PF_CUDA_ERR_NO_DEVICE;
    if (device_ordinal < 0 || device_ordinal >= count) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(device_ordinal);
    PF_TRY(dg.status);
    int sms = 0;
    PF_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_ordinal));
    PFCUDARenderer* r = new PFCUDARenderer();
    r->device = device_ordinal;
    r->sms = sms > 0 ? (uint32_t)sms : 1u;
    if (options) r->options = *options;
    if ((e = cudaStreamCreateWithFlags(&r->own_stream, cudaStreamNonBlocking)) ||
        (e = cudaStreamCreateWithFlags(&r->copy_stream, cudaStreamNonBlocking)) ||
        (e = cudaEventCreateWithFlags(&r->points_done, cudaEventDisableTiming)) ||
        (e = cudaEventCreateWithFlags(&r->prior_done, cudaEventDisableTiming)) ||
        (e = cudaStreamCreateWithFlags(&r->branch_stream, cudaStreamNonBlocking)) ||
        (e = cudaStreamCreateWithFlags(&r->column_stream, cudaStreamNonBlocking)) ||
        (e = cudaEventCreateWithFlags(&r->fork_ev[0], cudaEventDisableTiming)) ||
        (e = cudaEventCreateWithFlags(&r->fork_ev[1], cudaEventDisableTiming)) ||
        (e = cudaEventCreateWithFlags(&r->fork_ev[2], cudaEventDisableTiming)) ||
        (e = cudaEventCreateWithFlags(&r->join_ev[0], cudaEventDisableTiming)) ||
        (e = cudaEventCreateWithFlags(&r->join_ev[1], cudaEventDisableTiming)) ||
        (e = cudaEventCreateWithFlags(&r->join_ev[2], cudaEventDisableTiming)) ||
        (e = cudaEventCreate(&r->ev0)) || (e = cudaEventCreate(&r->ev1)) ||
        (e = cudaMallocHost((void**)&r->h_counters, sizeof(Counters))) || (e = r->counters.ensure(1))) {
        PFCUDARendererDestroy(r);
        return cuda_status(e);
    }
    r->stream = r->own_stream;
    *out_renderer = r;
    return PF_CUDA_OK;
}

int32_t PFCUDARendererDestroy(PFCUDARendererRef r) {
    if (!r) return PF_CUDA_OK;
    DeviceGuard dg(r->device);
    if (r->stream) cudaStreamSynchronize(r->stream);
    release_graph(r);
    r->pts.release(); r->pts_t.release(); r->flags.release(); r->starts.release();
    r->ord_contour.release(); r->ord_path.release(); r->contour_segs.release(); r->contour_seg_base.release();
    r->segs.release(); r->first_ord.release(); r->paint.release(); r->local_index.release();
    r->scene_of.release(); r->clip_gpath.release(); r->rule.release(); r->is_clip.release();
    r->scenes_dev.release(); r->scene_st.release(); r->tile_rect.release(); r->tile_offset.release(); r->col_offset.release();
    r->seg_line_count.release(); r->seg_line_base.release(); r->seg_warp.release(); r->lines.release(); r->line_path.release();
    r->seg_leaves.release(); r->path_bin.release();
    r->line_fill_count.release(); r->line_fill_base.release(); r->tile_fill_count.release();
    r->tile_fill_base.release(); r->tile_alpha.release(); r->alpha_owner.release(); r->tile_delta.release();
    r->tile_delta_scan.release(); r->path_tiles.release(); r->path_cols.release();
    r->col_backdrop.release(); r->zbuf.release(); r->fills.release(); r->fill_e.release(); r->tiles.release();
    r->clips.release(); r->screen_cnt.release(); r->screen_base.release(); r->vis.release(); r->vis_info.release();
    r->vis_key.release(); r->vis_mask.release(); r->mask_items.release();
    r->scan_partials.release(); r->scan_partials_branch.release(); r->scan_lookback.release(); r->counters.release();
    r->out_tmp.release();
    r->draw_index.release(); r->blend.release(); r->occludes.release(); r->overlay.release();
    r->starts_raw.release(); r->path_ncont.release(); r->scene_ranges.release(); r->path_in.release();
    r->scene_pack.release(); r->pack_info.release(); r->overlay_opaque.release(); r->alpha_default.release();
    r->overlays.release(); r->texels.release(); r->alpha_in.release(); r->fills_f.release(); r->line_seg.release();
    r->line_t.release(); r->tape.release();
    r->grad_mask.release(); r->grad_alpha_tmp.release();
    if (r->h_counters) cudaFreeHost(r->h_counters);
    r->stage.release();
    drop_replay(r);
    if (r->ev0) cudaEventDestroy(r->ev0);
    if (r->ev1) cudaEventDestroy(r->ev1);
    for (int i = 0; i <= PF_CUDA_STAGE_COUNT; i++)
        if (r->stage_ev[i]) cudaEventDestroy(r->stage_ev[i]);
    if (r->own_stream) cudaStreamDestroy(r->own_stream);
    if (r->copy_stream) {
        cudaStreamSynchronize(r->copy_stream);
        cudaStreamDestroy(r->copy_stream);
    }
    if (r->points_done) cudaEventDestroy(r->points_done);
    if (r->prior_done) cudaEventDestroy(r->prior_done);
    if (r->branch_stream) {
        cudaStreamSynchronize(r->branch_stream);
        cudaStreamDestroy(r->branch_stream);
    }
    if (r->column_stream) {
        cudaStreamSynchronize(r->column_stream);
        cudaStreamDestroy(r->column_stream);
    }
    for (int k = 0; k < 3; k++) {
        if (r->fork_ev[k]) cudaEventDestroy(r->fork_ev[k]);
        if (r->join_ev[k]) cudaEventDestroy(r->join_ev[k]);
    }
    stroke_work_destroy(r->stroke);
    delete r;
    return PF_CUDA_OK;
}

int32_t PFCUDARendererSetStream(PFCUDARendererRef r, void* stream) {
    if (!r) return PF_CUDA_ERR_INVALID;
    r->stream = stream ? (cudaStream_t)stream : r->own_stream;
    release_graph(r);
    return PF_CUDA_OK;
}

int32_t PFCUDARendererSetOptions(PFCUDARendererRef r, const PFCUDARendererOptions* options) {
    if (!r || !options || (options->flags & ~PF_CUDA_RENDERER_D3D11_SEMANTICS)) return PF_CUDA_ERR_INVALID;
    r->options = *options;
    release_graph(r);
    return PF_CUDA_OK;
}

// The scene tables of an upload whose point copies are already enqueued. The
// host lays out the scenes (O(scenes) work) and stages the caller's records;
// the per-path tables, the contour order, the clip chains and the segment
// records are built on the device (pf_pack.cu, then the segment kernels).
static int32_t upload_tables(PFCUDARendererRef r, const PFCUDASceneDesc* scenes, const PFCUDASceneTarget* targets,
                             uint32_t scene_count, uint64_t np_total, uint64_t nc_total, uint64_t P) {
    cudaStream_t s = r->stream;
    const size_t Pz = (size_t)P;
    const uint32_t nb = (uint32_t)nc_total;  // contour boundary slots: contours + 1 per scene
    std::vector<uint32_t> texels;
    std::vector<OverlayDev> overlays;
    std::vector<uint8_t> overlay_opaque;
    std::vector<ScenePackDev> packs(scene_count);
    r->scenes.assign(scene_count, SceneInfo());
    r->scenes_host.assign(scene_count, SceneDev{});
    uint32_t point_base = 0, contour_base = 0, gp = 0, screen_total = 0, draw_base = 0;
    for (uint32_t k = 0; k < scene_count; k++) {
        const PFCUDASceneDesc& sc = scenes[k];
        SceneInfo& si = r->scenes[k];
        si.first_path = gp;
        si.nclip = sc.clip_path_count;
        si.ndraw = sc.draw_path_count;
        si.view_box = sc.view_box;
        si.screen = screen_rect_of(sc.view_box);
        int32_t sw = std::max(0, si.screen.z - si.screen.x), sh = std::max(0, si.screen.w - si.screen.y);
        si.screen_offset = screen_total;
        si.screen_count = (uint32_t)sw * (uint32_t)sh;
        screen_total += si.screen_count;
        if ((sc.gradient_count && !sc.gradients) || (sc.pattern_count && !sc.patterns)) return PF_CUDA_ERR_INVALID;
        if ((uint64_t)overlays.size() + sc.gradient_count + sc.pattern_count > 0xfffeu)
            return PF_CUDA_ERR_INVALID;  // 16-bit overlay ids in the visible records
        const uint32_t ov_base = (uint32_t)overlays.size();
        for (uint32_t q = 0; q < sc.gradient_count + sc.pattern_count; q++) {
            OverlayDev od;
            bool opaque = false;
            const int32_t rc = q < sc.gradient_count
                                   ? build_gradient(sc.gradients[q], &od, texels, &opaque)
                                   : build_pattern(sc.patterns[q - sc.gradient_count], &od, texels, &opaque);
            if (rc != PF_CUDA_OK) return rc;
            overlays.push_back(od);
            overlay_opaque.push_back(opaque ? 1 : 0);
        }
        packs[k] = ScenePackDev{gp, sc.clip_path_count, sc.draw_path_count, contour_base, sc.contour_count,
                                point_base, sc.point_count, draw_base, ov_base, sc.gradient_count + sc.pattern_count};
        SceneDev& d = r->scenes_host[k];
        d.view_box = make_float4(sc.view_box.origin.x, sc.view_box.origin.y, sc.view_box.lower_right.x,
                                 sc.view_box.lower_right.y);
        d.screen = si.screen;
        d.screen_offset = si.screen_offset;
        d.first_path = si.first_path;
        d.clip_count = si.nclip;
        d.draw_count = si.ndraw;
        if (targets) {
            set_target(r, k, targets[k]);
            si.explicit_target = true;
        }
        gp += sc.clip_path_count + sc.draw_path_count;
        draw_base += sc.draw_path_count;
        point_base += sc.point_count;
        contour_base += sc.contour_count + 1;
    }

    // ---- device buffers --------------------------------------------------------
    // Contour references: one per contour of each path; more only when paths
    // share contours, found after packing (the buffers then grow and the
    // order is packed again).
    uint32_t cap = std::max(r->ord_cap, nb);
    cudaError_t e;
    auto ensure_order = [&](uint32_t c) -> cudaError_t {
        cudaError_t x;
        if ((x = r->ord_contour.ensure((size_t)c + 1)) || (x = r->ord_path.ensure((size_t)c + 1)) ||
            (x = r->contour_segs.ensure((size_t)c + 1)) || (x = r->contour_seg_base.ensure((size_t)c + 1)) ||
            (x = r->scan_partials.ensure(std::max<size_t>(Pz, c) / 2048 + 2)))
            return x;
        r->ord_cap = c;
        return cudaSuccess;
    };
    if ((e = ensure_order(cap)) || (e = r->starts.ensure((size_t)nb + 1)) || (e = r->starts_raw.ensure((size_t)nb + 1)) ||
        (e = r->path_in.ensure(Pz + 1)) || (e = r->scene_pack.ensure(scene_count)) ||
        (e = r->path_ncont.ensure(Pz + 1)) || (e = r->first_ord.ensure(Pz + 1)) || (e = r->paint.ensure(Pz + 1)) ||
        (e = r->local_index.ensure(Pz + 1)) || (e = r->scene_of.ensure(Pz + 1)) || (e = r->clip_gpath.ensure(Pz + 1)) ||
        (e = r->rule.ensure(Pz + 1)) || (e = r->is_clip.ensure(Pz + 1)) || (e = r->tile_rect.ensure(Pz + 1)) || (e = r->path_bin.ensure(Pz + 1)) ||
        (e = r->draw_index.ensure(Pz + 1)) || (e = r->alpha_default.ensure((size_t)draw_base + 1)) ||
        (e = r->blend.ensure(Pz + 1)) || (e = r->occludes.ensure(Pz + 1)) || (e = r->overlay.ensure(Pz + 1)) ||
        (e = r->overlays.ensure(overlays.size() + 1)) || (e = r->overlay_opaque.ensure(overlays.size() + 1)) ||
        (e = r->texels.ensure(texels.size() + 1)) || (e = r->tile_offset.ensure(Pz + 1)) ||
        (e = r->col_offset.ensure(Pz + 1)) || (e = r->scenes_dev.ensure(scene_count)) ||
        (e = r->pack_info.ensure(1)) || (e = r->scene_ranges.ensure(2 * (size_t)scene_count)))
        return cuda_status(e);

    // ---- the caller's records through the pinned staging ----------------------
    const size_t stage_bytes = HostStage::room(4 * (size_t)nb) + HostStage::room(sizeof(PFCUDAPath) * Pz) +
                               HostStage::room(sizeof(ScenePackDev) * scene_count) +
                               HostStage::room(sizeof(OverlayDev) * overlays.size()) +
                               HostStage::room(4 * texels.size()) + HostStage::room(overlay_opaque.size()) +
                               HostStage::room(sizeof(PackInfo)) + HostStage::room(8 * (size_t)scene_count);
    if ((e = r->stage.begin(stage_bytes))) return cuda_status(e);
    HostStage& hs = r->stage;
    uint32_t* raw = hs.take<uint32_t>(nb);
    PFCUDAPath* paths = hs.take<PFCUDAPath>(Pz);
    for (uint32_t k = 0; k < scene_count; k++) {
        const PFCUDASceneDesc& sc = scenes[k];
        const ScenePackDev& pk = packs[k];
        // contour c of the scene is global contour contour_base + c; its end is
        // the next boundary, so the scene's boundaries (count + 1) are copied whole
        if (sc.contour_count == 0) raw[pk.contour_base] = 0;
        else if (sc.memory == PF_MEMORY_HOST)
            std::memcpy(raw + pk.contour_base, sc.contour_starts, sizeof(uint32_t) * ((size_t)sc.contour_count + 1));
        if (sc.clip_path_count)
            std::memcpy(paths + pk.first_path, sc.clip_paths, sizeof(PFCUDAPath) * sc.clip_path_count);
        if (sc.draw_path_count)
            std::memcpy(paths + pk.first_path + sc.clip_path_count, sc.draw_paths,
                        sizeof(PFCUDAPath) * sc.draw_path_count);
    }
    auto h2d = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
        return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s) : cudaSuccess;
    };
    if ((e = h2d(r->starts_raw.p, raw, 4 * (size_t)nb)) || (e = h2d(r->path_in.p, paths, sizeof(PFCUDAPath) * Pz)) ||
        (e = h2d(r->scene_pack.p, hs.put(packs), sizeof(ScenePackDev) * scene_count)) ||
        (e = h2d(r->overlays.p, hs.put(overlays), sizeof(OverlayDev) * overlays.size())) ||
        (e = h2d(r->texels.p, hs.put(texels), 4 * texels.size())) ||
        (e = h2d(r->overlay_opaque.p, hs.put(overlay_opaque), overlay_opaque.size())))
        return cuda_status(e);
    // The points queue behind the small copies above (copies in one direction
    // share an engine in issue order), so the packing below starts at once.
    for (uint32_t k = 0; k < scene_count; k++) {
        const PFCUDASceneDesc& sc = scenes[k];
        const cudaMemcpyKind kind = sc.memory == PF_MEMORY_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
        if (sc.point_count)
            PF_TRY(cudaMemcpyAsync(r->pts.p + packs[k].point_base, sc.points, sizeof(float2) * sc.point_count, kind,
                                   r->copy_stream));
    }
    PF_TRY(cudaEventRecord(r->points_done, r->copy_stream));
    for (uint32_t k = 0; k < scene_count; k++) {  // boundaries already in device memory
        const PFCUDASceneDesc& sc = scenes[k];
        if (sc.contour_count && sc.memory == PF_MEMORY_DEVICE)
            PF_TRY(cudaMemcpyAsync(r->starts_raw.p + packs[k].contour_base, sc.contour_starts,
                                   sizeof(uint32_t) * ((size_t)sc.contour_count + 1), cudaMemcpyDeviceToDevice, s));
    }
    PackInfo* hinfo = hs.take<PackInfo>(1);
    uint32_t* hranges = hs.take<uint32_t>(2 * (size_t)scene_count);

    // ---- packing on the device -------------------------------------------------
    PackInfo* info = r->pack_info.p;
    ScanTemp tmp{r->scan_partials.p, (uint32_t)r->scan_partials.cap};
    PF_TRY(cudaMemsetAsync(info, 0, sizeof(PackInfo), s));
    launch_pack_starts(r->starts_raw.p, r->starts.p, r->scene_pack.p, scene_count, nb, (uint32_t)np_total, info, s);
    const PathTablesDev t{r->path_ncont.p, r->paint.p,      r->local_index.p,   r->scene_of.p,
                          r->clip_gpath.p, r->rule.p,       r->is_clip.p,       r->draw_index.p,
                          r->alpha_default.p, r->blend.p,   r->overlay.p,       r->occludes.p};
    launch_pack_paths(r->path_in.p, (uint32_t)P, r->scene_pack.p, scene_count, r->overlay_opaque.p, t, info, s);
    launch_scan(r->path_ncont.p, r->first_ord.p, nullptr, (uint32_t)P, (uint32_t)P, 0, &info->nord, tmp, s);
    launch_pack_chains(r->clip_gpath.p, r->is_clip.p, r->scene_of.p, r->scene_pack.p, (uint32_t)P, info, s);
    // Segments per contour reference (SegmentsD3D11::add_path): count, scan,
    // and the scene ranges, then one read-back.
    auto pack_segments = [&]() -> cudaError_t {
        tmp = ScanTemp{r->scan_partials.p, (uint32_t)r->scan_partials.cap};
        launch_pack_order(r->path_in.p, (uint32_t)P, r->scene_pack.p, r->scene_of.p, r->path_ncont.p, r->first_ord.p,
                          cap, r->ord_contour.p, r->ord_path.p, s);
        launch_contour_segcount(r->ord_contour.p, &info->nord, cap, r->starts.p, nb, r->flags.p, r->contour_segs.p,
                                &info->status, s);
        launch_scan(r->contour_segs.p, r->contour_seg_base.p, &info->nord, 0, cap, 0, &info->segs, tmp, s);
        launch_pack_ranges(r->scene_pack.p, scene_count, r->first_ord.p, r->contour_seg_base.p, &info->nord, cap,
                           r->scene_ranges.p, s);
        cudaError_t x;
        if ((x = cudaGetLastError()) ||
            (x = cudaMemcpyAsync(hinfo, info, sizeof(PackInfo), cudaMemcpyDeviceToHost, s)) ||
            (scene_count && (x = cudaMemcpyAsync(hranges, r->scene_ranges.p, 8 * (size_t)scene_count,
                                                 cudaMemcpyDeviceToHost, s))) ||
            (x = hs.mark(s)))
            return x;
        return cudaStreamSynchronize(s);
    };
    if ((e = pack_segments())) return cuda_status(e);
    if ((hinfo->status & kStatusMalformed) || hinfo->refs >= 0x7fffffffull) return PF_CUDA_ERR_INVALID;
    if (hinfo->nord > cap) {  // paths share contours: grow and pack the order again
        cap = (uint32_t)hinfo->nord;
        if ((e = ensure_order(cap)) || (e = pack_segments())) return cuda_status(e);
        if (hinfo->status & kStatusMalformed) return PF_CUDA_ERR_INVALID;
    }
    const uint32_t nord = (uint32_t)hinfo->nord;
    if (hinfo->segs >= 0x7fffffffull) return PF_CUDA_ERR_INVALID;
    const uint32_t S = (uint32_t)hinfo->segs;
    if ((e = r->segs.ensure((size_t)S + 1)) || (e = r->seg_line_count.ensure((size_t)S + 1)) ||
        (e = r->seg_line_base.ensure((size_t)S + 1)) || (e = r->seg_leaves.ensure((size_t)S + 1)) ||
        (e = r->seg_warp.ensure(2 * (((size_t)S + 31) / 32 + 2))))
        return cuda_status(e);
    launch_contour_segemit(r->ord_contour.p, r->ord_path.p, &info->nord, cap, r->starts.p, nb, r->flags.p,
                           r->contour_seg_base.p, r->segs.p, s);
    PF_TRY(cudaGetLastError());
    for (uint32_t k = 0; k < scene_count; k++) {
        r->scenes[k].seg_begin = hranges[2 * k];
        r->scenes[k].seg_end = hranges[2 * k + 1];
    }
    PF_TRY(upload_scene_records(r));

    r->clip_chain_max = hinfo->chain_max;
    r->nested_clips = (hinfo->flags & kPackNestedClips) != 0;
    r->paint_effects = !overlays.empty() || (hinfo->flags & kPackBlendModes) != 0;
    r->P = (uint32_t)P;
    r->ND = draw_base;
    r->diff_valid = false;
    r->NP = (uint32_t)np_total;
    r->NC = (uint32_t)nc_total;
    r->nord = nord;
    r->S = S;
    r->screen_total = screen_total;
    // first-frame capacity guesses; grown on overflow and kept across frames
    r->tile_cap = std::max<uint32_t>(r->tile_cap, std::max<uint32_t>(1u << 16, 4 * screen_total));
    r->col_cap = std::max<uint32_t>(r->col_cap, std::max<uint32_t>(1u << 16, 16 * r->P));
    r->fill_cap = std::max<uint32_t>(r->fill_cap, std::max<uint32_t>(1u << 18, 4 * S));
    r->line_cap = std::max<uint32_t>(r->line_cap, std::max<uint32_t>(1u << 16, 2 * S));
    r->vis_cap = std::max<uint32_t>(r->vis_cap, r->tile_cap);
    r->has_scene = true;  // the segment records complete in stream order before any frame
    return PF_CUDA_OK;
}

int32_t PFCUDASceneUploadBatch(PFCUDARendererRef r, const PFCUDASceneDesc* scenes, const PFCUDASceneTarget* targets,
                               uint32_t scene_count) {
    if (!r || !scenes || scene_count == 0) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    cudaStream_t s = r->stream;
    release_graph(r);
    r->has_scene = false;

    uint64_t np_total = 0, nc_total = 0, P = 0;
    for (uint32_t k = 0; k < scene_count; k++) {
        const PFCUDASceneDesc& sc = scenes[k];
        if (sc.memory != PF_MEMORY_HOST && sc.memory != PF_MEMORY_DEVICE) return PF_CUDA_ERR_INVALID;
        if ((sc.clip_path_count && !sc.clip_paths) || (sc.draw_path_count && !sc.draw_paths)) return PF_CUDA_ERR_INVALID;
        if (sc.contour_count && !sc.contour_starts) return PF_CUDA_ERR_INVALID;
        if (sc.point_count && (!sc.points || !sc.point_flags)) return PF_CUDA_ERR_INVALID;
        np_total += sc.point_count;
        nc_total += (uint64_t)sc.contour_count + 1;  // each scene keeps its own end boundary
        P += (uint64_t)sc.clip_path_count + sc.draw_path_count;
    }
    if (np_total >= 0x7fffffffull || nc_total >= 0x7fffffffull || P >= 0x7fffffffull) return PF_CUDA_ERR_INVALID;

    // The point arrays are the bulk of an upload: their copies go first, so
    // that from pinned memory they run while the tables are built. The flags
    // go on the frame stream (segment packing reads them); the points, eight
    // times larger, on the copy stream, after every earlier frame on the frame
    // stream (which may still read the old points).
    cudaError_t e;
    if ((e = r->pts.ensure(np_total)) || (e = r->flags.ensure(np_total))) return cuda_status(e);
    PF_TRY(cudaEventRecord(r->prior_done, s));
    PF_TRY(cudaStreamWaitEvent(r->copy_stream, r->prior_done, 0));
    uint64_t point_base = 0;
    for (uint32_t k = 0; k < scene_count; k++) {
        const PFCUDASceneDesc& sc = scenes[k];
        const cudaMemcpyKind kind = sc.memory == PF_MEMORY_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
        if (sc.point_count)
            PF_TRY(cudaMemcpyAsync(r->flags.p + point_base, sc.point_flags, sc.point_count, kind, s));
        point_base += sc.point_count;
    }
    const int32_t rc = upload_tables(r, scenes, targets, scene_count, np_total, nc_total, P);
    // Later work on the frame stream sees the points, and no copy that reads
    // the caller's arrays outlives the call.
    const cudaError_t e1 = cudaStreamWaitEvent(s, r->points_done, 0);
    const cudaError_t e2 = cudaEventSynchronize(r->points_done);
    if (rc != PF_CUDA_OK) {
        cudaStreamSynchronize(s);
        return rc;
    }
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
        r->has_scene = false;
        return cuda_status(e1 != cudaSuccess ? e1 : e2);
    }
    return PF_CUDA_OK;
}

int32_t PFCUDASceneUpload(PFCUDARendererRef r, const PFCUDASceneDesc* sc) {
    if (!r || !sc) return PF_CUDA_ERR_INVALID;
    return PFCUDASceneUploadBatch(r, sc, nullptr, 1);
}

// Whether [p, p + bytes) lies inside one page-locked host allocation, asked
// of the driver (cuPointerGetAttribute's range attributes, looked up through
// the runtime so that nothing links the driver library). Any failure is a no.
static bool inside_host_allocation(const void* p, size_t bytes) {
    using GetAttr = CUresult (*)(void*, CUpointer_attribute, CUdeviceptr);
    static GetAttr get = [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            fn = nullptr;
        return (GetAttr)fn;
    }();
    if (!get) return false;
    CUdeviceptr start = 0;
    size_t size = 0;
    const CUdeviceptr a = (CUdeviceptr)(uintptr_t)p;
    if (get(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, a) != CUDA_SUCCESS ||
        get(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, a) != CUDA_SUCCESS)
        return false;
    return start <= a && bytes <= size && a - start <= size - bytes;
}

static int32_t render_plain(PFCUDARendererRef r, const PFCUDABuildOptions* options, int32_t width, int32_t height,
                            void* out, int32_t out_memory, int32_t format) {
    if (!r || !out) return PF_CUDA_ERR_INVALID;
    if (!r->has_scene) return PF_CUDA_ERR_NO_SCENE;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    bool changed = false;
    int32_t rc = prepare_plain_targets(r, width, height, &changed);
    if (rc) return rc;
    if (changed) PF_TRY(upload_scene_records(r));
    const size_t elem = format == PF_CUDA_FORMAT_RGBA8 ? 4 : (format == PF_CUDA_FORMAT_R8 ? 1 : 4);
    const size_t bytes = (size_t)width * (size_t)height * elem;
    void* dst = out;
    bool staged = out_memory == PF_MEMORY_HOST_COPY;
    if (out_memory == PF_MEMORY_HOST) {
        // Page-locked host memory is mapped into the device's address space:
        // the composite writes the frame there itself (no device copy and no
        // separate device-to-host pass), and pixels outside the screen tiles
        // keep the caller's values. Pageable memory goes through a device copy.
        // The whole image must lie in the one allocation: the GPU writes it.
        cudaPointerAttributes pa{};
        if (cudaPointerGetAttributes(&pa, out) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer &&
            inside_host_allocation(out, bytes))
            dst = pa.devicePointer;
        else
            staged = true;
        (void)cudaGetLastError();
    } else if (out_memory != PF_MEMORY_DEVICE && out_memory != PF_MEMORY_HOST_COPY) {
        return PF_CUDA_ERR_INVALID;
    }
    if (staged) {
        PF_TRY(r->out_tmp.ensure(bytes));
        dst = r->out_tmp.p;
        // Pixels outside every scene's screen tiles are not written: they keep
        // the caller's values, as they do in a device buffer.
        bool covered = false;
        for (const SceneInfo& si : r->scenes)
            covered = covered || (!si.explicit_target && si.screen.x <= 0 && si.screen.y <= 0 &&
                                  (int64_t)si.screen.z * 16 >= width && (int64_t)si.screen.w * 16 >= height);
        if (!covered) PF_TRY(cudaMemcpyAsync(dst, out, bytes, cudaMemcpyHostToDevice, r->stream));
    }
    const ImageCopy copy{out, dst, bytes};
    return run_frame(r, options, format, dst, make_range(r, 0, (uint32_t)r->scenes.size()), false,
                     staged ? &copy : nullptr);
}

int32_t PFCUDARenderScene(PFCUDARendererRef r, const PFCUDABuildOptions* options, int32_t width, int32_t height,
                          uint8_t* out, int32_t out_memory) {
    return render_plain(r, options, width, height, out, out_memory, PF_CUDA_FORMAT_RGBA8);
}

int32_t PFCUDARenderCoverage(PFCUDARendererRef r, const PFCUDABuildOptions* options, int32_t width, int32_t height,
                             float* out, int32_t out_memory) {
    return render_plain(r, options, width, height, out, out_memory, PF_CUDA_FORMAT_F32);
}

int32_t PFCUDARenderSceneAsync(PFCUDARendererRef r, const PFCUDABuildOptions* options, int32_t width,
                               int32_t height, uint8_t* out_rgba8_device) {
    if (!r || !out_rgba8_device) return PF_CUDA_ERR_INVALID;
    if (!r->has_scene) return PF_CUDA_ERR_NO_SCENE;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    bool changed = false;
    int32_t rc = prepare_plain_targets(r, width, height, &changed);
    if (rc) return rc;
    if (changed) PF_TRY(upload_scene_records(r));
    r->last = make_range(r, 0, (uint32_t)r->scenes.size());
    PF_TRY(ensure_frame_buffers(r));
    PF_TRY(enqueue_frame(r, options, PF_CUDA_FORMAT_RGBA8, out_rgba8_device, r->last));
    return PF_CUDA_OK;
}

int32_t PFCUDARenderBatch(PFCUDARendererRef r, const PFCUDABuildOptions* options, uint32_t first, uint32_t count,
                          int32_t format, void* out_device) {
    if (!r || !out_device || format < 0 || format > 2) return PF_CUDA_ERR_INVALID;
    if (!valid_range(r, first, count)) return r->has_scene ? PF_CUDA_ERR_INVALID : PF_CUDA_ERR_NO_SCENE;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    return run_frame(r, options, format, out_device, make_range(r, first, count));
}

int32_t PFCUDARenderBatchAsync(PFCUDARendererRef r, const PFCUDABuildOptions* options, uint32_t first,
                               uint32_t count, int32_t format, void* out_device) {
    if (!r || !out_device || format < 0 || format > 2) return PF_CUDA_ERR_INVALID;
    if (!valid_range(r, first, count)) return r->has_scene ? PF_CUDA_ERR_INVALID : PF_CUDA_ERR_NO_SCENE;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    r->last = make_range(r, first, count);
    PF_TRY(ensure_frame_buffers(r));
    PF_TRY(enqueue_frame(r, options, format, out_device, r->last));
    return PF_CUDA_OK;
}

int32_t PFCUDARenderStatus(PFCUDARendererRef r, uint64_t* out_needed) {
    if (!r) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    PF_TRY(cudaMemcpyAsync(r->h_counters, r->counters.p, sizeof(Counters), cudaMemcpyDeviceToHost, r->stream));
    PF_TRY(cudaStreamSynchronize(r->stream));
    Counters h = *r->h_counters;
    record_stats(r, h, 0.0f);
    if (out_needed) *out_needed = std::max({h.needed_fills, h.needed_tiles, h.needed_visible, h.needed_lines});
    if (h.status & kCapacityBits) grow(r, h);
    return status_to_code(h.status);
}

int32_t PFCUDAGraphCapture(PFCUDARendererRef r, const PFCUDABuildOptions* options, uint32_t first, uint32_t count,
                           int32_t format, void* out_device) {
    if (!r) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    int32_t rc = PFCUDARenderBatch(r, options, first, count, format, out_device);
    if (rc != PF_CUDA_OK) return rc;
    release_graph(r);
    const bool prof = r->profiling;
    r->profiling = false;
    PF_TRY(cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue_frame(r, options, format, out_device, r->last);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(r->stream, &g);
    r->profiling = prof;
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return PF_CUDA_ERR_LAUNCH;
    }
    r->graph = g;
    PF_TRY(cudaGraphInstantiate(&r->graph_exec, g, 0));
    r->graph_has_opts = options != nullptr;
    r->graph_opts = options ? *options : PFCUDABuildOptions{};
    r->graph_format = format;
    r->graph_out = out_device;
    r->graph_range = r->last;
    r->graph_key = frame_key(r, options, format, out_device, r->last);
    return PF_CUDA_OK;
}

int32_t PFCUDAGraphLaunch(PFCUDARendererRef r) {
    if (!r || !r->graph_exec) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    // The graph holds the buffer pointers and sizes of its capture; a frame
    // or upload since then that regrew a buffer or changed a size would make
    // it launch on freed memory, so it is refused (capture it again).
    if (frame_key(r, r->graph_has_opts ? &r->graph_opts : nullptr, r->graph_format, r->graph_out, r->graph_range) !=
        r->graph_key)
        return PF_CUDA_ERR_INVALID;
    PF_TRY(cudaGraphLaunch(r->graph_exec, r->stream));
    return PF_CUDA_OK;
}

int32_t PFCUDAGraphRelease(PFCUDARendererRef r) {
    if (!r) return PF_CUDA_ERR_INVALID;
    release_graph(r);
    return PF_CUDA_OK;
}

int32_t PFCUDASetTuning(PFCUDARendererRef r, const PFCUDATuning* t) {
    if (!r || !t) return PF_CUDA_ERR_INVALID;
    auto in = [](int v, std::initializer_list<int> ok) { return std::find(ok.begin(), ok.end(), v) != ok.end(); };
    if (!in(t->flatten_threads, {64, 128, 256}) || !in(t->bin_threads, {128, 256, 512}) ||
        t->bin_blocks_per_sm < 4 || t->bin_blocks_per_sm > 64 || !in(t->composite_warps, {2, 4, 8}) ||
        !in(t->composite_batch, {1, 2, 4, 8}) || t->mask_stage_fills < 0 || t->mask_stage_fills > 128)
        return PF_CUDA_ERR_INVALID;
    r->tune = TuneParams{t->flatten_threads, t->bin_threads, t->bin_blocks_per_sm, t->composite_warps,
                         t->composite_batch, t->mask_stage_fills};
    release_graph(r);
    return PF_CUDA_OK;
}

int32_t PFCUDAGetTuning(PFCUDARendererRef r, PFCUDATuning* t) {
    if (!r || !t) return PF_CUDA_ERR_INVALID;
    *t = PFCUDATuning{r->tune.flatten_threads, r->tune.bin_threads, r->tune.bin_blocks_per_sm, r->tune.comp_warps,
                      r->tune.comp_batch, r->tune.mask_stage};
    return PF_CUDA_OK;
}

int32_t PFCUDAAutotune(PFCUDARendererRef r, const PFCUDABuildOptions* options, uint32_t first, uint32_t count,
                       int32_t format, void* out_device, int32_t repeats, PFCUDATuning* out_best) {
    if (!r || repeats <= 0) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    int32_t rc = PFCUDARenderBatch(r, options, first, count, format, out_device);  // sizes the buffers
    if (rc != PF_CUDA_OK) return rc;
    const Range g = r->last;
    auto time_it = [&](const TuneParams& tp, float* ms_out) -> int32_t {
        r->tune = tp;
        std::vector<float> v;
        for (int i = 0; i < repeats + 1; i++) {
            PF_TRY(cudaEventRecord(r->ev0, r->stream));
            PF_TRY(enqueue_frame(r, options, format, out_device, g));
            PF_TRY(cudaEventRecord(r->ev1, r->stream));
            PF_TRY(cudaEventSynchronize(r->ev1));
            float ms = 0;
            PF_TRY(cudaEventElapsedTime(&ms, r->ev0, r->ev1));
            if (i > 0) v.push_back(ms);  // the first run warms the shape
        }
        std::sort(v.begin(), v.end());
        *ms_out = v[v.size() / 2];
        return PF_CUDA_OK;
    };
    TuneParams best = r->tune;
    float best_ms = 0;
    if ((rc = time_it(best, &best_ms))) return rc;
    const int flat[] = {64, 128, 256}, bin[] = {128, 256, 512}, bps[] = {4, 8, 16, 32}, cw[] = {2, 4, 8},
              cb[] = {1, 2, 4, 8}, ms[] = {0, 8, 32};
    for (int dim = 0; dim < 6; dim++) {
        const int* cand = dim == 0 ? flat : dim == 1 ? bin : dim == 2 ? bps : dim == 3 ? cw : dim == 4 ? cb : ms;
        const int nc = (dim == 2 || dim == 4) ? 4 : 3;
        for (int i = 0; i < nc; i++) {
            TuneParams tp = best;
            if (dim == 0) tp.flatten_threads = cand[i];
            if (dim == 1) tp.bin_threads = cand[i];
            if (dim == 2) tp.bin_blocks_per_sm = cand[i];
            if (dim == 3) tp.comp_warps = cand[i];
            if (dim == 4) tp.comp_batch = cand[i];
            if (dim == 5) tp.mask_stage = cand[i];
            float ms = 0;
            if ((rc = time_it(tp, &ms))) return rc;
            if (ms < best_ms) { best_ms = ms; best = tp; }
        }
    }
    r->tune = best;
    release_graph(r);
    // the final frame with the chosen shape leaves valid counters behind
    if ((rc = PFCUDARenderBatch(r, options, first, count, format, out_device))) return rc;
    if (out_best) PFCUDAGetTuning(r, out_best);
    return PF_CUDA_OK;
}

int32_t PFCUDAReadMasks(PFCUDARendererRef r, float* out_alpha, uint64_t alpha_cap, float* out_tile,
                        uint64_t tile_cap) {
    if (!r || !r->has_scene) return PF_CUDA_ERR_NO_SCENE;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    uint64_t A = r->stats.alpha_tile_count, T = r->stats.tile_count;
    if ((out_alpha && alpha_cap < A) || (out_tile && tile_cap < T)) return PF_CUDA_ERR_CAPACITY;
    FrameDev f = frame_dev(r, false, r->last, r->last_diff);
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
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    cudaStream_t s = r->stream;
    const Range& g = r->last;
    const uint64_t F = r->stats.fill_count, T = r->stats.tile_count, NPth = g.p1 - g.p0, NST = g.st1 - g.st0;
    if (fills && r->last_diff) return PF_CUDA_ERR_INVALID;  // differentiable frames keep FP32 fills only
    if (fills && F && !r->last_fill_order) {
        // the frame again, without composite, with each fill's emission index
        r->fill_order = true;
        const int32_t rc = run_frame(r, &r->last_opts, -1, nullptr, g);
        r->fill_order = false;
        // malformed input or a limit reached ends the frame as before; its
        // records are still read
        if (rc != PF_CUDA_OK && rc != PF_CUDA_ERR_INVALID && rc != PF_CUDA_ERR_LIMIT) return rc;
        if (r->stats.fill_count != F) return PF_CUDA_ERR_LAUNCH;
    }
    if ((fills || fill_tile) && fill_capacity < F) return PF_CUDA_ERR_CAPACITY;
    if ((tiles || clips) && tile_capacity < T) return PF_CUDA_ERR_CAPACITY;
    if ((path_tile_offsets || path_tile_rects) && path_capacity < NPth + 1) return PF_CUDA_ERR_CAPACITY;
    if (z_buffer && z_capacity < NST) return PF_CUDA_ERR_CAPACITY;
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
        uint64_t t = 0;
        for (uint64_t i = 0; i < F; i++) {
            while (t + 1 <= T && base[t + 1] <= i) t++;
            fill_tile[i] = (uint32_t)t;
        }
    }
    std::vector<uint32_t> off(NPth + 1);
    PF_TRY(cudaMemcpyAsync(off.data(), r->tile_offset.p + g.p0, (NPth + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    PF_TRY(cudaStreamSynchronize(s));
    if (tiles && T) {
        PF_TRY(cudaMemcpyAsync(tiles, r->tiles.p, T * sizeof(PFCUDATile), cudaMemcpyDeviceToHost, s));
        PF_TRY(cudaStreamSynchronize(s));
        // device records carry the global path index; report the index within
        // the clip paths or the draw paths, as TileObjectPrimitive::path_id
        for (uint64_t i = 0; i < T; i++) tiles[i].path_id = path_local_of(r, tiles[i].path_id, nullptr);
    }
    if (clips && T) {
        std::vector<int32_t> clip_of(NPth + 1);
        PF_TRY(cudaMemcpyAsync(clips, r->clips.p, T * sizeof(PFCUDAClip), cudaMemcpyDeviceToHost, s));
        PF_TRY(cudaMemcpyAsync(clip_of.data(), r->clip_gpath.p + g.p0, NPth * sizeof(int32_t), cudaMemcpyDeviceToHost,
                               s));
        PF_TRY(cudaStreamSynchronize(s));
        // tiles of clip paths and of unclipped draw paths carry no clip record
        // (the frame writes records only for clipped draw paths)
        for (uint64_t q = 0; q < NPth; q++)
            if (path_is_clip_of(r, g.p0 + q) || clip_of[q] < 0)
                for (uint32_t t = off[q]; t < off[q + 1]; t++) clips[t] = PFCUDAClip{0xffffffffu, 0, 0xffffffffu, 0};
    }
    if (path_tile_offsets) std::memcpy(path_tile_offsets, off.data(), (NPth + 1) * sizeof(uint32_t));
    if (path_tile_rects && NPth)
        PF_TRY(cudaMemcpyAsync(path_tile_rects, r->tile_rect.p + g.p0, NPth * sizeof(PFRectI), cudaMemcpyDeviceToHost, s));
    if (z_buffer && NST)
        PF_TRY(cudaMemcpyAsync(z_buffer, r->zbuf.p, NST * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    PF_TRY(cudaStreamSynchronize(s));
    return PF_CUDA_OK;
}

int32_t PFCUDASetProfiling(PFCUDARendererRef r, int32_t enable) {
    if (!r) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    if (enable && !r->stage_ev[0])
        for (int i = 0; i <= PF_CUDA_STAGE_COUNT; i++) PF_TRY(cudaEventCreate(&r->stage_ev[i]));
    r->profiling = enable != 0;
    return PF_CUDA_OK;
}

int32_t PFCUDAGetStageTimes(PFCUDARendererRef r, float* out_ms, int32_t capacity) {
    if (!r || !out_ms || capacity < PF_CUDA_STAGE_COUNT) return PF_CUDA_ERR_INVALID;
    if (!r->profiling) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    PF_TRY(cudaEventSynchronize(r->stage_ev[PF_CUDA_STAGE_COUNT]));
    for (int i = 0; i < PF_CUDA_STAGE_COUNT; i++) {
        float ms = 0;
        PF_TRY(cudaEventElapsedTime(&ms, r->stage_ev[i], r->stage_ev[i + 1]));
        out_ms[i] = ms;
    }
    return PF_CUDA_OK;
}

int32_t PFCUDAStrokeToFill(PFCUDARendererRef r, const PFCUDAStrokeInput* input, PFCUDAStrokeOutput* output) {
    if (!r || !input || !output) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    if (!r->stroke) r->stroke = stroke_work_create();
    return stroke_run(r->stroke, r->stream, input, output);
}

int32_t PFCUDADashOutlines(PFCUDARendererRef r, const PFCUDAStrokeInput* input, const PFCUDADashInput* dash,
                           PFCUDAOutlineOutput* output) {
    if (!r || !input || !dash || !output) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    if (!r->stroke) r->stroke = stroke_work_create();
    return dash_outlines(r->stroke, r->stream, input, dash, output);
}

int32_t PFCUDAStrokeToFillDashed(PFCUDARendererRef r, const PFCUDAStrokeInput* input, const PFCUDADashInput* dash,
                                 PFCUDAStrokeOutput* output) {
    if (!r || !input || !dash || !output) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    if (!r->stroke) r->stroke = stroke_work_create();
    return stroke_dashed(r->stroke, r->stream, input, dash, output);
}

int32_t PFCUDAExclusiveScan(PFCUDARendererRef r, const uint32_t* in, uint32_t* out, uint32_t n) {
    if (!r || !out || (!in && n) || n >= 0x80000000u) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    PF_TRY(r->scan_partials.ensure((size_t)n / 2048 + 2));
    ScanTemp tmp{r->scan_partials.p, (uint32_t)r->scan_partials.cap};
    launch_scan(in, out, nullptr, n, n, 0, nullptr, tmp, r->stream);
    PF_TRY(cudaGetLastError());
    PF_TRY(cudaStreamSynchronize(r->stream));
    return PF_CUDA_OK;
}

int32_t PFCUDASetPoints(PFCUDARendererRef r, const PFVector2F* points, uint64_t count, int32_t memory) {
    if (!r) return PF_CUDA_ERR_INVALID;
    if (!r->has_scene) return PF_CUDA_ERR_NO_SCENE;
    if (count != r->NP || (count && !points)) return PF_CUDA_ERR_INVALID;
    if (memory != PF_MEMORY_HOST && memory != PF_MEMORY_DEVICE) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    r->diff_valid = false;
    if (count)
        PF_TRY(cudaMemcpyAsync(r->pts.p, points, sizeof(float2) * count,
                               memory == PF_MEMORY_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                               r->stream));
    if (memory == PF_MEMORY_HOST) PF_TRY(cudaStreamSynchronize(r->stream));  // the caller may reuse its buffer
    return PF_CUDA_OK;
}

static int32_t diff_prologue(PFCUDARendererRef r, uint32_t first, uint32_t count, int32_t width, int32_t height,
                             const float* draw_alpha, float* out_device) {
    if (!r || !out_device) return PF_CUDA_ERR_INVALID;
    if (!valid_range(r, first, count)) return r->has_scene ? PF_CUDA_ERR_INVALID : PF_CUDA_ERR_NO_SCENE;
    if (r->nested_clips) return PF_CUDA_ERR_INVALID;  // the adjoint covers single-level clips
    if (r->paint_effects) return PF_CUDA_ERR_INVALID;  // and solid paint with SrcOver
    if (r->options.flags & PF_CUDA_RENDERER_D3D11_SEMANTICS) return PF_CUDA_ERR_INVALID;  // pieces rounded to 1/256 px
    if (width > 0 || height > 0) {
        bool changed = false;
        int32_t rc = prepare_plain_targets(r, width, height, &changed);
        if (rc) return rc;
        if (changed) PF_TRY(upload_scene_records(r));
    }
    PF_TRY(r->alpha_in.ensure((size_t)r->ND + 1));
    if (r->ND) {
        if (draw_alpha)
            PF_TRY(cudaMemcpyAsync(r->alpha_in.p, draw_alpha, sizeof(float) * r->ND, cudaMemcpyDeviceToDevice, r->stream));
        else
            PF_TRY(cudaMemcpyAsync(r->alpha_in.p, r->alpha_default.p, sizeof(float) * r->ND, cudaMemcpyDeviceToDevice,
                                   r->stream));
    }
    r->diff_buffers = true;
    r->diff_valid = false;
    return PF_CUDA_OK;
}

static void diff_epilogue(PFCUDARendererRef r, const PFCUDABuildOptions* options, const Range& g) {
    r->diff_valid = true;
    r->diff_range = g;
    r->diff_transformed = !is_identity(options);
    if (r->diff_transformed) {
        r->diff_m4[0] = options->transform.m00; r->diff_m4[1] = options->transform.m01;
        r->diff_m4[2] = options->transform.m10; r->diff_m4[3] = options->transform.m11;
    }
}

int32_t PFCUDARenderDiff(PFCUDARendererRef r, const PFCUDABuildOptions* options, uint32_t first, uint32_t count,
                         int32_t width, int32_t height, const float* draw_alpha, float* out_device) {
    if (!r) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    int32_t rc = diff_prologue(r, first, count, width, height, draw_alpha, out_device);
    if (rc != PF_CUDA_OK) return rc;
    const Range g = make_range(r, first, count);
    rc = run_frame(r, options, PF_CUDA_FORMAT_F32, out_device, g, true);
    if (rc != PF_CUDA_OK) return rc;
    diff_epilogue(r, options, g);
    return PF_CUDA_OK;
}

int32_t PFCUDARenderDiffAsync(PFCUDARendererRef r, const PFCUDABuildOptions* options, uint32_t first,
                              uint32_t count, int32_t width, int32_t height, const float* draw_alpha,
                              float* out_device) {
    if (!r) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    int32_t rc = diff_prologue(r, first, count, width, height, draw_alpha, out_device);
    if (rc != PF_CUDA_OK) return rc;
    const Range g = make_range(r, first, count);
    r->last = g;
    PF_TRY(ensure_frame_buffers(r));
    PF_TRY(enqueue_frame(r, options, PF_CUDA_FORMAT_F32, out_device, g, true));
    diff_epilogue(r, options, g);
    return PF_CUDA_OK;
}

int32_t PFCUDABackward(PFCUDARendererRef r, const float* d_image, PFVector2F* d_points, float* d_alpha) {
    if (!r || !d_image || !d_points) return PF_CUDA_ERR_INVALID;
    if (!r->diff_valid) return PF_CUDA_ERR_INVALID;
    DeviceGuard dg(r->device);
    PF_TRY(dg.status);
    cudaStream_t s = r->stream;
    const uint64_t before = launch_counter();
    PF_TRY(r->grad_mask.ensure(((size_t)r->tile_cap + 1) * 256));  // alpha ids < tiles <= tile_cap
    if (r->NP) PF_TRY(cudaMemsetAsync(d_points, 0, sizeof(float2) * r->NP, s));
    float* ga = d_alpha;
    if (!ga) {
        PF_TRY(r->grad_alpha_tmp.ensure((size_t)r->ND + 1));
        ga = r->grad_alpha_tmp.p;
    }
    if (r->ND) PF_TRY(cudaMemsetAsync(ga, 0, sizeof(float) * r->ND, s));
    FrameDev f = frame_dev(r, r->diff_transformed, r->diff_range, true);
    launch_composite_bwd(f, d_image, r->grad_mask.p, ga, s);
    launch_line_grad(f, r->grad_mask.p, (float2*)d_points, s);
    if (r->diff_transformed) launch_points_grad_transform((float2*)d_points, r->NP, r->diff_m4, s);
    PF_TRY(cudaGetLastError());
    r->stats.kernel_launches = launch_counter() - before;
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

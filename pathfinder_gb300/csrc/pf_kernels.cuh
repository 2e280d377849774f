// pf_kernels.cuh — launch wrappers of the CUDA level's kernels (host side).
#pragma once

#include "pf_device.cuh"

#include <utility>
#include <vector>

struct PFCUDAPath;

namespace pf {

// Launch shapes chosen by the autotuner (outputs do not depend on them).
struct TuneParams {
    int flatten_threads;   // threads per block of the flattening passes
    int bin_threads;       // threads per block of the binning passes
    int bin_blocks_per_sm; // grid of the binning passes = SMs x this
    int comp_warps;        // warps per block of the composite (2, 4 or 8)
    int comp_batch;        // screen tiles per work item of the persistent composite (1, 2, 4 or 8)
    int mask_stage;        // fill ranges of at least this many fills staged by bulk copy (0: none)
};

// One frame covers a contiguous range of the uploaded scenes; paths,
// segments and screen tiles of that range are contiguous too.  Path and
// segment arrays are indexed globally; per-frame arrays (tiles, lines, fills,
// screen tiles) are indexed from the start of the range.
struct FrameDev {
    // scene
    const float2* pts;           // points used by the tiler (transformed copy when needed)
    const SegRec* segs;
    uint32_t seg_begin, seg_count;
    PathDev path;
    const SceneDev* scenes;
    const uint32_t* scene_st;    // [scenes] each scene's first global screen tile
    uint32_t path_begin, path_count;
    uint32_t scene_begin, scene_count;
    uint32_t screen_begin;       // global index of the range's first screen tile
    TuneParams tune;
    uint32_t sms;                // multiprocessors of the renderer's device (grid sizes)
    // tile arrays (capacity tile_cap; +1 for scan totals)
    uint32_t tile_cap, col_cap, fill_cap, vis_cap, screen_count;
    uint32_t* tile_fill_count;   // [tile_cap+1]
    uint32_t* tile_fill_base;    // [tile_cap+1]
    uint32_t* tile_alpha;        // [tile_cap+1] exclusive scan of has-fill flags
    int32_t*  tile_delta;        // [tile_cap+1] backdrop deltas, row-major within a path (as the tiles)
    uint32_t* tile_delta_scan;   // [tile_cap+1] each tile's backdrop before propagation (column sums)
    uint32_t* path_tiles;        // [P+1] tiles per path (scan input)
    uint32_t* path_cols;         // [P+1] tile columns per path (scan input)
    PathCtx*  path_bin;          // [P+1] binning context per global path (written after the path scan)
    int32_t*  col_backdrop;      // [col_cap] above-rect column sums
    uint32_t* seg_line_count;    // [seg_count+1] flattened lines per input segment
    uint32_t* seg_line_base;     // [seg_count+1] exclusive scan (uniform dicing)
    uint32_t* seg_warp_lines;    // [seg_count/32+1] flattened lines per warp of 32 segments
    uint32_t* seg_warp_base;     // [seg_count/32+2] exclusive scan
    unsigned long long* seg_leaves;  // [seg_count] leaf start slots of each segment's subdivision (0: walked)
    float4*   lines;             // [line_cap] flattened lines in emission order
    uint32_t* line_path;         // [line_cap] global path of each line
    uint32_t* line_fill_count;   // [line_cap+1] kept fills per line (frames that write emission indices)
    uint32_t* line_fill_base;    // [line_cap+1] exclusive scan = emission index of the first fill
    uint32_t  line_cap;
    uint2*    fills;             // [fill_cap] LineSegmentU16
    uint32_t* fill_e;            // [fill_cap] emission index
    int4*     tiles;             // [tile_cap] PFCUDATile records
    int4*     clips;             // [tile_cap] PFCUDAClip records of the tiles of clipped draw paths (only)
    uint32_t* alpha_owner;       // [tile_cap] alpha id -> owning global tile
    int32_t*  zbuf;              // [screen_count]
    uint32_t* screen_cnt;        // [screen_count+1]
    uint32_t* screen_base;       // [screen_count+1]
    uint32_t* vis;               // [vis_cap] global tile indices
    int4*     vis_info;          // [vis_cap] per visible tile: see VisInfo
    unsigned long long* vis_key; // [vis_cap] global tile << 32 | slot: draw order within a screen tile
    uint4*    vis_mask;          // [vis_cap * 32] resolved coverage of each visible entry with a mask:
                                 //   16-bit unorm, lane l's 8 pixels (column l & 15, rows (l >> 4) * 8 ..) at 32 * slot + l
    int4*     mask_items;        // [vis_cap] visible entries with a mask: first fill, fill count, meta, slot
    Counters* counters;
    uint32_t dda_limit;
    uint32_t clip_chain_max;     // bound of clip-chain walks (longest chain in the batch)
    uint32_t paint_effects;      // some path of the batch has a gradient or a blend mode other than SrcOver
    // paint
    const OverlayDev* overlays;  // [paint overlays of the batch: gradients, then patterns]
    const uint32_t* texels;      // gradient ramps and pattern pages, RGBA8
    float inv_m[6];              // frame pixel -> scene coordinates (inverse build transform)
    // Differentiable frames (diff != 0): FP32 fills, the curve parameters of
    // every flattened line, and per visible (screen tile, path tile) entry the
    // composite tape the adjoint reads back.
    int diff;
    int d3d11;                   // the D3D11 level's semantics: uniform dicing, truncating bins
    float4*   fills_f;           // [fill_cap] tile-local FP32 fills
    uint32_t* line_seg;          // [line_cap] global segment of each line
    float2*   line_t;            // [line_cap] curve parameters of the line's ends
    uint32_t* tape;              // [vis_cap * 256] packed per pixel, see tape_pack
};

// What the composite needs of a visible tile, gathered by the visibility
// scatter so that the composite reads one record instead of a chain of
// dependent loads: x = first fill of its mask, y = fill count, z = paint
// (RGBA8), w = backdrop (bits 0-7, signed) | even-odd (bit 8) | kind (bits
// 9-10: 0 solid, 1 one mask, 2 clip-combined: read the tile and clip records,
// 3 clip chain) | blend mode (bits 11-15) | gradient index + 1 (bits 16-31,
// 0 = solid paint).  Bits 11-31 are zero for solid SrcOver paint.
enum : uint32_t { kVisSolid = 0, kVisMask = 1, kVisCombine = 2, kVisChain = 3 };

// Tile control bit of a draw tile whose clip path is itself clipped: its
// coverage is the fill rule applied to the minimum of |mask + backdrop| over
// the tile and its clip chain's tiles (the D3D11 level's per-level
// min(coverage, clip mask), shaders/d3d11/fill.cs.glsl:77-84).
constexpr uint32_t kCtrlClipChain = 0x4;
__host__ __device__ __forceinline__ int32_t vis_meta(int8_t backdrop, bool even_odd, uint32_t kind,
                                                     uint32_t paint_fx = 0) {
    return (int32_t)((uint32_t)(uint8_t)backdrop | ((even_odd ? 1u : 0u) << 8) | (kind << 9) | (paint_fx << 11));
}
// blend mode | (gradient index + 1) << 5, the paint effect bits of a visible record
__host__ __device__ __forceinline__ uint32_t paint_fx_bits(uint32_t blend, uint32_t gradient1) {
    return (blend & 31u) | (gradient1 << 5);
}

// One tape word per (visible entry, pixel): coverage c and the composite
// value d below the entry as 14-bit unorms (bits 0-13, 16-29), and the 2-bit
// derivative codes of dc/d(mask) (bits 14-15: the mask in tile.alpha, bits
// 30-31: the clip's mask of a combined tile).
constexpr float kTapeScale = 16383.0f;
__host__ __device__ __forceinline__ uint32_t tape_q(float v) {
    v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
    return (uint32_t)(v * kTapeScale + 0.5f);
}
__host__ __device__ __forceinline__ uint32_t tape_pack(float cov, float dprev, uint32_t code) {
    return tape_q(cov) | ((code & 3u) << 14) | (tape_q(dprev) << 16) | ((code >> 2) << 30);
}
__host__ __device__ __forceinline__ float tape_cov(uint32_t t) { return (float)(t & 0x3fffu) * (1.0f / kTapeScale); }
__host__ __device__ __forceinline__ float tape_dprev(uint32_t t) {
    return (float)((t >> 16) & 0x3fffu) * (1.0f / kTapeScale);
}
__host__ __device__ __forceinline__ uint32_t tape_code(uint32_t t) { return ((t >> 14) & 3u) | ((t >> 30) << 2); }

#ifdef __CUDACC__
__device__ __forceinline__ bool frame_ok(const FrameDev& f) {
    return f.counters->tiles <= f.tile_cap && f.counters->columns <= f.col_cap;
}

// Scene of a global screen tile: the last scene of the frame whose first
// screen tile is at or before it.
__device__ __forceinline__ uint32_t scene_of_screen_tile(const FrameDev& f, uint32_t st_global) {
    uint32_t lo = f.scene_begin, hi = f.scene_begin + f.scene_count;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (f.scene_st[mid] <= st_global) lo = mid; else hi = mid;
    }
    return lo;
}
#endif

// 2-bit derivative codes of the tape: 0 -> 0, 1 -> +1, 2 -> -1.
__host__ __device__ __forceinline__ uint32_t enc_d(float d) { return d > 0.0f ? 1u : (d < 0.0f ? 2u : 0u); }
__host__ __device__ __forceinline__ float dec_d(uint32_t c) { return c == 1u ? 1.0f : (c == 2u ? -1.0f : 0.0f); }

// Scan scratch.  `partials` serves the three-pass scans (reduce, partials,
// down-sweep).  With `lookback` set, scans run in one pass instead: each call
// takes a ticket word and one word per 2,048-value tile and lane from the
// region (which must be zero before the first call: frames clear it once),
// and reports a look-back that gave up in *status.
struct ScanTemp {
    uint32_t* partials;
    uint32_t cap;
    unsigned long long* lookback = nullptr;
    uint32_t lookback_cap = 0;   // words in the region
    uint32_t lookback_used = 0;  // words taken by earlier calls
    uint32_t* status = nullptr;
};

}  // namespace pf
struct PFCUDAGradient;
struct PFCUDAPattern;
struct PFCUDAStrokeInput;
struct PFCUDAStrokeOutput;
struct PFCUDADashInput;
struct PFCUDAOutlineOutput;
struct PFCUDAColorStop;
namespace pf {
// Paint overlays (host): the record of one gradient with its 256-texel ramp,
// or of one image pattern with its texture page, appended to `texels`;
// returns a PF_CUDA_* status.
int32_t build_gradient(const PFCUDAGradient& g, OverlayDev* out, std::vector<uint32_t>& texels, bool* opaque);
int32_t build_pattern(const PFCUDAPattern& p, OverlayDev* out, std::vector<uint32_t>& texels, bool* opaque);

// Stroke to fill (pf_stroke.cu): grow-only device work buffers and one
// synchronous run on stream s; returns a PF_CUDA_* status.
struct StrokeWork;
StrokeWork* stroke_work_create();
void stroke_work_destroy(StrokeWork* w);
int32_t stroke_run(StrokeWork* w, cudaStream_t s, const PFCUDAStrokeInput* in, PFCUDAStrokeOutput* out);
int32_t dash_outlines(StrokeWork* w, cudaStream_t s, const PFCUDAStrokeInput* in, const PFCUDADashInput* dash,
                      PFCUDAOutlineOutput* out);
int32_t stroke_dashed(StrokeWork* w, cudaStream_t s, const PFCUDAStrokeInput* in, const PFCUDADashInput* dash,
                      PFCUDAStrokeOutput* out);

// Launch with programmatic stream serialisation while the calling thread's
// switch is on (frames set it around their launches): the kernel, which must
// start with pdl_enter(), may be scheduled before its predecessor on the
// stream has finished.  Launch errors are left for cudaGetLastError, as with
// the <<< >>> form.
bool& pdl_switch();
template <typename... KArgs, typename... Args>
inline void pdl_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl_switch() ? 1 : 0;
    (void)cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}
// Sets the calling thread's switch for the life of the object.
struct PdlScope {
    bool prev;
    explicit PdlScope(bool on) : prev(pdl_switch()) { pdl_switch() = on; }
    ~PdlScope() { pdl_switch() = prev; }
};

// Number of kernels this library has launched (host counter).
uint64_t launch_counter();
void count_launch(uint32_t n = 1);
// Multiprocessors of the current device (queried once per device; grid sizes
// of the launches that do not carry a FrameDev).
uint32_t device_sm_count();
// Blocks of `threads` threads of `kernel` resident on one multiprocessor of
// the current device (persistent grids are the multiprocessors times this);
// queried once per kernel, block size and device.
int resident_blocks_of(const void* kernel, int threads);
template <typename K>
int resident_blocks(K kernel, int threads) { return resident_blocks_of((const void*)kernel, threads); }


void launch_transform(const float2* in, float2* out, uint32_t n, const float* m6, cudaStream_t s);
// Segments per contour reference and their records. The reference count is
// the device-side *d_n clamped to the buffers' capacity cap (d_n NULL: cap).
// contour_total: contours behind contour_starts (a reference past it is malformed).
void launch_contour_segcount(const uint32_t* ord_contour, const uint64_t* d_n, uint32_t cap,
                             const uint32_t* contour_starts, uint32_t contour_total, const uint8_t* flags,
                             uint32_t* seg_count, uint32_t* status, cudaStream_t s);
void launch_contour_segemit(const uint32_t* ord_contour, const uint32_t* ord_path, const uint64_t* d_n, uint32_t cap,
                            const uint32_t* contour_starts, uint32_t contour_total, const uint8_t* flags,
                            const uint32_t* seg_base, SegRec* segs, cudaStream_t s);

// ---- scene packing at upload (pf_pack.cu) ----------------------------------
// One scene of an upload batch, as the packing kernels see it.
struct ScenePackDev {
    uint32_t first_path, nclip, ndraw;     // global index of the scene's path 0; clip, draw paths
    uint32_t contour_base, contour_count;  // global index of the scene's contour 0; contours
    uint32_t point_base, point_count;      // global index of the scene's point 0; points
    uint32_t draw_base;                    // global draw index of the scene's draw path 0
    uint32_t overlay_base, overlay_count;  // global overlay index of the scene's overlay 1, minus 1; count
};
// What the host reads back after packing.
struct PackInfo {
    uint64_t nord;       // contour references of all paths (a 32-bit scan total)
    uint64_t segs;       // segments of all references
    uint64_t refs;       // the same references summed in 64 bits: nord is valid while refs < 2^31
    uint32_t status;     // kStatusMalformed: an invalid record or index
    uint32_t chain_max;  // longest chain of clip paths behind a path
    uint32_t flags;      // kPackNestedClips | kPackBlendModes
    uint32_t pad;
};
constexpr uint32_t kPackNestedClips = 1u, kPackBlendModes = 2u;
// The per-path tables a frame reads (indexed by global path; draw-indexed for alpha).
struct PathTablesDev {
    uint32_t* ncont;        // contour references (0 for an invalid record); scanned into first_ord
    uint32_t* paint;        // RGBA8
    uint32_t* local;        // index within the scene's clip paths or draw paths
    uint32_t* scene_of;
    int32_t* clip;          // global clip path, or -1
    uint8_t* rule;
    uint8_t* is_clip;
    uint32_t* draw_index;   // kInvalid for clip paths
    float* alpha;           // default paint alpha of each draw path (draw-indexed)
    uint8_t* blend;
    uint32_t* overlay;      // global overlay + 1, or 0
    uint8_t* occludes;
};
// Global contour boundaries from each scene's own (validated) boundaries.
void launch_pack_starts(const uint32_t* raw, uint32_t* starts, const ScenePackDev* scenes, uint32_t scene_count,
                        uint32_t boundary_count, uint32_t point_total, PackInfo* info, cudaStream_t s);
void launch_pack_paths(const PFCUDAPath* paths, uint32_t path_count, const ScenePackDev* scenes,
                       uint32_t scene_count, const uint8_t* overlay_opaque, const PathTablesDev& t, PackInfo* info,
                       cudaStream_t s);
// ord_contour / ord_path from first_ord (references past cap are dropped: the host grows and re-runs).
void launch_pack_order(const PFCUDAPath* paths, uint32_t path_count, const ScenePackDev* scenes,
                       const uint32_t* scene_of, const uint32_t* ncont, const uint32_t* first_ord, uint32_t cap,
                       uint32_t* ord_contour, uint32_t* ord_path, cudaStream_t s);
void launch_pack_chains(const int32_t* clip, const uint8_t* is_clip, const uint32_t* scene_of,
                        const ScenePackDev* scenes, uint32_t path_count, PackInfo* info, cudaStream_t s);
// Per scene: [first segment, end segment).
void launch_pack_ranges(const ScenePackDev* scenes, uint32_t scene_count, const uint32_t* first_ord,
                        const uint32_t* seg_base, const uint64_t* d_nord, uint32_t cap, uint32_t* ranges,
                        cudaStream_t s);
void launch_bound(const FrameDev& f, const uint32_t* ord_contour, const uint32_t* contour_starts, cudaStream_t s);
void launch_path_scan(const FrameDev& f, ScanTemp& tmp, cudaStream_t s);
void launch_flatten(const FrameDev& f, ScanTemp& tmp, cudaStream_t s);
void launch_bin_count(const FrameDev& f, cudaStream_t s);
void launch_bin_emit(const FrameDev& f, cudaStream_t s);
// Exclusive scan of n (device-resident count at d_n, capacity n_cap) u32
// values; mode 0: values, mode 1: (value != 0).  Writes out[0..n] (out[n] = total)
// and, when total_out != NULL, the total as u64.
void launch_scan(const uint32_t* in, uint32_t* out, const uint64_t* d_n, uint32_t n_host, uint32_t n_cap,
                 int mode, uint64_t* total_out, ScanTemp& tmp, cudaStream_t s);
// The same scan of n host-counted values, each launch's status taken from its
// own return value (the runtime's pending error state is not read).
cudaError_t launch_scan_checked(const uint32_t* in, uint32_t* out, uint32_t n, ScanTemp& tmp, cudaStream_t s);
// Several exclusive scans over arrays of one length (device count at d_n,
// clamped to n_cap); scratch needs count * (n_cap / 2048 + 1) partials.
constexpr int kMaxScanLanes = 3;
struct ScanLanes {
    const uint32_t* in[kMaxScanLanes];
    uint32_t* out[kMaxScanLanes];
    uint64_t* total[kMaxScanLanes];
    int mode[kMaxScanLanes];
    // optional: the lane's inclusive sums, written after the lane's own reads
    // (so it may be the lane's input; lanes that read the same input come
    // before it)
    uint32_t* incl[kMaxScanLanes];
    int count;
};
void launch_scan_multi(const ScanLanes& lanes, const uint64_t* d_n, uint32_t n_cap, ScanTemp& tmp, cudaStream_t s);

void launch_column_backdrops(const FrameDev& f, cudaStream_t s);
void launch_propagate(const FrameDev& f, bool clip_pass, cudaStream_t s);
void launch_visible(const FrameDev& f, bool scatter, cudaStream_t s);
// mode 0: RGBA8, 1: R8 single channel, 2: FP32 single channel
// The fill pass: resolved coverage of every visible tile with a mask.
void launch_mask(const FrameDev& f, cudaStream_t s);
// The composite (after the fill pass).
void launch_composite(const FrameDev& f, int mode, void* out, const float4& background, cudaStream_t s);
void launch_masks(const FrameDev& f, float* alpha_masks, float* tile_cov, cudaStream_t s);

// Differentiable frames: the FP32 composite that records the tape, and the
// adjoint (dL/dimage -> dL/dmask per alpha tile and dL/dalpha per draw path,
// then dL/dmask -> dL/dpoints through every flattened line).
void launch_composite_diff(const FrameDev& f, float* out, const float4& background, cudaStream_t s);
void launch_composite_bwd(const FrameDev& f, const float* d_image, float* grad_mask, float* grad_alpha,
                          cudaStream_t s);
void launch_line_grad(const FrameDev& f, const float* grad_mask, float2* grad_points, cudaStream_t s);
void launch_points_grad_transform(float2* grad_points, uint32_t n, const float* m4, cudaStream_t s);

}  // namespace pf

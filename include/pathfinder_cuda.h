/*
 * pathfinder_cuda.h — C ABI of the CUDA renderer level (sm_103a, one GPU).
 *
 * This is the drop-in boundary for Pathfinder's compute rasterization path
 * (bound -> flatten -> bin into 16x16 tiles -> backdrop propagate -> group
 * fills by tile -> trapezoid-area fill -> tile composite).  It plays the role
 * that `RendererLevel::D3D11` (renderer/src/gpu/options.rs:41-46) plays in the
 * reference: the scene builder hands over the scene outlines once per scene
 * epoch (`RenderCommand::UploadSceneD3D11`, renderer/src/gpu_data.rs:75-101,
 * renderer/src/builder.rs:190-216) and then asks for frames.
 *
 * Conventions, in the style of the reference's C bindings (c/src/lib.rs):
 *   - opaque handles, created by `*Create` and released by `*Destroy`
 *     (c/src/lib.rs:606-620);
 *   - unlike the reference, every call returns an int32_t status
 *     (PF_CUDA_OK == 0); a capacity failure reports the size it needed;
 *   - pointers are plain; each argument states whether it may point to host
 *     or device memory;
 *   - all calls are asynchronous on the renderer's stream unless they say
 *     that they synchronise.
 *
 * Reference interfaces these entry points replace are cited per function.
 */
#ifndef PATHFINDER_CUDA_H
#define PATHFINDER_CUDA_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PF_CUDA_ABI_VERSION 1

/* ---- status codes -------------------------------------------------------- */
#define PF_CUDA_OK                 0
#define PF_CUDA_ERR_INVALID        1  /* bad argument or malformed scene            */
#define PF_CUDA_ERR_CAPACITY       2  /* a device buffer was too small (see needed) */
#define PF_CUDA_ERR_LAUNCH         3  /* a CUDA call failed                          */
#define PF_CUDA_ERR_NO_DEVICE      4  /* no CUDA device / driver                     */
#define PF_CUDA_ERR_LIMIT          5  /* a bounded device loop hit its limit         */
#define PF_CUDA_ERR_NO_SCENE       6  /* render called before a scene was uploaded   */

/* ---- geometry / colour (same layout as c/src/lib.rs:102-170) ------------- */
typedef struct PFVector2F { float x, y; } PFVector2F;
typedef struct PFVector2I { int32_t x, y; } PFVector2I;
typedef struct PFRectF { PFVector2F origin, lower_right; } PFRectF;
typedef struct PFRectI { PFVector2I origin, lower_right; } PFRectI;
typedef struct PFColorU { uint8_t r, g, b, a; } PFColorU;
typedef struct PFColorF { float r, g, b, a; } PFColorF;
/* Row-major, as PFMatrix2x2F/PFTransform2F in c/src/lib.rs:150-162. */
typedef struct PFTransform2F { float m00, m01, m10, m11; PFVector2F vector; } PFTransform2F;

/* ---- point flags and fill rules (content/src/outline.rs:32-41,
 *      content/src/fill.rs) ---------------------------------------------- */
#define PF_POINT_FLAG_CONTROL_POINT_0 0x01
#define PF_POINT_FLAG_CONTROL_POINT_1 0x02
#define PF_FILL_RULE_WINDING  0
#define PF_FILL_RULE_EVEN_ODD 1
/* BlendMode (content/src/effects.rs:99-167), numbered with the default
 * (SrcOver) at 0.  Porter-Duff modes blend with the reference's blend states
 * (renderer/src/gpu/blend.rs); the others mix with the destination as the
 * reference's composite() does (shaders/tile_fragment.inc.glsl:414-535).
 * Clear, Copy, SrcIn, DestIn, SrcOut and DestAtop are destructive: the path's
 * tiles span the whole view box (renderer/src/builder.rs:430-434). */
#define PF_BLEND_MODE_SRC_OVER     0
#define PF_BLEND_MODE_CLEAR        1
#define PF_BLEND_MODE_COPY         2
#define PF_BLEND_MODE_SRC_IN       3
#define PF_BLEND_MODE_SRC_OUT      4
#define PF_BLEND_MODE_SRC_ATOP     5
#define PF_BLEND_MODE_DEST_IN      6
#define PF_BLEND_MODE_DEST_OUT     7
#define PF_BLEND_MODE_DEST_OVER    8
#define PF_BLEND_MODE_DEST_ATOP    9
#define PF_BLEND_MODE_XOR          10
#define PF_BLEND_MODE_LIGHTER      11
#define PF_BLEND_MODE_DARKEN       12
#define PF_BLEND_MODE_LIGHTEN      13
#define PF_BLEND_MODE_MULTIPLY     14
#define PF_BLEND_MODE_SCREEN       15
#define PF_BLEND_MODE_HARD_LIGHT   16
#define PF_BLEND_MODE_OVERLAY      17
#define PF_BLEND_MODE_COLOR_DODGE  18
#define PF_BLEND_MODE_COLOR_BURN   19
#define PF_BLEND_MODE_SOFT_LIGHT   20
#define PF_BLEND_MODE_DIFFERENCE   21
#define PF_BLEND_MODE_EXCLUSION    22
#define PF_BLEND_MODE_HUE          23
#define PF_BLEND_MODE_SATURATION   24
#define PF_BLEND_MODE_COLOR        25
#define PF_BLEND_MODE_LUMINOSITY   26
#define PF_BLEND_MODE_COUNT        27

/* Gradients (content/src/gradient.rs:27-81). */
#define PF_GRADIENT_LINEAR      0
#define PF_GRADIENT_RADIAL      1
#define PF_GRADIENT_WRAP_CLAMP  0
#define PF_GRADIENT_WRAP_REPEAT 1

/* ColorStop (content/src/gradient.rs:38-44). */
typedef struct PFCUDAColorStop {
    float    offset;                   /* 0 .. 1 */
    PFColorU color;
} PFCUDAColorStop;

/* Gradient (content/src/gradient.rs:27-33, 46-72), in scene coordinates.
 * Stops are ordered by offset, equal offsets in the order given
 * (Gradient::add, :158-164).  Rendered through a 256-texel ramp sampled with
 * linear filtering, as the reference's gradient tiles
 * (renderer/src/paint.rs:855-863). */
typedef struct PFCUDAGradient {
    int32_t  kind;                     /* PF_GRADIENT_LINEAR / PF_GRADIENT_RADIAL            */
    int32_t  wrap;                     /* PF_GRADIENT_WRAP_*                                 */
    PFVector2F from, to;               /* linear: the line; radial: the line between centres */
    float    radius0, radius1;         /* radial                                             */
    PFTransform2F transform;           /* radial: gradient space -> scene space              */
    const PFCUDAColorStop* stops;      /* host memory                                        */
    uint32_t stop_count;
    uint32_t reserved;
} PFCUDAGradient;

/* Gradient::sample (content/src/gradient.rs:188-211) of the gradient's
 * stops at t, and the 256-texel colour ramp the composite samples
 * (texel x = sample((x + 0.5) / 256), renderer/src/paint.rs:855-863).
 * Host-only; no device or renderer is needed. */
int32_t PFCUDAGradientSample(const PFCUDAGradient* gradient, float t, PFColorU* out);
int32_t PFCUDAGradientRamp(const PFCUDAGradient* gradient, PFColorU* out_256);

/* Image patterns (Pattern, content/src/pattern.rs:21-200, with PatternSource::
 * Image).  The image is placed as the reference's texture allocator places it:
 * on its own texture page, with one transparent texel of border on each axis
 * that does not repeat (renderer/src/paint.rs:498-530); pattern space (0, 0)
 * is the page's corner.  PatternFilter (content/src/effects.rs:64-95): a
 * one-direction Gaussian blur, or a colour matrix (5 columns of RGBA, the
 * feColorMatrix layout: out = M * colour + column 4).  The text filter
 * belongs to the text front-end and is not on this path. */
#define PF_PATTERN_REPEAT_X      0x1
#define PF_PATTERN_REPEAT_Y      0x2
#define PF_PATTERN_NO_SMOOTHING  0x4   /* nearest texel instead of linear filtering */
#define PF_PATTERN_FILTER_NONE          0
#define PF_PATTERN_FILTER_BLUR_X        1
#define PF_PATTERN_FILTER_BLUR_Y        2
#define PF_PATTERN_FILTER_COLOR_MATRIX  3

typedef struct PFCUDAPattern {
    const PFColorU* pixels;            /* width * height texels, row 0 first, straight alpha */
    uint32_t width, height;            /* >= 1                                            */
    PFTransform2F transform;           /* pattern space -> scene space                    */
    uint32_t flags;                    /* PF_PATTERN_* bits                               */
    int32_t  filter;                   /* PF_PATTERN_FILTER_*                             */
    float    blur_sigma;               /* BLUR_X / BLUR_Y: > 0                            */
    float    color_matrix[20];         /* COLOR_MATRIX: columns 0-4, RGBA each            */
} PFCUDAPattern;

#define PF_MEMORY_HOST   0
#define PF_MEMORY_DEVICE 1
/* Frame outputs only (PFCUDARenderScene, PFCUDARenderCoverage): host memory
 * written by one device-to-host copy of the frame's image, which the copy
 * engine makes after the composite, instead of by the composite itself.  On
 * page-locked memory the copy leaves the SMs free for other streams' work
 * (frames in flight on other renderers). */
#define PF_MEMORY_HOST_COPY 2

/* One path of the scene: a range of contours of the shared outline buffers.
 * Mirrors DrawPath / ClipPath (renderer/src/scene.rs:441-472): outline,
 * paint (a colour, or a colour with a gradient or pattern overlay), fill rule, blend mode,
 * optional clip path. */
typedef struct PFCUDAPath {
    uint32_t first_contour;
    uint32_t contour_count;
    PFColorU paint;          /* draw paths: solid paint; ignored for clip paths  */
    int32_t  clip_path;      /* draw paths: index into clip paths, or -1         */
    uint8_t  fill_rule;      /* PF_FILL_RULE_*                                   */
    uint8_t  blend_mode;     /* draw paths: PF_BLEND_MODE_*                      */
    uint16_t overlay;        /* draw paths: 0 = solid paint; 1 <= k <= gradient_count:
                                gradients[k - 1]; above: patterns[k - 1 - gradient_count].
                                The overlay's colour SrcIn the paint (its alpha x paint alpha) */
} PFCUDAPath;

/* The scene as flat outline buffers.  Every contour is treated as closed
 * (Outline::close_all_contours, content/src/outline.rs:279-281, applied by
 * Scene::apply_render_options, renderer/src/scene.rs:228-274).
 * Contour c owns points [contour_starts[c], contour_starts[c+1]). */
typedef struct PFCUDASceneDesc {
    const PFVector2F* points;          /* point_count                        */
    const uint8_t*    point_flags;     /* point_count PF_POINT_FLAG_* bits    */
    const uint32_t*   contour_starts;  /* contour_count + 1                   */
    const PFCUDAPath* clip_paths;      /* host memory always                  */
    const PFCUDAPath* draw_paths;      /* host memory always                  */
    uint32_t point_count;
    uint32_t contour_count;
    uint32_t clip_path_count;
    uint32_t draw_path_count;
    PFRectF  view_box;                 /* Scene::set_view_box                 */
    int32_t  memory;                   /* PF_MEMORY_* for points/flags/starts */
    const PFCUDAGradient* gradients;   /* host memory; may be NULL when unused */
    uint32_t gradient_count;
    const PFCUDAPattern* patterns;     /* host memory; may be NULL when unused */
    uint32_t pattern_count;
} PFCUDASceneDesc;

/* BuildOptions (renderer/src/options.rs:53-61): only the 2-D transform is on
 * this path (dilation and subpixel AA are front-end preprocessing). */
typedef struct PFCUDABuildOptions {
    PFTransform2F transform;
    int32_t       has_transform;       /* 0: identity (no arithmetic applied) */
} PFCUDABuildOptions;

/* RendererOptions (renderer/src/gpu/options.rs:19-33). */
typedef struct PFCUDARendererOptions {
    PFColorF background_color;         /* premultiplied clear colour           */
    int32_t  has_background_color;     /* 0: transparent                       */
    int32_t  flags;                    /* PF_CUDA_RENDERER_* bits, 0 = default */
} PFCUDARendererOptions;

/* The D3D11 level's tiling semantics instead of the CPU tiler's (as choosing
 * RendererLevel::D3D11, renderer/src/gpu/options.rs:41-46): curves diced
 * uniformly by Sederberg's bound and lines into pieces of at most 16 px, piece
 * ends rounded to 1/256 px (shaders/d3d11/dice.cs.glsl), binned without the
 * view-box clip with truncating 8.8 fills (shaders/d3d11/bin.cs.glsl).  Fills
 * then differ from the CPU tiler's; coverage, resolve and composite do not
 * change.  Not available for differentiable frames. */
#define PF_CUDA_RENDERER_D3D11_SEMANTICS 0x1

/* RenderStats (renderer/src/gpu/perf.rs:21-44) + the device counters of the
 * last frame. */
typedef struct PFCUDARenderStats {
    uint64_t path_count;
    uint64_t segment_count;     /* input segments (lines+quads+cubics, with close) */
    uint64_t line_count;        /* flattened lines                                 */
    uint64_t fill_count;        /* fills (Fill records)                            */
    uint64_t tile_count;        /* path tiles (TileObjectPrimitive records)        */
    uint64_t alpha_tile_count;  /* tiles with a mask                               */
    uint64_t visible_tile_count;/* tiles composited after occlusion culling        */
    uint64_t screen_tile_count;
    uint64_t status;            /* device status bits of the last frame            */
    double   gpu_time_ms;       /* CUDA-event time of the last frame               */
    uint64_t kernel_launches;   /* kernels this library launched for the frame     */
    uint64_t mask_tile_count;   /* visible tiles whose coverage the fill pass computed */
    uint64_t mask_fill_count;   /* fills those tiles hold (the fills the fill pass reads) */
} PFCUDARenderStats;

/* Record layouts read back for parity checks. */
/* Fill (renderer/src/gpu_data.rs:354-363): LineSegmentU16 in 8.8 fixed point
 * relative to the tile; `link` here is the fill's emission index in the CPU
 * tiler's order (path, segment, flattened line, DDA step, auxiliary). */
typedef struct PFCUDAFill {
    uint16_t from_x, from_y, to_x, to_y;
    uint32_t emission_index;
} PFCUDAFill;
/* TileObjectPrimitive (renderer/src/gpu_data.rs:264-275). */
typedef struct PFCUDATile {
    int16_t  tile_x, tile_y;
    uint32_t alpha_tile_id;     /* 0xffffffff: solid tile */
    uint32_t path_id;           /* index within clip paths or within draw paths */
    uint16_t color;
    uint8_t  ctrl;              /* 0: clip path tile; bit 0 nonzero, bit 1 even-odd; bit 2: behind a
                                   clip chain (its clip path is itself clipped; coverage is the rule
                                   applied to the minimum of |mask + backdrop| over the chain) */
    int8_t   backdrop;
} PFCUDATile;
/* Clip (renderer/src/gpu_data.rs:436-442). */
typedef struct PFCUDAClip {
    uint32_t dest_tile_id;
    int32_t  dest_backdrop;
    uint32_t src_tile_id;
    int32_t  src_backdrop;
} PFCUDAClip;

typedef struct PFCUDARenderer* PFCUDARendererRef;

/* ---- renderer lifetime ---------------------------------------------------
 * Replaces PFGLRendererCreate / PFMetalRendererCreate (c/src/lib.rs:606-615,
 * 646-657) and Renderer::new (renderer/src/gpu/renderer.rs:181-341). */
int32_t PFCUDARendererCreate(int32_t device_ordinal,
                             const PFCUDARendererOptions* options,
                             PFCUDARendererRef* out_renderer);
/* Replaces PFGLRendererDestroy (c/src/lib.rs:618-620). */
int32_t PFCUDARendererDestroy(PFCUDARendererRef renderer);
/* Runs subsequent work on `stream` (a cudaStream_t; NULL = the renderer's own;
 * (void*)1 = cudaStreamLegacy, the legacy default stream). */
int32_t PFCUDARendererSetStream(PFCUDARendererRef renderer, void* stream);
/* Renderer::set_options background colour (gpu/options.rs:27-30). */
int32_t PFCUDARendererSetOptions(PFCUDARendererRef renderer,
                                 const PFCUDARendererOptions* options);

/* ---- scene upload ----------------------------------------------------------
 * Replaces RenderCommand::UploadSceneD3D11 + RendererD3D11::upload_scene
 * (renderer/src/gpu/d3d11/renderer.rs:236-241) and the segment packing of
 * SegmentsD3D11::add_path (renderer/src/builder.rs:804-841), which here runs
 * on the GPU.  Copies the outline buffers to device memory (host or device
 * source per desc->memory).  The scene stays resident until the next upload
 * (scene-epoch caching, renderer/src/builder.rs:190-216). */
int32_t PFCUDASceneUpload(PFCUDARendererRef renderer, const PFCUDASceneDesc* scene);

/* ---- frames ----------------------------------------------------------------
 * Scene::build_and_render (renderer/src/scene.rs:369-381) for the CUDA level:
 * Renderer::begin_scene / render_command / end_scene
 * (renderer/src/gpu/renderer.rs:350-460) with the seven D3D11 dispatches
 * (renderer/src/gpu/d3d11/renderer.rs:427-782) replaced by this library's
 * kernels.  Writes premultiplied RGBA8, row 0 = top, into `out_rgba8`
 * (width*height*4 bytes; host or device memory, or host memory written by a
 * copy, per out_memory): every pixel
 * of the view box's 16x16 screen tiles; pixels outside them keep the
 * buffer's contents.  Synchronises the stream before returning. */
int32_t PFCUDARenderScene(PFCUDARendererRef renderer,
                          const PFCUDABuildOptions* options,
                          int32_t width, int32_t height,
                          uint8_t* out_rgba8, int32_t out_memory);

/* Same frame, but only enqueued: no synchronisation and no status readback.
 * `out_rgba8_device` must be device memory.  Capacity overflow is reported
 * by the next PFCUDARenderStatus call.  Used for CUDA-graph capture. */
int32_t PFCUDARenderSceneAsync(PFCUDARendererRef renderer,
                               const PFCUDABuildOptions* options,
                               int32_t width, int32_t height,
                               uint8_t* out_rgba8_device);
/* Synchronises and returns the status of the frames enqueued since the last
 * call (PF_CUDA_OK or the first error), with the needed capacity on overflow. */
int32_t PFCUDARenderStatus(PFCUDARendererRef renderer, uint64_t* out_needed);

/* Single-channel FP32 render: per pixel, SrcOver of (paint alpha x coverage)
 * over the draw paths in order; used by the differentiable form.  Row 0 = top.
 * Synchronises. */
int32_t PFCUDARenderCoverage(PFCUDARendererRef renderer,
                             const PFCUDABuildOptions* options,
                             int32_t width, int32_t height,
                             float* out, int32_t out_memory);

/* Raw mask of every alpha tile (the D3D9 mask texture contents, fill.fs.glsl:
 * sum of trapezoid areas, no backdrop) as FP32 [alpha_tile_count][16][16],
 * and the resolved coverage of every path tile (sampleMask,
 * shaders/tile_fragment.inc.glsl:539-556) as FP32 [tile_count][16][16].
 * Either pointer may be NULL.  Host memory.  Valid after a render call. */
int32_t PFCUDAReadMasks(PFCUDARendererRef renderer,
                        float* out_alpha_masks, uint64_t alpha_capacity,
                        float* out_tile_coverage, uint64_t tile_capacity);

/* Read back the records of the last frame for parity checks (host memory).
 * fills: grouped by tile; within a tile in any order (emission_index gives
 * the canonical order).  fill_tile: the global tile index of each fill.
 * tiles: one record per path tile, clip paths first, each path row-major
 * over its tile rect.  path_tile_offsets: clip_count+draw_count+1 entries.
 * clips: one record per draw tile of a clipped draw path (gpu_data Clip).
 * z_buffer: one i32 per screen tile.  Any pointer may be NULL. */
int32_t PFCUDAReadRecords(PFCUDARendererRef renderer,
                          PFCUDAFill* fills, uint32_t* fill_tile, uint64_t fill_capacity,
                          PFCUDATile* tiles, uint64_t tile_capacity,
                          uint32_t* path_tile_offsets, PFRectI* path_tile_rects,
                          uint64_t path_capacity,
                          PFCUDAClip* clips, int32_t* z_buffer, uint64_t z_capacity);

/* Renderer::stats (renderer/src/gpu/renderer.rs:626) + last_rendering_time
 * (:537). */
int32_t PFCUDAGetStats(PFCUDARendererRef renderer, PFCUDARenderStats* out_stats);

/* ---- batched frames --------------------------------------------------------
 * Many independent scenes (glyph sets, tiles of an atlas, a batch of
 * differentiable scenes) rendered by one set of launches: the batch is
 * uploaded once and any contiguous range of its scenes is one frame.  The
 * reference renders one scene per Renderer call; this has no direct
 * counterpart there. */
#define PF_CUDA_FORMAT_RGBA8 0   /* premultiplied RGBA8, 4 bytes per pixel */
#define PF_CUDA_FORMAT_R8    1   /* single channel, SrcOver of paint alpha x coverage, 1 byte */
#define PF_CUDA_FORMAT_F32   2   /* the same single channel as float */

/* Where a scene's pixels go: scene pixel (x, y) inside `clip` is written to
 * element out_offset + (y - origin_y) * pitch + (x - origin_x) of the output
 * buffer (elements of the format's size).  Pixels outside `clip` are not
 * written, so scenes may share one output (e.g. glyph cells of an atlas). */
typedef struct PFCUDASceneTarget {
    uint64_t out_offset;
    int32_t  pitch;
    int32_t  origin_x, origin_y;
    PFRectI  clip;
} PFCUDASceneTarget;

/* Upload `scene_count` scenes (each as in PFCUDASceneUpload) with their
 * targets.  Replaces the resident scene(s). */
int32_t PFCUDASceneUploadBatch(PFCUDARendererRef renderer, const PFCUDASceneDesc* scenes,
                               const PFCUDASceneTarget* targets, uint32_t scene_count);
/* Render scenes [first_scene, first_scene + scene_count) of the uploaded batch
 * into device memory `out_device` in `format`; synchronises, regrows buffers
 * and re-runs once on overflow. */
int32_t PFCUDARenderBatch(PFCUDARendererRef renderer, const PFCUDABuildOptions* options,
                          uint32_t first_scene, uint32_t scene_count, int32_t format, void* out_device);
/* The same frame, only enqueued (check PFCUDARenderStatus afterwards). */
int32_t PFCUDARenderBatchAsync(PFCUDARendererRef renderer, const PFCUDABuildOptions* options,
                               uint32_t first_scene, uint32_t scene_count, int32_t format, void* out_device);

/* CUDA graph of a whole frame: runs the frame once synchronously (sizing the
 * buffers), then captures its launches into a graph bound to these
 * arguments.  PFCUDAGraphLaunch replays it asynchronously on the renderer's
 * stream (status via PFCUDARenderStatus; an overflow there means the scene
 * changed: capture again).  Uploading a scene releases the graph. */
int32_t PFCUDAGraphCapture(PFCUDARendererRef renderer, const PFCUDABuildOptions* options,
                           uint32_t first_scene, uint32_t scene_count, int32_t format, void* out_device);
int32_t PFCUDAGraphLaunch(PFCUDARendererRef renderer);
int32_t PFCUDAGraphRelease(PFCUDARendererRef renderer);

/* Launch shapes of the kernels (outputs never depend on them). */
typedef struct PFCUDATuning {
    int32_t flatten_threads;     /* 64, 128 or 256 */
    int32_t bin_threads;         /* 128, 256 or 512 */
    int32_t bin_blocks_per_sm;   /* 4 .. 64: the count pass's grid (the emit pass runs two waves of
                                    resident blocks beside propagation and visibility) */
    int32_t composite_warps;     /* 2, 4 or 8 */
    int32_t composite_batch;     /* screen tiles per work item of the persistent composite: 1, 2, 4 or 8 */
    int32_t mask_stage_fills;    /* 0: the fill pass reads each mask tile's fills from global memory (the
                                    default); 1 .. 128: ranges of at least this many fills are copied into
                                    shared memory by bulk copy (cp.async.bulk + mbarrier), one work item
                                    ahead of their use */
} PFCUDATuning;
int32_t PFCUDASetTuning(PFCUDARendererRef renderer, const PFCUDATuning* tuning);
int32_t PFCUDAGetTuning(PFCUDARendererRef renderer, PFCUDATuning* out_tuning);
/* Autotuner: times `repeats` frames of the given range per candidate shape
 * (coordinate descent over the six parameters), keeps the fastest and
 * returns it.  Synchronises. */
int32_t PFCUDAAutotune(PFCUDARendererRef renderer, const PFCUDABuildOptions* options,
                       uint32_t first_scene, uint32_t scene_count, int32_t format, void* out_device,
                       int32_t repeats, PFCUDATuning* out_best);

/* Per-stage CUDA-event timing of subsequent frames (Renderer timer queries,
 * renderer/src/gpu/perf.rs:96-186, bucketed like RenderTime :223-240).
 * Stages: 0 bound, 1 flatten, 2 bin count, 3 scans, 4 bin emit,
 * 5 propagate, 6 visibility, 7 fill (coverage of the visible mask tiles),
 * 8 composite.  Stage-timed frames run every kernel in order on the
 * renderer's stream (other frames run independent stages side by side). */
#define PF_CUDA_STAGE_COUNT 9
int32_t PFCUDASetProfiling(PFCUDARendererRef renderer, int32_t enable);
/* Milliseconds per stage of the last profiled frame; synchronises. */
int32_t PFCUDAGetStageTimes(PFCUDARendererRef renderer, float* out_ms, int32_t capacity);

/* Device-wide exclusive prefix sum of `n` uint32 values, the primitive that
 * turns per-tile fill counts into fill offsets and tile-has-fill flags into
 * alpha-tile ids (it replaces the D3D11 level's counter readbacks,
 * renderer/src/gpu/d3d11/renderer.rs:218-229, :634-648).  `in` and `out`
 * are device pointers (`in` may be NULL when n == 0); out[0..n] is written,
 * out[n] = total.  Scratch comes
 * from the renderer (grown with cudaMalloc when needed).  Runs on the
 * renderer's stream and synchronises. */
int32_t PFCUDAExclusiveScan(PFCUDARendererRef renderer, const uint32_t* in, uint32_t* out, uint32_t n);

/* The same scan for callers that cannot allocate device memory while they
 * work (a frame loop that must not stall on cudaMalloc's implicit device
 * synchronisation, a host whose device memory belongs to its own pool, code
 * running while another module captures a CUDA graph).  This entry point has
 * no counterpart in the reference.  It allocates nothing: its scratch is a
 * fixed 32 KiB device array that every GPU loading the library holds until
 * the process exits.  At most 16,777,216 values per call; larger n returns
 * PF_CUDA_ERR_CAPACITY without launching.  `in`/`out` are device pointers
 * (`in` may be NULL when n == 0), out[0..n] is written, out[n] = total.
 * Asynchronous on `stream` (a cudaStream_t, NULL = legacy default stream).
 * The first call on a device looks up the array's device address, so make
 * that first call before any stream capture; the address is kept for the
 * life of the process, so the library must not be used across a reset of the
 * device (cudaDeviceReset).  All calls share the array: calls that overlap on
 * the GPU race, so serialise them.  The status covers this call's own
 * launches only: the runtime's pending error from earlier work is neither
 * read nor cleared. */
int32_t PFCUDAExclusiveScanNoAlloc(const uint32_t* in, uint32_t* out, uint32_t n, void* stream);

/* ---- differentiable rendering ----------------------------------------------
 * No counterpart in the reference (it has no backward pass); the entry points
 * follow PFCUDARenderCoverage.  A differentiable frame renders single-channel
 * FP32 coverage (SrcOver of alpha x coverage) from FP32 fills, without the
 * 8.8 rounding of the parity path, so the image is piecewise smooth in the
 * control points, and keeps a per-pixel tape for PFCUDABackward.  Gradients
 * are exact for pixels wholly inside the scene's view box (use pixel-aligned
 * view boxes), hold the flattening (the subdivision of each curve) fixed, and
 * are one-sided at coverage kinks (|winding| = 1 for nonzero, the even-odd
 * fold, the clip combine's min). */

/* Replaces every point of the uploaded scene or batch (batch order, `count`
 * = all points) without re-uploading the structure; `memory` says where
 * `points` lives.  Contours, flags and paths stay as uploaded. */
int32_t PFCUDASetPoints(PFCUDARendererRef renderer, const PFVector2F* points, uint64_t count,
                        int32_t memory);

/* Differentiable frame over scenes [first, first + count).  Scenes uploaded
 * without a target draw into a width x height FP32 image, as in
 * PFCUDARenderCoverage; pass width = height = 0 to keep the targets of
 * PFCUDASceneUploadBatch.  `draw_alpha` (device, one float per draw path of
 * the whole batch in batch order; NULL = paint alpha / 255) is the paint
 * alpha; it is copied.  Synchronous (sizes its buffers like
 * PFCUDARenderBatch). */
int32_t PFCUDARenderDiff(PFCUDARendererRef renderer, const PFCUDABuildOptions* options, uint32_t first,
                         uint32_t count, int32_t width, int32_t height, const float* draw_alpha,
                         float* out_device);
/* The same frame enqueued without synchronising (buffers as sized by earlier
 * frames; an overflow surfaces in PFCUDARenderStatus, and the frame and its
 * adjoint must then be re-run). */
int32_t PFCUDARenderDiffAsync(PFCUDARendererRef renderer, const PFCUDABuildOptions* options, uint32_t first,
                              uint32_t count, int32_t width, int32_t height, const float* draw_alpha,
                              float* out_device);

/* Adjoint of the last PFCUDARenderDiff (PF_CUDA_ERR_INVALID if another frame,
 * upload or PFCUDASetPoints came in between).  d_image: dL/d(image), device,
 * laid out as that frame's output.  Overwrites d_points (device, one PFVector2F
 * per uploaded point: dL/d(point), zero for points outside the range) and
 * d_alpha (device, one float per draw path, may be NULL).  Enqueued on the
 * renderer's stream without synchronising. */
int32_t PFCUDABackward(PFCUDARendererRef renderer, const float* d_image, PFVector2F* d_points,
                       float* d_alpha);

/* ---- stroke to fill ----------------------------------------------------------
 * OutlineStrokeToFill (content/src/stroke.rs:24-190): each contour of an
 * outline is offset by half the line width on both sides, segment by segment,
 * with the stroke's joins between pieces and its caps at the ends of open
 * contours; a closed contour gives two closed contours, an open one gives one.
 * The result is an outline to fill with the nonzero rule, as the reference's
 * front-ends use it.  Runs on the GPU, with the reference's single-precision
 * op order: the same input gives the same output points. */
#define PF_LINE_CAP_BUTT    0
#define PF_LINE_CAP_SQUARE  1
#define PF_LINE_CAP_ROUND   2
#define PF_LINE_JOIN_MITER  0
#define PF_LINE_JOIN_BEVEL  1
#define PF_LINE_JOIN_ROUND  2

/* StrokeStyle (content/src/stroke.rs:45-56); miter_limit for PF_LINE_JOIN_MITER
 * (LineJoin::Miter(f32); the default style is width 1, butt, miter 10). */
typedef struct PFCUDAStrokeStyle {
    float   line_width;
    int32_t line_cap;      /* PF_LINE_CAP_*  */
    int32_t line_join;     /* PF_LINE_JOIN_* */
    float   miter_limit;
} PFCUDAStrokeStyle;

/* Outlines to stroke.  Contour c owns points [contour_starts[c],
 * contour_starts[c+1]) and is closed when contour_closed[c] != 0; outline o owns
 * contours [outline_starts[o], outline_starts[o+1]) and is stroked with
 * styles[o].  All arrays in `memory`. */
typedef struct PFCUDAStrokeInput {
    const PFVector2F* points;
    const uint8_t*    point_flags;      /* PF_POINT_FLAG_* bits */
    const uint32_t*   contour_starts;   /* contour_count + 1 */
    const uint8_t*    contour_closed;   /* contour_count */
    const uint32_t*   outline_starts;   /* outline_count + 1 */
    const PFCUDAStrokeStyle* styles;    /* outline_count */
    uint32_t point_count, contour_count, outline_count;
    int32_t  memory;                    /* PF_MEMORY_* */
} PFCUDAStrokeInput;

/* The stroked outlines: closed contours as flat buffers (in `memory`).  Input
 * contour c gives output contours in order (two for a closed contour, forward
 * then backward; one for an open one); outline_starts (outline_count + 1)
 * gives each outline's output contours.  point_count / contour_count are
 * written; with too little capacity the call returns PF_CUDA_ERR_CAPACITY,
 * writes the sizes needed and nothing else. */
typedef struct PFCUDAStrokeOutput {
    PFVector2F* points;
    uint8_t*    point_flags;
    uint32_t*   contour_starts;         /* contour_capacity + 1 */
    uint32_t*   outline_starts;         /* outline_count + 1 */
    uint64_t    point_capacity, contour_capacity;
    uint64_t    point_count, contour_count;
    int32_t     memory;
} PFCUDAStrokeOutput;

/* Synchronous on the renderer's stream. */
int32_t PFCUDAStrokeToFill(PFCUDARendererRef renderer, const PFCUDAStrokeInput* input, PFCUDAStrokeOutput* output);

/* ---- dashes: OutlineDash (content/src/dash.rs:18-152) ------------------------
 * Outline o is dashed with the pattern dashes[dash_starts[o] .. dash_starts[o+1])
 * (alternating "on" and "off" lengths, used as given: the canvas front-end's
 * doubling of an odd-length pattern, canvas/src/lib.rs:253-262, is the
 * caller's) and the phase offsets[o].  The reference's walk, op for op: the
 * offset is reduced modulo the pattern's sum and the whole dashes it covers
 * are skipped (DashState::new), then each segment of each contour (closing
 * segments included) is cut where the distance left in the current dash runs
 * out, distances being chord lengths (Segment::arc_length /
 * time_for_distance, content/src/segment.rs:246-254); the pieces of an "on"
 * dash form one open contour, which continues across the outline's contours.
 * An outline with an empty pattern is passed through unchanged (the
 * front-ends only dash a non-empty pattern, canvas/src/lib.rs:340,
 * svg/src/lib.rs:159).  A pattern must hold finite non-negative lengths with a
 * positive finite sum, and its offset must be finite (PF_CUDA_ERR_INVALID
 * otherwise).  An outline whose walk takes more than 2^20 steps (a cut or a
 * whole segment each) is cut short there and the call returns
 * PF_CUDA_ERR_LIMIT with the output complete up to that point.  One GPU thread
 * walks one outline: the distance left carries from segment to segment in
 * single precision, so the outlines are the parallel unit.  Arrays in the
 * stroke input's memory. */
typedef struct PFCUDADashInput {
    const float*    dashes;             /* dash_starts[outline_count] lengths */
    const uint32_t* dash_starts;        /* outline_count + 1 */
    const float*    offsets;            /* outline_count */
} PFCUDADashInput;

/* Outlines as flat buffers (in `memory`) with each contour's closed flag: the
 * layout of PFCUDAStrokeInput, so a dashed result can be stroked as it is.
 * Sizes and capacity as in PFCUDAStrokeOutput. */
typedef struct PFCUDAOutlineOutput {
    PFVector2F* points;
    uint8_t*    point_flags;
    uint32_t*   contour_starts;         /* contour_capacity + 1 */
    uint8_t*    contour_closed;         /* contour_capacity */
    uint32_t*   outline_starts;         /* outline_count + 1 */
    uint64_t    point_capacity, contour_capacity;
    uint64_t    point_count, contour_count;
    int32_t     memory;
} PFCUDAOutlineOutput;

/* OutlineDash::dash + into_outline for every outline of `input` (its styles
 * are not read and may be NULL).  Synchronous on the renderer's stream. */
int32_t PFCUDADashOutlines(PFCUDARendererRef renderer, const PFCUDAStrokeInput* input, const PFCUDADashInput* dash,
                           PFCUDAOutlineOutput* output);

/* The front-ends' stroke of a dashed outline (svg/src/lib.rs:159-167,
 * canvas/src/lib.rs:340-350): dashes, then OutlineStrokeToFill of the dashed
 * outlines with input->styles, both on the device with no copy between them.
 * Output as PFCUDAStrokeToFill's; PF_CUDA_ERR_LIMIT from either stage. */
int32_t PFCUDAStrokeToFillDashed(PFCUDARendererRef renderer, const PFCUDAStrokeInput* input,
                                 const PFCUDADashInput* dash, PFCUDAStrokeOutput* output);

/* Human-readable text for a status code (static storage). */
const char* PFCUDAStatusString(int32_t status);

/* ---- frames in flight (no reference counterpart in this form) --------------
 * The CUDA level's SceneProxy (renderer/src/concurrent/scene_proxy.rs:11-20,
 * :86-121 builds scenes on a worker thread and keeps a bounded number of
 * render commands in flight): `depth` renderers on one device, each with its
 * own stream, buffers and worker thread, render the submitted frames in
 * submission order, at most `depth` at once, so one frame's upload and image
 * copy overlap the other frames' kernels. */
typedef struct PFCUDAPipeline* PFCUDAPipelineRef;
int32_t PFCUDAPipelineCreate(int32_t device_ordinal, int32_t depth,
                             const PFCUDARendererOptions* options,
                             PFCUDAPipelineRef* out_pipeline);
/* Waits for every submitted frame, then frees the renderers and threads.  No
 * other call on the pipeline may be in progress or follow; statuses not yet
 * waited for are dropped. */
int32_t PFCUDAPipelineDestroy(PFCUDAPipelineRef pipeline);
/* Queues one frame: PFCUDASceneUpload of `scene` on the next free renderer,
 * then PFCUDARenderScene(options, width, height, out_rgba8, out_memory)
 * (options may be NULL: identity).  Returns at once with the frame's ticket
 * (1, 2, ...).  The scene's buffers, `out_rgba8` and `options` must stay
 * valid and unchanged until the frame is done.  For host outputs,
 * PF_MEMORY_HOST_COPY into page-locked memory keeps the SMs for the other
 * frames. */
int32_t PFCUDAPipelineSubmit(PFCUDAPipelineRef pipeline, const PFCUDASceneDesc* scene,
                             const PFCUDABuildOptions* options, int32_t width, int32_t height,
                             uint8_t* out_rgba8, int32_t out_memory, uint64_t* out_ticket);
/* *out_done = 1 when frame `ticket` is done (its status then waits for
 * PFCUDAPipelineWait), else 0.  PF_CUDA_ERR_INVALID for a ticket that was
 * never submitted or was already waited for. */
int32_t PFCUDAPipelinePoll(PFCUDAPipelineRef pipeline, uint64_t ticket, int32_t* out_done);
/* Waits for frame `ticket` and returns its status: the upload's or the
 * frame's error, else PF_CUDA_OK.  A ticket is waited for once;
 * PF_CUDA_ERR_INVALID for one never submitted or already waited for. */
int32_t PFCUDAPipelineWait(PFCUDAPipelineRef pipeline, uint64_t ticket);

#ifdef __cplusplus
}
#endif
#endif /* PATHFINDER_CUDA_H */

// pf_raster.cu — backdrop propagation, occlusion, visibility lists and the
// fused fill + composite of the CUDA level.
//
// Stage map (reference -> here):
//   Tiler::prepare_tiles (renderer/src/tiler.rs:93-163) and the D3D9 z-buffer
//   (renderer/src/builder.rs:1013-1029)                    -> k_propagate
//   per-screen-tile lists + sort (shaders/d3d11/sort.cs.glsl:60-95,
//   occlusion test of shaders/d3d9/tile.vs.glsl:51-55)      -> k_visible, k_composite (sort)
//   fill (shaders/d3d11/fill.cs.glsl:61-88, fill_area.inc.glsl:11-27),
//   clip combine (shaders/d3d9/tile_clip_combine.fs.glsl:27-30),
//   sampleMask + calculateColor + SrcOver
//   (shaders/tile_fragment.inc.glsl:539-613, shaders/d3d11/tile.cs.glsl:91-159)
//                                                            -> k_composite
//
// Device tile records use the PFCUDATile layout with one difference: the
// path field holds the global path index (the readback converts it to the
// index within the clip or draw paths).  Screen-tile arrays (z-buffer, list
// counts) are indexed from the first screen tile of the frame's scene range.
#include "pf_kernels.cuh"
#include "pathfinder_cuda.h"

#include <algorithm>
#include <atomic>

namespace pf {

__device__ __forceinline__ int4 pack_tile(int32_t tx, int32_t ty, uint32_t alpha, uint32_t gp, uint16_t color,
                                          uint8_t ctrl, int8_t backdrop) {
    int4 r;
    r.x = (int)(((uint32_t)(uint16_t)(int16_t)tx) | ((uint32_t)(uint16_t)(int16_t)ty << 16));
    r.y = (int)alpha;
    r.z = (int)gp;
    r.w = (int)((uint32_t)color | ((uint32_t)ctrl << 16) | ((uint32_t)(uint8_t)backdrop << 24));
    return r;
}
__device__ __forceinline__ int8_t tile_backdrop(int4 r) { return (int8_t)((uint32_t)r.w >> 24); }
__device__ __forceinline__ uint32_t tile_ctrl(int4 r) { return ((uint32_t)r.w >> 16) & 0xffu; }
__device__ __forceinline__ int32_t tile_x(int4 r) { return (int32_t)(int16_t)((uint32_t)r.x & 0xffffu); }
__device__ __forceinline__ int32_t tile_y(int4 r) { return (int32_t)(int16_t)((uint32_t)r.x >> 16); }

// A solid tile occludes only if it resolves to full coverage: for the
// nonzero rule any nonzero backdrop (the reference's test,
// renderer/src/builder.rs:1013-1029), for even-odd an odd backdrop.
__device__ __forceinline__ bool solid_occludes(int8_t b, bool even_odd) {
    if (b == 0) return false;
    return even_odd ? ((b & 1) != 0) : true;
}

__device__ __forceinline__ uint32_t upper_bound_u32(const uint32_t* a, uint32_t n, uint32_t v) {
    // first index i in [0, n) with a[i] > v
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (a[mid] <= v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Screen tile of (tx, ty) in its scene, relative to the frame; false outside.
__device__ __forceinline__ bool frame_screen_tile(const FrameDev& f, const SceneDev& sc, int32_t tx, int32_t ty,
                                                  uint32_t* st) {
    const int4 s = sc.screen;
    if (!(s.x <= tx && s.y <= ty && tx <= s.z - 1 && ty <= s.w - 1)) return false;
    *st = sc.screen_offset - f.screen_begin + (uint32_t)((ty - s.y) * (s.z - s.x) + (tx - s.x));
    return true;
}

// ---------------------------------------------------------------------------
// Column backdrops (Tiler::prepare_tiles's running backdrop down each column,
// renderer/src/tiler.rs:93-111): the backdrop of tile (ox, oy) is the column's
// above-rect sum plus the deltas of the tiles above it (wrapping int32 sums).
// A thread walks one column of one path top to bottom; the lanes of a warp
// take neighbouring columns, so every read and write of a row is coalesced
// (the deltas and the tiles are row-major within a path).
// ---------------------------------------------------------------------------
__global__ void k_column_backdrops(FrameDev f) {
    pdl_enter();
    if (!frame_ok(f) || f.path_count == 0) return;
    const uint32_t NC = (uint32_t)f.counters->columns;
    const uint32_t* coffs = f.path.col_offset + f.path_begin;
    const int32_t* __restrict__ delta = f.tile_delta;
    uint32_t* __restrict__ out = f.tile_delta_scan;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < NC; c += gridDim.x * blockDim.x) {
        const uint32_t gp = f.path_begin + upper_bound_u32(coffs, f.path_count + 1, c) - 1;
        const int4 r = f.path.tile_rect[gp];
        const uint32_t w = (uint32_t)(r.z - r.x), h = (uint32_t)(r.w - r.y);
        uint32_t g = f.path.tile_offset[gp] + (c - f.path.col_offset[gp]);
        uint32_t acc = (uint32_t)f.col_backdrop[c];
        uint32_t oy = 0;
        for (; oy + 4 <= h; oy += 4, g += 4 * w) {  // four rows' reads in flight at once
            const uint32_t d0 = (uint32_t)delta[g], d1 = (uint32_t)delta[g + w];
            const uint32_t d2 = (uint32_t)delta[g + 2 * w], d3 = (uint32_t)delta[g + 3 * w];
            out[g] = acc;
            out[g + w] = acc + d0;
            out[g + 2 * w] = acc + d0 + d1;
            out[g + 3 * w] = acc + d0 + d1 + d2;
            acc += d0 + d1 + d2 + d3;
        }
        for (; oy < h; oy++, g += w) {
            const uint32_t d = (uint32_t)delta[g];
            out[g] = acc;
            acc += d;
        }
    }
}

void launch_column_backdrops(const FrameDev& f, cudaStream_t s) {
    if (f.path_count == 0) return;
    count_launch();
    pdl_launch(k_column_backdrops, f.sms * 16, 256, 0, s, f);
}

// ---------------------------------------------------------------------------
// propagate: one thread per tile; clip tiles in the first launch, draw tiles
// in the second (draw tiles of clipped paths read their clip's final tiles).
// Path sizes are log-normal, so per-path work items would leave a long tail.
// ---------------------------------------------------------------------------
__global__ void k_propagate(FrameDev f, int clip_pass) {
    pdl_enter();
    if (!frame_ok(f) || f.path_count == 0) return;
    const uint32_t T = (uint32_t)f.counters->tiles;
    const uint32_t* offs = f.path.tile_offset + f.path_begin;
    // A one-scene frame has its clip paths' tiles first: each pass visits only
    // its own tiles and searches only its own paths.
    uint32_t g_begin = 0, g_end = T, p_lo = 0, p_n = f.path_count + 1;
    if (f.scene_count == 1) {
        const uint32_t nclip = f.scenes[f.scene_begin].clip_count;
        if (clip_pass) { g_end = offs[nclip]; p_n = nclip + 1; }
        else { g_begin = offs[nclip]; p_lo = nclip; p_n = f.path_count + 1 - nclip; }
    }
    for (uint32_t g = g_begin + blockIdx.x * blockDim.x + threadIdx.x; g < g_end; g += gridDim.x * blockDim.x) {
        const uint32_t gp = f.path_begin + p_lo + upper_bound_u32(offs + p_lo, p_n, g) - 1;
        const bool is_clip = f.path.is_clip[gp] != 0;
        if (is_clip != (clip_pass != 0)) continue;
        const int4 r = f.path.tile_rect[gp];
        const int32_t w = r.z - r.x, h = r.w - r.y;
        const uint32_t tbase = f.path.tile_offset[gp];
        const bool even_odd = f.path.rule[gp] == 1;
        const uint8_t ctrl = is_clip ? 0 : (even_odd ? 0x2 : 0x1);
        const uint32_t local = f.path.local_index[gp];
        const uint16_t color = is_clip ? 0 : (uint16_t)(local & 0xffffu);
        const int32_t clip_gp = is_clip ? -1 : f.path.clip_gpath[gp];

        const uint32_t i = g - tbase;
        const int32_t ox = (int32_t)(i % (uint32_t)w), oy = (int32_t)(i / (uint32_t)w);
        const int32_t acc = (int32_t)f.tile_delta_scan[g];  // the column backdrop (k_column_backdrops)
        const bool has_fill = f.tile_fill_base[g + 1] > f.tile_fill_base[g];
        const uint32_t own_alpha = has_fill ? f.tile_alpha[g] : kInvalid;
        if (has_fill) f.alpha_owner[own_alpha] = g;
        uint32_t alpha = own_alpha;
        int8_t backdrop = (int8_t)acc;
        const int32_t tx = r.x + ox, ty = r.y + oy;
        uint8_t tile_ctrl_bits = ctrl;
        if (clip_gp >= 0 && f.path.clip_gpath[clip_gp] >= 0) {
            // Clip chain: the tile stays as built unless a clip level lacks a
            // tile here or has an empty one (the composite takes the minimum
            // over the chain).  Clip paths keep their own records, so every
            // level is final after the clip pass.
            tile_ctrl_bits = (uint8_t)(ctrl | kCtrlClipChain);
            bool culled = false;
            int32_t q = clip_gp;
            for (uint32_t it = 0; q >= 0 && it <= f.clip_chain_max; it++) {
                const int4 cr = f.path.tile_rect[q];
                if (!(cr.x <= tx && cr.y <= ty && tx <= cr.z - 1 && ty <= cr.w - 1)) { culled = true; break; }
                const int4 ct = f.tiles[f.path.tile_offset[q] + (uint32_t)((ty - cr.y) * (cr.z - cr.x) + (tx - cr.x))];
                if ((uint32_t)ct.y == kInvalid && tile_backdrop(ct) == 0) { culled = true; break; }
                q = f.path.clip_gpath[q];
            }
            if (culled) { alpha = kInvalid; backdrop = 0; }
            f.clips[g] = make_int4((int)kInvalid, 0, (int)kInvalid, 0);
        } else if (clip_gp >= 0) {
            const int4 cr = f.path.tile_rect[clip_gp];
            int4 clip_rec = make_int4((int)kInvalid, 0, (int)kInvalid, 0);
            if (cr.x <= tx && cr.y <= ty && tx <= cr.z - 1 && ty <= cr.w - 1) {
                const uint32_t cg = f.path.tile_offset[clip_gp] + (uint32_t)((ty - cr.y) * (cr.z - cr.x) + (tx - cr.x));
                const int4 ct = f.tiles[cg];
                const uint32_t calpha = (uint32_t)ct.y;
                const int8_t cb = tile_backdrop(ct);
                if (calpha != kInvalid && alpha != kInvalid) {
                    clip_rec = make_int4((int)alpha, (int)backdrop, (int)calpha, (int)cb);
                    backdrop = 0;
                } else if (calpha != kInvalid && alpha == kInvalid && backdrop != 0) {
                    alpha = calpha;
                    backdrop = cb;
                } else if (calpha == kInvalid && cb == 0) {
                    alpha = kInvalid;
                    backdrop = 0;
                }
            } else {
                alpha = kInvalid;
                backdrop = 0;
            }
            f.clips[g] = clip_rec;
        }  // tiles of unclipped paths get no clip record: every reader checks the path's clip first
        f.tiles[g] = pack_tile(tx, ty, alpha, gp, color, tile_ctrl_bits, backdrop);
        // differentiable frames occlude with the FP32 paint alpha being optimised;
        // a tile behind a clip chain may be partly covered, so it never occludes
        const bool opaque = (is_clip || (tile_ctrl_bits & kCtrlClipChain)) ? false
                                    : (f.path.alpha_f ? f.path.alpha_f[f.path.draw_index[gp]] >= 1.0f
                                                      : f.path.occludes[gp] != 0);
        if (opaque && alpha == kInvalid && solid_occludes(backdrop, even_odd)) {
            uint32_t st;
            if (frame_screen_tile(f, f.scenes[f.path.scene[gp]], tx, ty, &st)) atomicMax(&f.zbuf[st], (int32_t)local);
        }
    }
}

void launch_propagate(const FrameDev& f, bool clip_pass, cudaStream_t s) {
    if (f.path_count == 0) return;
    { count_launch(); pdl_launch(k_propagate, f.sms * 16, 256, 0, s, f, clip_pass ? 1 : 0); }
}

// ---------------------------------------------------------------------------
// visibility: count per screen tile, then scatter global tile indices
// ---------------------------------------------------------------------------
__global__ void k_visible(FrameDev f, int scatter) {
    pdl_enter();
    if (scatter && blockIdx.x == 0 && threadIdx.x == 0 && f.counters->visible > f.vis_cap) {
        atomicOr(&f.counters->status, kStatusVisibleCapacity);  // the visibility scan's total
        f.counters->needed_visible = f.counters->visible;
    }
    uint64_t T = f.counters->tiles;
    if (!frame_ok(f)) return;
    if (scatter && f.counters->visible > f.vis_cap) return;
    for (uint64_t gi = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; gi < T; gi += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t g = (uint32_t)gi;
        int4 rec = f.tiles[g];
        if (tile_ctrl(rec) == 0) continue;                                  // clip path tile
        if ((uint32_t)rec.y == kInvalid && tile_backdrop(rec) == 0) continue;  // empty (builder.rs:1016-1018)
        const uint32_t gp = (uint32_t)rec.z;
        uint32_t st;
        if (!frame_screen_tile(f, f.scenes[f.path.scene[gp]], tile_x(rec), tile_y(rec), &st)) continue;
        if ((int32_t)f.path.local_index[gp] < f.zbuf[st]) continue;  // occluded (tile.vs.glsl:51-55)
        if (!scatter) {
            atomicAdd(&f.screen_cnt[st], 1u);
        } else {
            uint32_t slot = f.screen_base[st] + atomicSub(&f.screen_cnt[st], 1u) - 1u;
            if (slot < f.vis_cap) {
                f.vis[slot] = g;
                f.vis_key[slot] = ((unsigned long long)g << 32) | slot;
                uint32_t kind = (uint32_t)rec.y == kInvalid ? kVisSolid : kVisMask;
                if (tile_ctrl(rec) & kCtrlClipChain) kind = kVisChain;
                else if (kind == kVisMask && f.path.clip_gpath[gp] >= 0) {
                    const int4 crec = f.clips[g];
                    if ((uint32_t)crec.x != kInvalid && (uint32_t)crec.z != kInvalid) kind = kVisCombine;
                }
                uint32_t b0 = 0, nf = 0;
                if (kind == kVisMask) {
                    const uint32_t owner = f.alpha_owner[(uint32_t)rec.y];
                    b0 = f.tile_fill_base[owner];
                    nf = f.tile_fill_base[owner + 1] - b0;
                }
                const int32_t meta = vis_meta(tile_backdrop(rec), (tile_ctrl(rec) & 0x2u) != 0, kind,
                                              f.paint_effects ? paint_fx_bits(f.path.blend[gp], f.path.overlay[gp])
                                                              : 0u);
                f.vis_info[slot] = make_int4((int)b0, (int)nf, (int)f.path.paint[gp], meta);
                if (kind != kVisSolid) {
                    // the mask kernel's work list, one slot reservation per warp
                    const uint32_t m = __activemask();
                    const int leader = __ffs(m) - 1, lane = threadIdx.x & 31;
                    uint32_t at = 0;
                    if (lane == leader) at = atomicAdd(&f.counters->mask_items, (uint32_t)__popc(m));
                    at = __shfl_sync(m, at, leader) + (uint32_t)__popc(m & ((1u << lane) - 1u));
                    if (at < f.vis_cap) f.mask_items[at] = make_int4((int)b0, (int)nf, meta, (int)slot);
                }
            }
        }
    }
}

void launch_visible(const FrameDev& f, bool scatter, cudaStream_t s) {
    { count_launch(); pdl_launch(k_visible, f.sms * 8, 256, 0, s, f, scatter ? 1 : 0); }
}

// ---------------------------------------------------------------------------
// warp-level building blocks
// ---------------------------------------------------------------------------
// Bitonic network in its "all comparators ascending" form: for block size k
// the first step compares i with i ^ (k - 1), later steps i with i ^ j.  Slots
// at or beyond n act as +inf and are never touched, so n need not be a power
// of two.  One warp; `a` in shared or global memory.
template <typename K>
__device__ void warp_bitonic_sort(K* a, uint32_t n) {
    const int lane = threadIdx.x & 31;
    uint32_t N = 1;
    while (N < n) N <<= 1;
    for (uint32_t k = 2; k <= N; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = lane; i < N; i += 32) {
                uint32_t l = (j == (k >> 1)) ? (i ^ (k - 1)) : (i ^ j);
                if (l > i && l < n) {
                    K x = a[i], y = a[l];
                    if (y < x) { a[i] = y; a[l] = x; }
                }
            }
            __syncwarp();
        }
    }
}

// Ascending bitonic sort of one key per lane over lanes [0, N), N a power of
// two no larger than 32; lanes past the list hold the largest key.  Shuffles
// only: no shared memory and no warp barriers.
__device__ __forceinline__ unsigned long long warp_sort_lanes(unsigned long long v, uint32_t N) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t k = 2; k <= N; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            const unsigned long long o = __shfl_xor_sync(0xffffffffu, v, j);
            const bool ascending = (lane & k) == 0, low = (lane & j) == 0;
            v = (ascending == low) ? (o < v ? o : v) : (o > v ? o : v);
        }
    }
    return v;
}

struct __align__(16) CovBuf { int acc[256]; int carry[256]; };  // cleared with int4 stores

// Accumulate `count` fills into `buf` (one warp); fetch(i, x0, y0, x1, y1)
// gives fill i in tile pixels.
template <class Fetch>
__device__ __forceinline__ void warp_accumulate(uint32_t count, Fetch&& fetch, CovBuf& buf) {
    const int lane = threadIdx.x & 31;
    int4* z = reinterpret_cast<int4*>(&buf);  // acc and carry: 512 ints
#pragma unroll
    for (int k = 0; k < 4; k++) z[lane + 32 * k] = make_int4(0, 0, 0, 0);
    __syncwarp();
    // Work items are (fill, pixel column) pairs, spread over the lanes: a
    // warp scan of the column counts of 32 fills, then each lane finds the
    // fill of its item with a 5-step search over the scanned counts.
    for (uint32_t base = 0; base < count; base += 32) {
        const uint32_t i = base + lane;
        float x0 = 0.0f, y0 = 0.0f, x1 = 0.0f, slope = 0.0f;
        int c0 = 0, ncol = 0;
        if (i < count) {
            float y1;
            fetch(i, x0, y0, x1, y1);
            if (x0 != x1) {
                slope = __fdividef(y1 - y0, x1 - x0);
                c0 = max((int)floorf(fminf(x0, x1)), 0);
                const int c1 = min((int)ceilf(fmaxf(x0, x1)) - 1, 15);
                ncol = max(c1 - c0 + 1, 0);
            }
        }
        int incl = ncol;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        for (int k0 = 0; k0 < total; k0 += 32) {
            const int k = k0 + lane;
            int j = 0;  // owner: the first lane whose inclusive count exceeds k
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const int v = __shfl_sync(0xffffffffu, incl, j + step - 1);
                if (v <= k) j += step;
            }
            const float ox0 = __shfl_sync(0xffffffffu, x0, j), oy0 = __shfl_sync(0xffffffffu, y0, j);
            const float ox1 = __shfl_sync(0xffffffffu, x1, j), osl = __shfl_sync(0xffffffffu, slope, j);
            const int oc0 = __shfl_sync(0xffffffffu, c0, j);
            const int oex = __shfl_sync(0xffffffffu, incl - ncol, j);
            if (k < total) accumulate_fill_column(ox0, oy0, ox1, osl, oc0 + (k - oex), buf.acc, buf.carry);
        }
    }
    __syncwarp();
}

// `count` packed LineSegmentU16 fills at `src` (global or shared memory).
__device__ __forceinline__ void warp_accumulate_packed(const uint2* src, uint32_t count, CovBuf& buf) {
    warp_accumulate(count, [&](uint32_t i, float& x0, float& y0, float& x1, float& y1) {
        const uint2 rec = src[i];
        x0 = (float)(rec.x & 0xffffu) * (1.0f / 256.0f); y0 = (float)(rec.x >> 16) * (1.0f / 256.0f);
        x1 = (float)(rec.y & 0xffffu) * (1.0f / 256.0f); y1 = (float)(rec.y >> 16) * (1.0f / 256.0f);
    }, buf);
}

// Fills [b0, b1) (one alpha tile's).  DIFF reads the FP32 fills of
// differentiable frames.
template <bool DIFF = false>
__device__ __forceinline__ void warp_accumulate_fills(const FrameDev& f, uint32_t b0, uint32_t b1, CovBuf& buf) {
    if constexpr (DIFF) {
        warp_accumulate(b1 - b0, [&](uint32_t i, float& x0, float& y0, float& x1, float& y1) {
            const float4 rec = f.fills_f[b0 + i];
            x0 = rec.x; y0 = rec.y; x1 = rec.z; y1 = rec.w;
        }, buf);
    } else {
        warp_accumulate_packed(f.fills + b0, b1 - b0, buf);
    }
}

// The same for alpha tile `alpha`, its fill range found through its owner.
template <bool DIFF = false>
__device__ __forceinline__ void warp_accumulate_tile(const FrameDev& f, uint32_t alpha, CovBuf& buf) {
    const uint32_t owner = f.alpha_owner[alpha];
    warp_accumulate_fills<DIFF>(f, f.tile_fill_base[owner], f.tile_fill_base[owner + 1], buf);
}

// Lane (col = lane & 15, half = lane >> 4) owns rows half*8 .. half*8+7 of
// column col.  Returns the accumulated coverage of those 8 pixels (fixed
// point): acc + the carry prefix down the column.
__device__ __forceinline__ void warp_column_values(const CovBuf& buf, int out[8]) {
    const int lane = threadIdx.x & 31, col = lane & 15, half = lane >> 4;
    int run = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        int r = half * 8 + k;
        run += buf.carry[r * 16 + col];
        out[k] = buf.acc[r * 16 + col] + run;
    }
    int top = __shfl_sync(0xffffffffu, run, col);  // rows 0..7 total of this column
    if (half) {
#pragma unroll
        for (int k = 0; k < 8; k++) out[k] += top;
    }
}

constexpr uint32_t kWarpListCap = 128;
struct WarpScratch { uint32_t keys[kWarpListCap]; CovBuf b0, b1; };

// Per-pixel coverage of one path tile for this lane's 8 pixels.
// |mask + backdrop| of one tile for this lane's 8 pixels (the backdrop alone
// for a solid tile).
__device__ __forceinline__ void tile_abs_winding8(const FrameDev& f, int4 rec, CovBuf& b, float m[8]) {
    const float bd = (float)tile_backdrop(rec);
    if ((uint32_t)rec.y != kInvalid) {
        int v[8];
        warp_accumulate_tile(f, (uint32_t)rec.y, b);
        warp_column_values(b, v);
        __syncwarp();  // the buffer is cleared by the next accumulation
#pragma unroll
        for (int k = 0; k < 8; k++) m[k] = fabsf((float)v[k] * kCovInvScale + bd);
    } else {
#pragma unroll
        for (int k = 0; k < 8; k++) m[k] = fabsf(bd);
    }
}

// Coverage of a tile behind a clip chain: the fill rule applied to the
// minimum of |mask + backdrop| over the tile and each clip level's tile at the
// same coordinates (all present: the propagation culled the tile otherwise).
__device__ __forceinline__ void chain_coverage8(const FrameDev& f, int4 rec, CovBuf& b, float cov[8]) {
    float m[8], mq[8];
    tile_abs_winding8(f, rec, b, m);
    const int32_t tx = tile_x(rec), ty = tile_y(rec);
    int32_t q = f.path.clip_gpath[(uint32_t)rec.z];
    for (uint32_t it = 0; q >= 0 && it <= f.clip_chain_max; it++) {
        const int4 cr = f.path.tile_rect[q];
        if (!(cr.x <= tx && cr.y <= ty && tx <= cr.z - 1 && ty <= cr.w - 1)) break;  // culled by propagation
        const int4 ct = f.tiles[f.path.tile_offset[q] + (uint32_t)((ty - cr.y) * (cr.z - cr.x) + (tx - cr.x))];
        tile_abs_winding8(f, ct, b, mq);
#pragma unroll
        for (int k = 0; k < 8; k++) m[k] = fminf(m[k], mq[k]);
        q = f.path.clip_gpath[q];
    }
    const bool even_odd = (tile_ctrl(rec) & 0x2u) != 0;
#pragma unroll
    for (int k = 0; k < 8; k++) cov[k] = resolve_coverage(m[k], even_odd);
}

__device__ __forceinline__ void tile_coverage8(const FrameDev& f, int4 rec, uint32_t g, CovBuf& b0, CovBuf& b1,
                                               float cov[8]) {
    const uint32_t gp = (uint32_t)rec.z;
    if (tile_ctrl(rec) & kCtrlClipChain) {
        chain_coverage8(f, rec, b0, cov);
        return;
    }
    const bool even_odd = (tile_ctrl(rec) & 0x2u) != 0;
    const float bd = (float)tile_backdrop(rec);
    bool combine = false;
    int4 crec = make_int4(0, 0, 0, 0);
    if (tile_ctrl(rec) != 0 && f.path.clip_gpath[gp] >= 0) {  // draw tiles only carry clip records
        crec = f.clips[g];
        combine = (uint32_t)crec.x != kInvalid && (uint32_t)crec.z != kInvalid;
    }
    if (combine) {
        // tile_clip_combine.fs.glsl:27-30, then sampleMask with the zeroed backdrop
        int vd[8], vs[8];
        warp_accumulate_tile(f, (uint32_t)crec.x, b0);
        warp_accumulate_tile(f, (uint32_t)crec.z, b1);
        warp_column_values(b0, vd);
        warp_column_values(b1, vs);
#pragma unroll
        for (int k = 0; k < 8; k++) {
            float m = fminf(fabsf((float)vd[k] * kCovInvScale + (float)crec.y),
                            fabsf((float)vs[k] * kCovInvScale + (float)crec.w));
            cov[k] = resolve_coverage(m + bd, even_odd);
        }
    } else if ((uint32_t)rec.y != kInvalid) {
        int v[8];
        warp_accumulate_tile(f, (uint32_t)rec.y, b0);
        warp_column_values(b0, v);
#pragma unroll
        for (int k = 0; k < 8; k++) cov[k] = resolve_coverage((float)v[k] * kCovInvScale + bd, even_odd);
    } else {
        float c = resolve_coverage(bd, even_odd);
#pragma unroll
        for (int k = 0; k < 8; k++) cov[k] = c;
    }
    __syncwarp();  // buffers are reused by the next tile
}

// ---------------------------------------------------------------------------
// paint effects: gradient colour (tile_fragment.inc.glsl:75-90, 274-307,
// 560-613) and blend modes (renderer/src/gpu/blend.rs:42-160 for the
// Porter-Duff modes, the shader's composite(), tile_fragment.inc.glsl:414-537,
// for the others).  Solid SrcOver tiles never come here.
// ---------------------------------------------------------------------------
// The colour texture transform of a gradient for this frame: the gradient's
// map composed with the inverse build transform (`transform *=
// render_transform`, renderer/src/paint.rs:637; Transform2F * Transform2F,
// geometry/src/transform2d.rs:115-121, 301-310) and rounded to binary16 as the
// metadata texture stores it (renderer/src/gpu/renderer.rs:711-719).
__device__ __forceinline__ void gradient_frame_transform(const FrameDev& f, const OverlayDev& gd, float t[6]) {
    const float* G = gd.g;
    const float* R = f.inv_m;
    t[0] = round_f16(fadd(fmul(G[0], R[0]), fmul(G[1], R[3])));
    t[1] = round_f16(fadd(fmul(G[0], R[1]), fmul(G[1], R[4])));
    t[2] = round_f16(fadd(fadd(fmul(G[0], R[2]), fmul(G[1], R[5])), G[2]));
    t[3] = round_f16(fadd(fmul(G[3], R[0]), fmul(G[4], R[3])));
    t[4] = round_f16(fadd(fmul(G[3], R[1]), fmul(G[4], R[4])));
    t[5] = round_f16(fadd(fadd(fmul(G[3], R[2]), fmul(G[4], R[5])), G[5]));
}

__device__ __forceinline__ float4 unpack_unorm8(uint32_t v) {
    const float s = 1.0f / 255.0f;
    return make_float4((float)(v & 0xffu) * s, (float)((v >> 8) & 0xffu) * s, (float)((v >> 16) & 0xffu) * s,
                       (float)(v >> 24) * s);
}

// Linear filtering of the 256-texel ramp at texture coordinate u, clamped to
// the edge texels or repeated (TextureSamplingFlags::REPEAT_U,
// renderer/src/paint.rs:469-474).  A NaN coordinate (the reference leaves it
// to the sampler) gives transparent black.
__device__ __forceinline__ float4 ramp_sample(const uint32_t* ramp, float u, int32_t wrap) {
    if (wrap == PF_GRADIENT_WRAP_REPEAT) u = u - floorf(u);
    if (!(u == u)) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    u = fminf(fmaxf(u, -1.0f), 2.0f);
    const float x = u * 256.0f - 0.5f;
    const float x0 = floorf(x), w1 = x - x0;
    int i0 = (int)x0, i1 = i0 + 1;
    if (wrap == PF_GRADIENT_WRAP_REPEAT) { i0 &= 255; i1 &= 255; }
    else { i0 = min(max(i0, 0), 255); i1 = min(max(i1, 0), 255); }
    const float4 c0 = unpack_unorm8(__ldg(ramp + i0)), c1 = unpack_unorm8(__ldg(ramp + i1));
    const float w0 = 1.0f - w1;
    return make_float4(c0.x * w0 + c1.x * w1, c0.y * w0 + c1.y * w1, c0.z * w0 + c1.z * w1,
                       c0.w * w0 + c1.w * w1);
}

// Separable blend functions (compositeRGB, tile_fragment.inc.glsl:420-517),
// one channel: d destination, s source.
__device__ __forceinline__ float blend_screen(float d, float s) { return d + s - d * s; }
__device__ __forceinline__ float blend_hard_light(float d, float s) {
    return s <= 0.5f ? d * 2.0f * s : blend_screen(d, 2.0f * s - 1.0f);
}
__device__ __forceinline__ float blend_color_dodge(float d, float s) {
    return d == 0.0f ? 0.0f : (s == 1.0f ? 1.0f : d / (1.0f - s));
}
__device__ __forceinline__ float blend_separable(uint32_t mode, float d, float s) {
    switch (mode) {
    case PF_BLEND_MODE_MULTIPLY: return d * s;
    case PF_BLEND_MODE_SCREEN: return blend_screen(d, s);
    case PF_BLEND_MODE_OVERLAY: return blend_hard_light(s, d);
    case PF_BLEND_MODE_DARKEN: return fminf(d, s);
    case PF_BLEND_MODE_LIGHTEN: return fmaxf(d, s);
    case PF_BLEND_MODE_COLOR_DODGE: return blend_color_dodge(d, s);
    case PF_BLEND_MODE_COLOR_BURN: return 1.0f - blend_color_dodge(1.0f - d, 1.0f - s);
    case PF_BLEND_MODE_HARD_LIGHT: return blend_hard_light(d, s);
    case PF_BLEND_MODE_SOFT_LIGHT: {
        const float dark = d <= 0.25f ? ((16.0f * d - 12.0f) * d + 4.0f) * d : sqrtf(d);
        const float factor = s <= 0.5f ? d * (1.0f - d) : dark - d;
        return d + (s * 2.0f - 1.0f) * factor;
    }
    case PF_BLEND_MODE_DIFFERENCE: return fabsf(d - s);
    default: return d + s - 2.0f * d * s;  // Exclusion
    }
}

__device__ __forceinline__ float blend_divide(float n, float d) { return d != 0.0f ? n / d : 0.0f; }

// compositeRGBToHSL / compositeHSLToRGB (tile_fragment.inc.glsl:431-448): the
// reference's own HSL variant (saturation c / v), restated as written.
__device__ __forceinline__ float3 blend_rgb_to_hsl(float r, float g, float b) {
    const float v = fmaxf(fmaxf(r, g), b), lo = fminf(fminf(r, g), b);
    const float c = v - lo, l = lo + (v - lo) * 0.5f;
    float tx, ty, tz;
    if (r == v) { tx = 0.0f; ty = g; tz = b; }
    else if (g == v) { tx = 2.0f; ty = b; tz = r; }
    else { tx = 4.0f; ty = r; tz = g; }
    const float h = 1.0471975511965976f * blend_divide(tx * c + ty - tz, c);
    return make_float3(h, blend_divide(c, v), l);
}
__device__ __forceinline__ float blend_hsl_channel(float k0, float h, float s, float l) {
    const float a = s * fminf(l, 1.0f - l);
    float k = k0 + h * 1.9098593171027443f;
    k = k - 12.0f * floorf(k * (1.0f / 12.0f));  // GLSL mod(k, 12)
    return l - fminf(fmaxf(fminf(k - 3.0f, 9.0f - k), -1.0f), 1.0f) * a;
}

// One pixel: straight source colour (sr, sg, sb), source alpha a (paint alpha
// x coverage), premultiplied destination d.  The framebuffer is UNORM, so
// every result is clamped to [0, 1].
__device__ __forceinline__ void blend_pixel(uint32_t mode, float sr, float sg, float sb, float a, float& d0,
                                            float& d1, float& d2, float& d3) {
    const float da = d3;
    if (mode <= PF_BLEND_MODE_LIGHTER) {
        float fs, fd;  // source and destination factors (blend.rs:42-144; Copy: no blending)
        switch (mode) {
        case PF_BLEND_MODE_CLEAR: fs = 0.0f; fd = 0.0f; break;
        case PF_BLEND_MODE_COPY: fs = 1.0f; fd = 0.0f; break;
        case PF_BLEND_MODE_SRC_IN: fs = da; fd = 0.0f; break;
        case PF_BLEND_MODE_SRC_OUT: fs = 1.0f - da; fd = 0.0f; break;
        case PF_BLEND_MODE_SRC_ATOP: fs = da; fd = 1.0f - a; break;
        case PF_BLEND_MODE_DEST_IN: fs = 0.0f; fd = a; break;
        case PF_BLEND_MODE_DEST_OUT: fs = 0.0f; fd = 1.0f - a; break;
        case PF_BLEND_MODE_DEST_OVER: fs = 1.0f - da; fd = 1.0f; break;
        case PF_BLEND_MODE_DEST_ATOP: fs = 1.0f - da; fd = a; break;
        case PF_BLEND_MODE_XOR: fs = 1.0f - da; fd = 1.0f - a; break;
        case PF_BLEND_MODE_LIGHTER: fs = 1.0f; fd = 1.0f; break;
        default: fs = 1.0f; fd = 1.0f - a; break;  // SrcOver
        }
        d0 = __saturatef(sr * a * fs + d0 * fd);
        d1 = __saturatef(sg * a * fs + d1 * fd);
        d2 = __saturatef(sb * a * fs + d2 * fd);
        d3 = __saturatef(a * fs + da * fd);
        return;
    }
    // composite() reads the destination from a copy of the RGBA8 framebuffer
    // (copy_alpha_tiles_to_dest_blend_texture, renderer/src/gpu/d3d9/
    // renderer.rs:405-407): the destination it sees is quantised to 8 bits.
    d0 = rintf(__saturatef(d0) * 255.0f) * (1.0f / 255.0f);
    d1 = rintf(__saturatef(d1) * 255.0f) * (1.0f / 255.0f);
    d2 = rintf(__saturatef(d2) * 255.0f) * (1.0f / 255.0f);
    const float dq = rintf(__saturatef(da) * 255.0f) * (1.0f / 255.0f);
    float b0, b1, b2;
    if (mode >= PF_BLEND_MODE_HUE) {
        const float3 dh = blend_rgb_to_hsl(d0, d1, d2), sh = blend_rgb_to_hsl(sr, sg, sb);
        float h = dh.x, s = dh.y, l = dh.z;  // compositeHSL (tile_fragment.inc.glsl:471-482)
        if (mode == PF_BLEND_MODE_HUE) h = sh.x;
        else if (mode == PF_BLEND_MODE_SATURATION) s = sh.y;
        else if (mode == PF_BLEND_MODE_COLOR) { h = sh.x; s = sh.y; }
        else l = sh.z;
        b0 = blend_hsl_channel(0.0f, h, s, l);
        b1 = blend_hsl_channel(8.0f, h, s, l);
        b2 = blend_hsl_channel(4.0f, h, s, l);
    } else {
        b0 = blend_separable(mode, d0, sr);
        b1 = blend_separable(mode, d1, sg);
        b2 = blend_separable(mode, d2, sb);
    }
    // composite() (tile_fragment.inc.glsl:519-537): output alpha 1
    const float ws = a * (1.0f - dq), wb = a * dq, wd = 1.0f - a;
    d0 = __saturatef(ws * sr + wb * b0 + wd * d0);
    d1 = __saturatef(ws * sg + wb * b1 + wd * d1);
    d2 = __saturatef(ws * sb + wb * b2 + wd * d2);
    d3 = 1.0f;
}

// One sample of a pattern's texture page at UV (u, v): linear filtering or the
// nearest texel (NEAREST_MIN | NEAREST_MAG, renderer/src/paint.rs:545-548),
// each axis repeated or clamped to the edge (REPEAT_U / REPEAT_V, :537-543);
// the non-repeating axes' edges are the page's transparent border.  A NaN
// coordinate gives transparent black.
__device__ __forceinline__ float4 page_sample(const uint32_t* tex, int W, int H, uint32_t flags, float u, float v) {
    const bool rx = (flags & PF_PATTERN_REPEAT_X) != 0, ry = (flags & PF_PATTERN_REPEAT_Y) != 0;
    if (rx) u = u - floorf(u);
    if (ry) v = v - floorf(v);
    if (!(u == u) || !(v == v)) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    u = fminf(fmaxf(u, -1.0f), 2.0f);
    v = fminf(fmaxf(v, -1.0f), 2.0f);
    // after the wrap above, repeated indices lie in [-1, size]: one correction suffices
    auto wrap_x = [&](int i) { return rx ? (i < 0 ? i + W : (i >= W ? i - W : i)) : min(max(i, 0), W - 1); };
    auto wrap_y = [&](int i) { return ry ? (i < 0 ? i + H : (i >= H ? i - H : i)) : min(max(i, 0), H - 1); };
    if (flags & PF_PATTERN_NO_SMOOTHING)
        return unpack_unorm8(__ldg(tex + wrap_y((int)floorf(v * (float)H)) * W + wrap_x((int)floorf(u * (float)W))));
    const float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    const float x0 = floorf(x), y0 = floorf(y), wx = x - x0, wy = y - y0;
    const int ix0 = wrap_x((int)x0), ix1 = wrap_x((int)x0 + 1), iy0 = wrap_y((int)y0), iy1 = wrap_y((int)y0 + 1);
    const float4 c00 = unpack_unorm8(__ldg(tex + iy0 * W + ix0)), c10 = unpack_unorm8(__ldg(tex + iy0 * W + ix1));
    const float4 c01 = unpack_unorm8(__ldg(tex + iy1 * W + ix0)), c11 = unpack_unorm8(__ldg(tex + iy1 * W + ix1));
    auto lerp4 = [](float4 a, float4 b, float t) {
        return make_float4(a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t, a.z + (b.z - a.z) * t, a.w + (b.w - a.w) * t);
    };
    return lerp4(lerp4(c00, c10, wx), lerp4(c01, c11, wx), wy);
}

// A pattern's colour at UV (u, v) through its filter: filterNone, filterBlur
// (shaders/tile_fragment.inc.glsl:309-347, the incremental Gaussian with two
// taps per linear fetch) or filterColorMatrix (:349-359).
__device__ __noinline__ float4 pattern_color(const OverlayDev& od, const uint32_t* tex, float u, float v) {
    const int W = (int)od.page_w, H = (int)od.page_h;
    if (od.filter == PF_PATTERN_FILTER_COLOR_MATRIX) {
        const float4 c = page_sample(tex, W, H, od.flags, u, v);
        const float* m = od.matrix;
        return make_float4(m[0] * c.x + m[4] * c.y + m[8] * c.z + m[12] * c.w + m[16],
                           m[1] * c.x + m[5] * c.y + m[9] * c.z + m[13] * c.w + m[17],
                           m[2] * c.x + m[6] * c.y + m[10] * c.z + m[14] * c.w + m[18],
                           m[3] * c.x + m[7] * c.y + m[11] * c.z + m[15] * c.w + m[19]);
    }
    if (od.filter != PF_PATTERN_FILTER_BLUR_X && od.filter != PF_PATTERN_FILTER_BLUR_Y)
        return page_sample(tex, W, H, od.flags, u, v);
    const float sx = od.blur[0] / (float)W, sy = od.blur[1] / (float)H;
    const int support = (int)od.blur[2];
    float gx = od.blur[3], gy = od.blur[4];
    const float gz = od.blur[5];
    float sum = gx;
    float4 c = page_sample(tex, W, H, od.flags, u, v);
    c = make_float4(c.x * gx, c.y * gx, c.z * gx, c.w * gx);
    gx *= gy; gy *= gz;
    for (int i = 1; i <= support; i += 2) {
        float partial = gx;
        gx *= gy; gy *= gz;
        partial += gx;
        const float o = (float)i + gx / partial;
        const float4 a = page_sample(tex, W, H, od.flags, u - sx * o, v - sy * o);
        const float4 b = page_sample(tex, W, H, od.flags, u + sx * o, v + sy * o);
        c.x += (a.x + b.x) * partial; c.y += (a.y + b.y) * partial;
        c.z += (a.z + b.z) * partial; c.w += (a.w + b.w) * partial;
        sum += 2.0f * partial;
        gx *= gy; gy *= gz;
    }
    return make_float4(c.x / sum, c.y / sum, c.z / sum, c.w / sum);
}

// Composite one visible tile with paint effects into this lane's 8 pixels
// (column col, rows half*8 .. half*8+7 of screen tile (tx, ty)).  The pixel
// loop stays rolled, with the destination in a local array: unrolled, the
// blend modes' code overflows the instruction cache.
__device__ __forceinline__ void composite_paint_tile(const FrameDev& f, uint32_t fx, uint32_t paint, const float cov[8],
                                                     int32_t tx, int32_t ty, int col, int half, float d0[8],
                                                     float d1[8], float d2[8], float d3[8]) {
    const uint32_t mode = fx & 31u, grad1 = fx >> 5;
    const float4 base = unpack_unorm8(paint);
    float4 dd[8];
    float cv[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        dd[k] = make_float4(d0[k], d1[k], d2[k], d3[k]);
        cv[k] = cov[k];
    }
    const OverlayDev* gd = grad1 ? &f.overlays[grad1 - 1] : nullptr;
    const uint32_t* ramp = f.texels + (gd ? gd->texel_offset : 0u);
    float t[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    int32_t wrap = 0;
    bool radial = false, pattern = false;
    float fx0 = 0.0f, fy0 = 0.0f, vx = 0.0f, vy = 0.0f, r0 = 0.0f, dr = 0.0f, qa = 0.0f;
    if (gd) {
        gradient_frame_transform(f, *gd, t);
        wrap = gd->wrap;
        radial = gd->kind == PF_GRADIENT_RADIAL;
        pattern = gd->kind == kOverlayPattern;
        // filterRadialGradient (tile_fragment.inc.glsl:274-307): per-tile terms
        fx0 = gd->from_x; fy0 = gd->from_y; vx = gd->vec_x; vy = gd->vec_y; r0 = gd->r0;
        dr = gd->r1 - gd->r0;
        qa = (vx * vx + vy * vy) - dr * dr;
    }
    const float px = (float)(tx * 16 + col) + 0.5f;
#pragma unroll 1
    for (int k = 0; k < 8; k++) {
        float4 c = base;
        float a = base.w * cv[k];
        if (gd) {
            const float py = (float)(ty * 16 + half * 8 + k) + 0.5f;
            const float u = t[0] * px + t[1] * py + t[2];
            if (pattern) {
                c = pattern_color(*gd, ramp, u, t[3] * px + t[4] * py + t[5]);
            } else if (!radial) {
                c = ramp_sample(ramp, u, wrap);
            } else {
                const float v = t[3] * px + t[4] * py + t[5];
                const float dpx = u - fx0, dpy = v - fy0;
                const float qb = (dpx * vx + dpy * vy) + r0 * dr;
                const float qc = (dpx * dpx + dpy * dpy) - r0 * r0;
                const float disc = qb * qb - qa * qc;
                c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (disc != 0.0f) {
                    const float sq = sqrtf(disc);
                    float lo = (sq + qb) / qa, hi = (-sq + qb) / qa;
                    if (lo > hi) { const float tmp = lo; lo = hi; hi = tmp; }
                    c = ramp_sample(ramp, lo >= 0.0f ? lo : hi, wrap);
                }
            }
            // combineColor0 SrcIn (tile_fragment.inc.glsl:81-89): the texel's
            // colour, its alpha times the base colour's
            a = c.w * base.w * cv[k];
        }
        float4 d = dd[k];
        blend_pixel(mode, c.x, c.y, c.z, a, d.x, d.y, d.z, d.w);
        dd[k] = d;
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
        d0[k] = dd[k].x; d1[k] = dd[k].y; d2[k] = dd[k].z; d3[k] = dd[k].w;
    }
}

// ---------------------------------------------------------------------------
// Fill + composite in two kernels.  k_mask: one warp per visible tile with a
// mask (the fill pass, shaders/d3d11/fill.cs.glsl:61-88, with the resolve and
// clip combine of the tile pass) writes its resolved coverage as 16-bit
// unorms; visible entries are independent, so every warp works on its own
// tile.  k_composite: a persistent kernel whose warps pull batches of screen
// tiles from a work counter and composite each screen tile's visible list in
// draw order (tile.cs.glsl:91-159) from those coverages.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 pack_cov16(const float cov[8]) {
    auto q = [](float c) { return (uint32_t)__float2uint_rn(__saturatef(c) * 65535.0f); };
    return make_uint4(q(cov[0]) | (q(cov[1]) << 16), q(cov[2]) | (q(cov[3]) << 16), q(cov[4]) | (q(cov[5]) << 16),
                      q(cov[6]) | (q(cov[7]) << 16));
}
__device__ __forceinline__ void unpack_cov16(uint4 m, float cov[8]) {
    const float s = 1.0f / 65535.0f;
    cov[0] = (float)(m.x & 0xffffu) * s; cov[1] = (float)(m.x >> 16) * s;
    cov[2] = (float)(m.y & 0xffffu) * s; cov[3] = (float)(m.y >> 16) * s;
    cov[4] = (float)(m.z & 0xffffu) * s; cov[5] = (float)(m.z >> 16) * s;
    cov[6] = (float)(m.w & 0xffffu) * s; cov[7] = (float)(m.w >> 16) * s;
}

// ---- bulk copies (cp.async.bulk) into shared memory, completed on an mbarrier
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// orders this thread's earlier shared-memory accesses before later bulk copies into the same memory
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bulk_copy_to_smem(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// Bounded wait for phase `parity` of `bar` to complete (false: gave up).
constexpr uint32_t kCopyWaitLimit = 1u << 22;
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity) {
    for (uint32_t it = 0; it < kCopyWaitLimit; it++)
        if (mbar_test(bar, parity)) return true;
    return false;
}

// The fill pass (k_mask): each warp takes every (total warps)-th entry of
// the mask work list and writes the entry's resolved coverage to its slot.
// Two forms: by default the fills are read from global memory by the lanes
// that accumulate them (the work list read one entry ahead); with the
// tuning knob mask_stage_fills, a fill range of at least that many fills is
// copied into the warp's shared memory by one bulk copy (rounded out to
// 16-byte boundaries) one entry ahead of its use.  Ranges larger than a
// staging buffer, and clip-combined or clip-chain tiles (which read tile and
// clip records), are read from global memory in both.
constexpr int kMaskKernelWarps = 4;
constexpr uint32_t kStageFills = 128;  // per staging buffer (1 KiB)
struct MaskScratch {
    CovBuf b0, b1;
    uint2 stage[2][kStageFills];
    unsigned long long bar[2];
};

// Coverage of work-list entry e, with a mask entry's fills read from src, to
// the entry's slot.
__device__ __forceinline__ void mask_entry(const FrameDev& f, int4 e, const uint2* src, CovBuf& b0, CovBuf& b1) {
    const uint32_t kind = ((uint32_t)e.z >> 9) & 3u, slot = (uint32_t)e.w;
    float cov[8];
    if (kind == kVisMask) {
        int v[8];
        warp_accumulate_packed(src, (uint32_t)e.y, b0);
        warp_column_values(b0, v);
        __syncwarp();  // the buffer is cleared by the next tile
        const bool even_odd = ((uint32_t)e.z >> 8) & 1u;
        const float bd = (float)(int8_t)(e.z & 0xff);
#pragma unroll
        for (int q = 0; q < 8; q++) cov[q] = resolve_coverage((float)v[q] * kCovInvScale + bd, even_odd);
    } else {  // clip-combined or behind a clip chain: from the tile and clip records
        const uint32_t g = (uint32_t)(f.vis_key[slot] >> 32);
        tile_coverage8(f, f.tiles[g], g, b0, b1, cov);
    }
    f.vis_mask[(size_t)slot * 32u + (uint32_t)(threadIdx.x & 31)] = pack_cov16(cov);
}

__device__ __forceinline__ bool mask_pass_ok(const FrameDev& f) {
    return frame_ok(f) && f.counters->fills <= f.fill_cap && f.counters->visible <= f.vis_cap;
}
__device__ __forceinline__ uint32_t mask_entry_count(const FrameDev& f) {
    return (uint32_t)min((unsigned long long)f.counters->mask_items, (unsigned long long)f.vis_cap);
}

__global__ void __launch_bounds__(kMaskKernelWarps * 32, 8) k_mask(FrameDev f) {
    pdl_enter();
    __shared__ CovBuf bufs[kMaskKernelWarps][2];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (!mask_pass_ok(f)) return;
    const uint32_t M = mask_entry_count(f);
    const uint32_t stride = gridDim.x * kMaskKernelWarps;
    uint32_t k = blockIdx.x * kMaskKernelWarps + wid;
    if (k >= M) return;
    const int4 none = make_int4(0, 0, 0, 0);
    int4 cur = f.mask_items[k];
    unsigned long long fills_read = 0;  // the fills of this warp's tiles (frame statistics)
    for (; k < M; k += stride) {
        const int4 nxt = k + stride < M ? f.mask_items[k + stride] : none;
        fills_read += (uint32_t)cur.y;
        mask_entry(f, cur, f.fills + (uint32_t)cur.x, bufs[wid][0], bufs[wid][1]);
        cur = nxt;
    }
    if (lane == 0) atomicAdd((unsigned long long*)&f.counters->mask_fills, fills_read);
}

// Issue the bulk copy of entry `e`'s fills into staging buffer `buf` (lane 0;
// every lane gets the same answer: whether it was issued).
__device__ __forceinline__ bool stage_fills(const FrameDev& f, int4 e, MaskScratch& ws, int buf) {
    const uint32_t kind = ((uint32_t)e.z >> 9) & 3u;
    if (kind != kVisMask || e.y == 0 || e.y < f.tune.mask_stage) return false;
    const uint32_t first = (uint32_t)e.x & ~1u, end = ((uint32_t)e.x + (uint32_t)e.y + 1u) & ~1u;
    if (end - first > kStageFills) return false;
    if ((threadIdx.x & 31) == 0) {
        fence_proxy_async_smem();  // the buffer's previous contents were read through the generic proxy
        bulk_copy_to_smem(ws.stage[buf], f.fills + first, (end - first) * 8u, &ws.bar[buf]);
    }
    return true;
}

// The staged form: the work list is read two entries ahead and the fills of
// the next entry are in flight while the current one accumulates.
__global__ void __launch_bounds__(kMaskKernelWarps * 32, 8) k_mask_staged(FrameDev f) {
    pdl_enter();
    __shared__ MaskScratch scratch[kMaskKernelWarps];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    MaskScratch& ws = scratch[wid];
    if (!mask_pass_ok(f)) return;
    const uint32_t M = mask_entry_count(f);
    const uint32_t stride = gridDim.x * kMaskKernelWarps;
    uint32_t k = blockIdx.x * kMaskKernelWarps + wid;
    if (k >= M) return;
    if (lane == 0) {
        mbar_init(&ws.bar[0], 1);
        mbar_init(&ws.bar[1], 1);
        fence_mbar_init();
    }
    __syncwarp();
    const int4 none = make_int4(0, 0, 0, 0);  // past the list: no work
    int4 cur = f.mask_items[k];
    int4 nxt = k + stride < M ? f.mask_items[k + stride] : none;
    uint32_t phase = 0;  // bit b: parity of the next completion of buffer b
    int buf = 0;
    bool cur_staged = stage_fills(f, cur, ws, buf);
    bool stalled = false;
    int stall_buf = 0;
    uint32_t stall_parity = 0;
    unsigned long long fills_read = 0;
    for (; k < M; k += stride) {
        const int4 later = k + 2 * stride < M ? f.mask_items[k + 2 * stride] : none;
        const bool nxt_staged = !stalled && stage_fills(f, nxt, ws, buf ^ 1);
        fills_read += (uint32_t)cur.y;
        const uint2* src = f.fills + (uint32_t)cur.x;
        if (cur_staged) {
            const uint32_t parity = (phase >> buf) & 1u;
            const bool arrived = mbar_wait(&ws.bar[buf], parity);
            phase ^= 1u << buf;
            if (arrived) {
                src = ws.stage[buf] + ((uint32_t)cur.x & 1u);
            } else if (!stalled) {
                stalled = true;  // no more copies: read global memory from here on
                stall_buf = buf;
                stall_parity = parity;
                if (lane == 0) atomicOr(&f.counters->status, kStatusCopyStall);
            }
        }
        mask_entry(f, cur, src, ws.b0, ws.b1);
        cur = nxt;
        nxt = later;
        cur_staged = nxt_staged;
        buf ^= 1;
    }
    if (lane == 0) atomicAdd((unsigned long long*)&f.counters->mask_fills, fills_read);
    // the copy a wait gave up on may still be in flight: wait for it again,
    // with the same bound, before the warp leaves its shared memory
    if (stalled) mbar_wait(&ws.bar[stall_buf], stall_parity);
}

void launch_mask(const FrameDev& f, cudaStream_t s) {
    if (f.screen_count == 0) return;
    count_launch();
    if (f.tune.mask_stage > 0) {
        const int blocks = (int)f.sms * resident_blocks(k_mask_staged, kMaskKernelWarps * 32);
        pdl_launch(k_mask_staged, blocks, kMaskKernelWarps * 32, 0, s, f);
    } else {
        const int blocks = (int)f.sms * resident_blocks(k_mask, kMaskKernelWarps * 32);
        pdl_launch(k_mask, blocks, kMaskKernelWarps * 32, 0, s, f);
    }
}

// Composite screen tile st (frame index) into this lane's 8 pixels: n
// visible entries from `base`; for n <= 32, lane_key is the lane's entry key
// (read ahead by the caller).
template <int MODE, bool PAINT>
__device__ __forceinline__ void composite_screen_tile(const FrameDev& f, uint32_t st, uint32_t base, uint32_t n,
                                                      unsigned long long lane_key, void* out, float4 bg) {
    const int lane = threadIdx.x & 31, col = lane & 15, half = lane >> 4;
    const SceneDev& sc = f.scenes[scene_of_screen_tile(f, f.screen_begin + st)];
    const int4 s = sc.screen;
    const int32_t sw = s.z - s.x;
    const uint32_t lst = f.screen_begin + st - sc.screen_offset;
    const uint32_t row = lst / (uint32_t)sw;
    const int32_t tx = s.x + (int32_t)(lst - row * (uint32_t)sw), ty = s.y + (int32_t)row;

    // draw order = global tile order (paths in order): sort the (tile, slot) keys
    const bool lane_list = n <= 32;  // one key per lane; longer lists sort in place in global memory
    int2 lane_info = make_int2(0, 0);  // paint, meta of the lane's entry in draw order
    if (lane_list) {
        uint32_t N = 1;
        while (N < n) N <<= 1;
        if (n > 1) lane_key = warp_sort_lanes(lane_key, N);
        if ((uint32_t)lane < n) {
            const int4 info = f.vis_info[(uint32_t)lane_key];
            lane_info = make_int2(info.z, info.w);
        }
    } else {
        warp_bitonic_sort(f.vis_key + base, n);
    }
    // Entry i of the draw order: its slot, record and coverage, fetched one
    // entry ahead.  A short list has every record in the lanes, so a solid
    // entry (whose slot holds no coverage) skips the coverage read; a long
    // list reads the coverage whatever the entry's kind, starting it before
    // the record is waited for (a solid entry's value is not used).
    auto entry = [&](uint32_t i, uint32_t& slot, uint4& mask, uint32_t& paint, uint32_t& meta) {
        if (lane_list) {
            slot = __shfl_sync(0xffffffffu, (uint32_t)lane_key, (int)i);
            paint = (uint32_t)__shfl_sync(0xffffffffu, lane_info.x, (int)i);
            meta = (uint32_t)__shfl_sync(0xffffffffu, lane_info.y, (int)i);
            mask = ((meta >> 9) & 3u) != kVisSolid ? f.vis_mask[(size_t)slot * 32u + (uint32_t)lane]
                                                   : make_uint4(0u, 0u, 0u, 0u);
        } else {
            slot = (uint32_t)f.vis_key[base + i];
            mask = f.vis_mask[(size_t)slot * 32u + (uint32_t)lane];
            const int4 info = f.vis_info[slot];
            paint = (uint32_t)info.z;
            meta = (uint32_t)info.w;
        }
    };

    float d0[8], d1[8], d2[8], d3[8];
#pragma unroll
    for (int k = 0; k < 8; k++) { d0[k] = bg.x; d1[k] = bg.y; d2[k] = bg.z; d3[k] = bg.w; }
    uint32_t n_slot = 0, n_paint = 0, n_meta = 0;
    uint4 n_mask = make_uint4(0u, 0u, 0u, 0u);
    if (n) entry(0, n_slot, n_mask, n_paint, n_meta);
    for (uint32_t i = 0; i < n; i++) {
        const uint32_t paint = n_paint, meta = n_meta;
        const uint4 m = n_mask;
        if (i + 1 < n) entry(i + 1, n_slot, n_mask, n_paint, n_meta);
        float cov[8];
        if (((meta >> 9) & 3u) == kVisSolid) {
            const float c = resolve_coverage((float)(int8_t)(meta & 0xffu), (meta >> 8) & 1u);
#pragma unroll
            for (int k = 0; k < 8; k++) cov[k] = c;
        } else {
            unpack_cov16(m, cov);
        }
        const uint32_t fx = PAINT ? (meta >> 11) : 0u;
        const float pa = (float)(paint >> 24) * (1.0f / 255.0f);
        if (PAINT && fx != 0) {
            composite_paint_tile(f, fx, paint, cov, tx, ty, col, half, d0, d1, d2, d3);
        } else if (MODE == 0) {
            const float pr = (float)(paint & 0xffu) * (1.0f / 255.0f);
            const float pg = (float)((paint >> 8) & 0xffu) * (1.0f / 255.0f);
            const float pb = (float)((paint >> 16) & 0xffu) * (1.0f / 255.0f);
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const float a = pa * cov[k], ia = 1.0f - a;
                d0[k] = pr * a + d0[k] * ia; d1[k] = pg * a + d1[k] * ia;
                d2[k] = pb * a + d2[k] * ia; d3[k] = a + d3[k] * ia;
            }
        } else {
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const float a = pa * cov[k];
                d3[k] = a + d3[k] * (1.0f - a);
            }
        }
    }
    const int X = tx * 16 + col;
    if (X < sc.clip.x || X >= sc.clip.z) return;
    const int Y0 = ty * 16 + half * 8;
    const bool rows_inside = Y0 >= sc.clip.y && Y0 + 8 <= sc.clip.w;
    uint64_t o = sc.out_offset + (uint64_t)(int64_t)(Y0 - sc.origin_y) * (uint64_t)(int64_t)sc.pitch +
                 (uint64_t)(int64_t)(X - sc.origin_x);
#pragma unroll
    for (int k = 0; k < 8; k++, o += (uint64_t)(int64_t)sc.pitch) {
        if (!rows_inside && (Y0 + k < sc.clip.y || Y0 + k >= sc.clip.w)) continue;
        if (MODE == 0) {
            auto q = [](float v) { return (uint32_t)__float2uint_rn(__saturatef(v) * 255.0f); };
            ((uint32_t*)out)[o] = q(d0[k]) | (q(d1[k]) << 8) | (q(d2[k]) << 16) | (q(d3[k]) << 24);
        } else if (MODE == 1) {
            ((uint8_t*)out)[o] = (uint8_t)__float2uint_rn(__saturatef(d3[k]) * 255.0f);
        } else {
            ((float*)out)[o] = d3[k];
        }
    }
}

// Persistent: each warp pulls batches of `comp_batch` screen tiles from the
// frame's work counter until none are left, so long lists do not hold up a
// fixed share of the grid.  At most 64 registers a thread, with paint effects
// too (32 warps an SM: the paint composite measured 0.408 ms at 64 registers
// against 0.434 at the 111 it takes unbounded, without spills either way).
template <int MODE, int WARPS, bool PAINT>
__global__ void __launch_bounds__(WARPS * 32, 32 / WARPS) k_composite(FrameDev f, void* out, float4 bg) {
    pdl_enter();
    const int lane = threadIdx.x & 31;
    const bool ok = frame_ok(f) && f.counters->fills <= f.fill_cap && f.counters->visible <= f.vis_cap;
    const uint32_t batch = (uint32_t)f.tune.comp_batch;
    for (uint32_t it = 0; it <= f.screen_count; it++) {  // bounded: each step takes at least one tile
        uint32_t st0 = 0;
        if (lane == 0) st0 = atomicAdd(&f.counters->composite_next, batch);
        st0 = __shfl_sync(0xffffffffu, st0, 0);
        if (st0 >= f.screen_count) break;
        const uint32_t nb = min(st0 + batch, f.screen_count) - st0;
        // the batch's list bounds (lane t: screen_base[st0 + t]); each tile's
        // keys are read while the previous tile composites
        const uint32_t lb = (ok && (uint32_t)lane <= nb) ? f.screen_base[st0 + lane] : 0u;
        auto keys = [&](uint32_t t, uint32_t& base, uint32_t& n) {
            base = __shfl_sync(0xffffffffu, lb, (int)t);
            n = __shfl_sync(0xffffffffu, lb, (int)t + 1) - base;
            return (n <= 32 && (uint32_t)lane < n) ? f.vis_key[base + lane] : ~0ull;
        };
        uint32_t base, n;
        unsigned long long key = keys(0, base, n);
        for (uint32_t t = 0; t < nb; t++) {
            uint32_t base_n = 0, n_n = 0;
            unsigned long long key_n = ~0ull;
            if (t + 1 < nb) key_n = keys(t + 1, base_n, n_n);
            composite_screen_tile<MODE, PAINT>(f, st0 + t, base, n, key, out, bg);
            base = base_n;
            n = n_n;
            key = key_n;
        }
    }
}

template <int MODE, int WARPS, bool PAINT>
void launch_composite_instance(const FrameDev& f, void* out, const float4& bg, cudaStream_t s) {
    const int threads = WARPS * 32;
    const uint32_t per_block = (uint32_t)f.tune.comp_batch * WARPS;
    const uint32_t needed = (f.screen_count + per_block - 1) / per_block;
    const uint32_t resident = f.sms * (uint32_t)resident_blocks(k_composite<MODE, WARPS, PAINT>, threads);
    count_launch();
    pdl_launch(k_composite<MODE, WARPS, PAINT>, std::max(1u, std::min(needed, resident)), threads, 0, s, f, out, bg);
}

template <int MODE, int WARPS>
void launch_composite_warps(const FrameDev& f, void* out, const float4& bg, cudaStream_t s) {
    if (f.paint_effects) launch_composite_instance<MODE, WARPS, true>(f, out, bg, s);
    else launch_composite_instance<MODE, WARPS, false>(f, out, bg, s);
}

template <int MODE>
void launch_composite_mode(const FrameDev& f, void* out, const float4& bg, cudaStream_t s) {
    const int w = f.tune.comp_warps;
    if (w == 2) launch_composite_warps<MODE, 2>(f, out, bg, s);
    else if (w == 8) launch_composite_warps<MODE, 8>(f, out, bg, s);
    else launch_composite_warps<MODE, 4>(f, out, bg, s);
}

void launch_composite(const FrameDev& f, int mode, void* out, const float4& bg, cudaStream_t s) {
    if (f.screen_count == 0) return;
    if (mode == 0) launch_composite_mode<0>(f, out, bg, s);
    else if (mode == 1) launch_composite_mode<1>(f, out, bg, s);
    else launch_composite_mode<2>(f, out, bg, s);
}

// ---------------------------------------------------------------------------
// differentiable frames: FP32 composite that records the adjoint's tape
// ---------------------------------------------------------------------------
// Coverage of one path tile for this lane's 8 pixels with d(coverage)/d(mask)
// codes: bits 0-1 for the mask of tile.alpha (own, or the clip's where the
// draw tile borrowed it), bits 2-3 for the clip's mask of a combined tile.
__device__ __forceinline__ void tile_coverage8_diff(const FrameDev& f, int4 rec, uint32_t g, WarpScratch& ws,
                                                    float cov[8], uint32_t code[8]) {
    const uint32_t gp = (uint32_t)rec.z;
    const bool even_odd = (tile_ctrl(rec) & 0x2u) != 0;
    const float bd = (float)tile_backdrop(rec);
    bool combine = false;
    int4 crec = make_int4(0, 0, 0, 0);
    if (tile_ctrl(rec) != 0 && f.path.clip_gpath[gp] >= 0) {  // draw tiles only carry clip records
        crec = f.clips[g];
        combine = (uint32_t)crec.x != kInvalid && (uint32_t)crec.z != kInvalid;
    }
    if (combine) {
        // min(|d|, |s|) picks one mask per pixel (ties: the draw path's own)
        int vd[8], vs[8];
        warp_accumulate_tile<true>(f, (uint32_t)crec.x, ws.b0);
        warp_accumulate_tile<true>(f, (uint32_t)crec.z, ws.b1);
        warp_column_values(ws.b0, vd);
        warp_column_values(ws.b1, vs);
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const float wd = (float)vd[k] * kCovInvScale + (float)crec.y;
            const float wc = (float)vs[k] * kCovInvScale + (float)crec.w;
            const bool own = fabsf(wd) <= fabsf(wc);
            float dc;
            cov[k] = resolve_coverage_d(fminf(fabsf(wd), fabsf(wc)) + bd, even_odd, &dc);
            const float dm = dc * ((own ? wd : wc) >= 0.0f ? 1.0f : -1.0f);
            code[k] = own ? enc_d(dm) : (enc_d(dm) << 2);
        }
    } else if ((uint32_t)rec.y != kInvalid) {
        int v[8];
        warp_accumulate_tile<true>(f, (uint32_t)rec.y, ws.b0);
        warp_column_values(ws.b0, v);
#pragma unroll
        for (int k = 0; k < 8; k++) {
            float dc;
            cov[k] = resolve_coverage_d((float)v[k] * kCovInvScale + bd, even_odd, &dc);
            code[k] = enc_d(dc);
        }
    } else {
        const float c = resolve_coverage(bd, even_odd);
#pragma unroll
        for (int k = 0; k < 8; k++) { cov[k] = c; code[k] = 0; }
    }
    __syncwarp();
}

// As k_composite in FP32 single-channel mode, with the paint alpha of the
// differentiable frame.  Per visible entry e (the screen tile's list in draw
// order, written back to vis) and pixel, the tape keeps the coverage, the
// composite value below the entry and the coverage derivative codes.
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_composite_diff(FrameDev f, float* out, float4 bg) {
    pdl_enter();
    __shared__ WarpScratch scratch[WARPS];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t st = blockIdx.x * WARPS + wid;
    if (st >= f.screen_count) return;
    WarpScratch& ws = scratch[wid];

    const SceneDev& sc = f.scenes[scene_of_screen_tile(f, f.screen_begin + st)];
    const int4 s = sc.screen;
    const int32_t sw = s.z - s.x;
    const uint32_t lst = f.screen_begin + st - sc.screen_offset;
    const int32_t tx = s.x + (int32_t)(lst % (uint32_t)sw), ty = s.y + (int32_t)(lst / (uint32_t)sw);
    const int col = lane & 15, half = lane >> 4;

    const bool ok = frame_ok(f) && f.counters->fills <= f.fill_cap && f.counters->visible <= f.vis_cap;
    uint32_t n = 0, base = 0;
    if (ok) { base = f.screen_base[st]; n = f.screen_base[st + 1] - base; }
    if (n <= kWarpListCap) {
        for (uint32_t i = lane; i < n; i += 32) ws.keys[i] = f.vis[base + i];
        __syncwarp();
        if (n > 1) {
            warp_bitonic_sort(ws.keys, n);
            for (uint32_t i = lane; i < n; i += 32) f.vis[base + i] = ws.keys[i];  // draw order for the adjoint
        }
    } else {
        warp_bitonic_sort(f.vis + base, n);
    }
    __syncwarp();
    const uint32_t* list = n <= kWarpListCap ? ws.keys : f.vis + base;

    float d[8];
#pragma unroll
    for (int k = 0; k < 8; k++) d[k] = bg.w;
    for (uint32_t i = 0; i < n; i++) {
        const uint32_t g = list[i];
        const int4 rec = f.tiles[g];
        float cov[8];
        uint32_t code[8];
        tile_coverage8_diff(f, rec, g, ws, cov, code);
        const float pa = f.path.alpha_f[f.path.draw_index[(uint32_t)rec.z]];
        const uint64_t t0 = (uint64_t)(base + i) * 256u + (uint32_t)(half * 128 + col);
#pragma unroll
        for (int k = 0; k < 8; k++) {
            f.tape[t0 + k * 16] = tape_pack(cov[k], d[k], code[k]);
            const float a = pa * cov[k];
            d[k] = a + d[k] * (1.0f - a);
        }
    }
    const int X = tx * 16 + col;
    if (X < sc.clip.x || X >= sc.clip.z) return;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int Y = ty * 16 + half * 8 + k;
        if (Y < sc.clip.y || Y >= sc.clip.w) continue;
        out[sc.out_offset + (uint64_t)(int64_t)(Y - sc.origin_y) * (uint64_t)(int64_t)sc.pitch +
            (uint64_t)(int64_t)(X - sc.origin_x)] = d[k];
    }
}

void launch_composite_diff(const FrameDev& f, float* out, const float4& bg, cudaStream_t s) {
    if (f.screen_count == 0) return;
    count_launch();
    pdl_launch(k_composite_diff<4>, (f.screen_count + 3) / 4, 128, 0, s, f, out, bg);
}

// ---------------------------------------------------------------------------
// readback of raw alpha masks and resolved tile coverage (parity checks)
// ---------------------------------------------------------------------------
constexpr int kMaskWarps = 4;

__global__ void k_alpha_masks(FrameDev f, float* out) {
    pdl_enter();
    __shared__ WarpScratch scratch[kMaskWarps];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t a = blockIdx.x * kMaskWarps + wid;
    if (a >= f.counters->alpha_tiles) return;
    if (f.diff) warp_accumulate_tile<true>(f, a, scratch[wid].b0);
    else warp_accumulate_tile<false>(f, a, scratch[wid].b0);
    int v[8];
    warp_column_values(scratch[wid].b0, v);
    const int col = lane & 15, half = lane >> 4;
#pragma unroll
    for (int k = 0; k < 8; k++) out[(uint64_t)a * 256 + (half * 8 + k) * 16 + col] = (float)v[k] * kCovInvScale;
}

__global__ void k_tile_cov(FrameDev f, float* out) {
    pdl_enter();
    __shared__ WarpScratch scratch[kMaskWarps];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t g = blockIdx.x * kMaskWarps + wid;
    if (g >= f.counters->tiles) return;
    float cov[8];
    if (f.diff) {
        uint32_t code[8];
        tile_coverage8_diff(f, f.tiles[g], g, scratch[wid], cov, code);
    } else {
        tile_coverage8(f, f.tiles[g], g, scratch[wid].b0, scratch[wid].b1, cov);
    }
    const int col = lane & 15, half = lane >> 4;
#pragma unroll
    for (int k = 0; k < 8; k++) out[(uint64_t)g * 256 + (half * 8 + k) * 16 + col] = cov[k];
}

void launch_masks(const FrameDev& f, float* alpha_masks, float* tile_cov, cudaStream_t s) {
    uint32_t blocks = (f.tile_cap + kMaskWarps - 1) / kMaskWarps + 1;
    if (alpha_masks) { count_launch(); pdl_launch(k_alpha_masks, blocks, kMaskWarps * 32, 0, s, f, alpha_masks); }
    if (tile_cov) { count_launch(); pdl_launch(k_tile_cov, blocks, kMaskWarps * 32, 0, s, f, tile_cov); }
}

}  // namespace pf

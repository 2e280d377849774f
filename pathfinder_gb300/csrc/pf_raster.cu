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
#include "pf_kernels.cuh"

namespace pf {

__device__ __forceinline__ uint32_t upper_bound_u32(const uint32_t* a, uint32_t n, uint32_t v) {
    // first index i in [0, n) with a[i] > v
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (a[mid] <= v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// path owning global tile g: the last path whose tile_offset <= g (and which has tiles)
__device__ __forceinline__ uint32_t path_of_tile(const FrameDev& f, uint32_t g) {
    return upper_bound_u32(f.path.tile_offset, f.path_count + 1, g) - 1;
}

__device__ __forceinline__ int4 pack_tile(int32_t tx, int32_t ty, uint32_t alpha, uint32_t path_id, uint16_t color,
                                          uint8_t ctrl, int8_t backdrop) {
    int4 r;
    r.x = (int)(((uint32_t)(uint16_t)(int16_t)tx) | ((uint32_t)(uint16_t)(int16_t)ty << 16));
    r.y = (int)alpha;
    r.z = (int)path_id;
    r.w = (int)((uint32_t)color | ((uint32_t)ctrl << 16) | ((uint32_t)(uint8_t)backdrop << 24));
    return r;
}
__device__ __forceinline__ int8_t tile_backdrop(int4 r) { return (int8_t)((uint32_t)r.w >> 24); }
__device__ __forceinline__ int32_t tile_x(int4 r) { return (int32_t)(int16_t)((uint32_t)r.x & 0xffffu); }
__device__ __forceinline__ int32_t tile_y(int4 r) { return (int32_t)(int16_t)((uint32_t)r.x >> 16); }

// A solid tile occludes only if it resolves to full coverage (see DESIGN:
// nonzero: any nonzero backdrop, as builder.rs:1013-1029; even-odd: odd).
__device__ __forceinline__ bool solid_occludes(int8_t b, bool even_odd) {
    if (b == 0) return false;
    return even_odd ? ((b & 1) != 0) : true;
}

// ---------------------------------------------------------------------------
// propagate: one thread per (path, tile column)
// ---------------------------------------------------------------------------
__global__ void k_propagate(FrameDev f, int clip_pass) {
    uint64_t C = f.counters->columns;
    if (f.counters->tiles > f.tile_cap || C > f.col_cap) return;
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < C; c += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t gp = upper_bound_u32(f.path.col_offset, f.path_count + 1, (uint32_t)c) - 1;
        bool is_clip = f.path.is_clip[gp] != 0;
        if (is_clip != (clip_pass != 0)) continue;
        int4 r = f.path.tile_rect[gp];
        int32_t w = r.z - r.x, h = r.w - r.y;
        int32_t ox = (int32_t)(c - f.path.col_offset[gp]);
        uint32_t tbase = f.path.tile_offset[gp];
        int32_t acc = f.col_backdrop[c];
        uint8_t rule = f.path.rule[gp];
        bool even_odd = rule == 1;
        uint8_t ctrl = is_clip ? 0 : (even_odd ? 0x2 : 0x1);
        uint32_t local = f.path.local_index[gp];
        uint16_t color = is_clip ? 0 : (uint16_t)(local & 0xffffu);
        int32_t clip_gp = is_clip ? -1 : f.path.clip_gpath[gp];
        int4 cr = make_int4(0, 0, 0, 0);
        uint32_t cbase = 0;
        if (clip_gp >= 0) { cr = f.path.tile_rect[clip_gp]; cbase = f.path.tile_offset[clip_gp]; }
        const SceneDev& sc = f.scenes[f.path.scene[gp]];
        bool occluder_path = !is_clip && ((f.path.paint[gp] >> 24) == 255u);
        for (int32_t oy = 0; oy < h; oy++) {
            uint32_t g = tbase + (uint32_t)(oy * w + ox);
            int32_t delta = f.tile_delta[g];
            bool has_fill = f.tile_fill_base[g + 1] > f.tile_fill_base[g];
            uint32_t own_alpha = has_fill ? f.tile_alpha[g] : kInvalid;
            if (has_fill) f.alpha_owner[own_alpha] = g;
            uint32_t alpha = own_alpha;
            int8_t backdrop = (int8_t)acc;
            int32_t tx = r.x + ox, ty = r.y + oy;
            if (clip_gp >= 0) {
                int4 clip_rec = make_int4((int)kInvalid, 0, (int)kInvalid, 0);
                if (cr.x <= tx && cr.y <= ty && tx <= cr.z - 1 && ty <= cr.w - 1) {
                    int4 ct = f.tiles[cbase + (uint32_t)((ty - cr.y) * (cr.z - cr.x) + (tx - cr.x))];
                    uint32_t calpha = (uint32_t)ct.y;
                    int8_t cb = tile_backdrop(ct);
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
            } else if (!is_clip) {
                f.clips[g] = make_int4((int)kInvalid, 0, (int)kInvalid, 0);
            }
            f.tiles[g] = pack_tile(tx, ty, alpha, local, color, ctrl, backdrop);
            if (occluder_path && alpha == kInvalid && solid_occludes(backdrop, even_odd)) {
                int4 s = sc.screen;
                if (s.x <= tx && s.y <= ty && tx <= s.z - 1 && ty <= s.w - 1) {
                    uint32_t st = sc.screen_offset + (uint32_t)((ty - s.y) * (s.z - s.x) + (tx - s.x));
                    atomicMax(&f.zbuf[st], (int32_t)local);
                }
            }
            acc += delta;
        }
    }
}

void launch_propagate(const FrameDev& f, bool clip_pass, uint32_t, uint32_t, uint32_t, cudaStream_t s) {
    { count_launch(); k_propagate<<<152 * 8, 128, 0, s>>>(f, clip_pass ? 1 : 0); }
}

// ---------------------------------------------------------------------------
// visibility: count per screen tile, then scatter global tile indices
// ---------------------------------------------------------------------------
__global__ void k_visible(FrameDev f, int scatter) {
    uint64_t T = f.counters->tiles;
    if (T > f.tile_cap || f.counters->columns > f.col_cap) return;
    if (scatter && f.counters->visible > f.vis_cap) return;
    for (uint64_t gi = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; gi < T; gi += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t g = (uint32_t)gi;
        int4 rec = f.tiles[g];
        uint32_t alpha = (uint32_t)rec.y;
        int8_t b = tile_backdrop(rec);
        uint32_t ctrl = ((uint32_t)rec.w >> 16) & 0xffu;
        if (ctrl == 0) continue;                       // clip path tile
        if (alpha == kInvalid && b == 0) continue;     // empty (builder.rs:1016-1018)
        uint32_t gp = path_of_tile(f, g);
        const SceneDev& sc = f.scenes[f.path.scene[gp]];
        int32_t tx = tile_x(rec), ty = tile_y(rec);
        int4 s = sc.screen;
        if (!(s.x <= tx && s.y <= ty && tx <= s.z - 1 && ty <= s.w - 1)) continue;
        uint32_t st = sc.screen_offset + (uint32_t)((ty - s.y) * (s.z - s.x) + (tx - s.x));
        if ((int32_t)(uint32_t)rec.z < f.zbuf[st]) continue;  // occluded (tile.vs.glsl:51-55)
        if (!scatter) {
            atomicAdd(&f.screen_cnt[st], 1u);
        } else {
            uint32_t slot = f.screen_base[st] + atomicSub(&f.screen_cnt[st], 1u) - 1u;
            if (slot < f.vis_cap) f.vis[slot] = g;
        }
    }
}

__global__ void k_check_visible(FrameDev f) {
    if (f.counters->visible > f.vis_cap) {
        atomicOr(&f.counters->status, kStatusVisibleCapacity);
        f.counters->needed_visible = f.counters->visible;
    }
}

void launch_visible(const FrameDev& f, bool scatter, cudaStream_t s) {
    if (scatter) { count_launch(); k_check_visible<<<1, 1, 0, s>>>(f); }
    { count_launch(); k_visible<<<152 * 8, 256, 0, s>>>(f, scatter ? 1 : 0); }
}

// ---------------------------------------------------------------------------
// fused fill + composite: one CTA (8 warps) per screen tile
// ---------------------------------------------------------------------------
constexpr int kCompThreads = 256;
constexpr int kCompWarps = kCompThreads / 32;
constexpr uint32_t kSortCap = 2048;

// Bitonic network in its "all comparators ascending" form: for block size k
// the first step compares i with i ^ (k - 1), later steps i with i ^ j.  Slots
// at or beyond n act as +inf and are never touched, so n need not be a power
// of two.
__device__ void bitonic_sort_u32(uint32_t* a, uint32_t n) {
    uint32_t N = 1;
    while (N < n) N <<= 1;
    for (uint32_t k = 2; k <= N; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) {
                uint32_t l = (j == (k >> 1)) ? (i ^ (k - 1)) : (i ^ j);
                if (l > i && l < n) {
                    uint32_t x = a[i], y = a[l];
                    if (y < x) { a[i] = y; a[l] = x; }
                }
            }
            __syncthreads();
        }
    }
}

struct CovBuf { int acc[256]; int carry[256]; };

__device__ __forceinline__ void warp_accumulate_tile(const FrameDev& f, uint32_t alpha, CovBuf& buf) {
    const int lane = threadIdx.x & 31;
    for (int k = lane; k < 256; k += 32) { buf.acc[k] = 0; buf.carry[k] = 0; }
    __syncwarp();
    uint32_t owner = f.alpha_owner[alpha];
    uint32_t b0 = f.tile_fill_base[owner], b1 = f.tile_fill_base[owner + 1];
    for (uint32_t i = b0 + lane; i < b1; i += 32) accumulate_fill_cells(f.fills[i], buf.acc, buf.carry);
}

__device__ __forceinline__ float buf_value(const CovBuf& b, int px, int py) {
    int s = b.acc[py * 16 + px];
    for (int r = 1; r <= py; r++) s += b.carry[r * 16 + px];
    return (float)s * kCovInvScale;
}

template <int MODE>
__global__ void __launch_bounds__(kCompThreads) k_composite(FrameDev f, void* out, float4 bg) {
    __shared__ uint32_t keys[kSortCap];
    __shared__ CovBuf bufs[kCompWarps][2];
    __shared__ int4 ent_rec[kCompWarps];
    __shared__ int4 ent_clip[kCompWarps];
    __shared__ uint32_t ent_gp[kCompWarps];

    const uint32_t st = blockIdx.x;
    // scene of this screen tile
    uint32_t si = 0;
    while (si + 1 < f.scene_count && f.scenes[si + 1].screen_offset <= st) si++;
    const SceneDev& sc = f.scenes[si];
    const int4 s = sc.screen;
    const int32_t sw = s.z - s.x;
    const uint32_t lst = st - sc.screen_offset;
    const int32_t tx = s.x + (int32_t)(lst % (uint32_t)sw), ty = s.y + (int32_t)(lst / (uint32_t)sw);
    const int px = threadIdx.x & 15, py = threadIdx.x >> 4;
    const int X = tx * 16 + px, Y = ty * 16 + py;

    bool ok = f.counters->tiles <= f.tile_cap && f.counters->columns <= f.col_cap &&
              f.counters->fills <= f.fill_cap && f.counters->visible <= f.vis_cap;
    uint32_t n = 0, base = 0;
    if (ok) { base = f.screen_base[st]; n = f.screen_base[st + 1] - base; }

    const uint32_t* list;
    if (n <= kSortCap) {
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) keys[i] = f.vis[base + i];
        __syncthreads();
        bitonic_sort_u32(keys, n);
        list = keys;
    } else {
        // rare: sort the list in place in global memory
        bitonic_sort_u32(f.vis + base, n);
        list = f.vis + base;
    }

    float d0 = bg.x, d1 = bg.y, d2 = bg.z, d3 = bg.w;  // premultiplied destination
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t b = 0; b < n; b += kCompWarps) {
        uint32_t i = b + (uint32_t)wid;
        if (i < n) {
            uint32_t g = list[i];
            int4 rec = f.tiles[g];
            uint32_t gp = path_of_tile(f, g);
            int4 crec = f.clips[g];
            if (lane == 0) { ent_rec[wid] = rec; ent_gp[wid] = gp; ent_clip[wid] = crec; }
            if (f.path.clip_gpath[gp] >= 0 && (uint32_t)crec.x != kInvalid && (uint32_t)crec.z != kInvalid) {
                warp_accumulate_tile(f, (uint32_t)crec.x, bufs[wid][0]);
                warp_accumulate_tile(f, (uint32_t)crec.z, bufs[wid][1]);
            } else if ((uint32_t)rec.y != kInvalid) {
                warp_accumulate_tile(f, (uint32_t)rec.y, bufs[wid][0]);
            }
        }
        __syncthreads();
        uint32_t m = n - b < (uint32_t)kCompWarps ? n - b : (uint32_t)kCompWarps;
        for (uint32_t k = 0; k < m; k++) {
            int4 rec = ent_rec[k];
            uint32_t gp = ent_gp[k];
            bool even_odd = ((((uint32_t)rec.w >> 16) & 0xffu) & 0x2u) != 0;
            int8_t bd = tile_backdrop(rec);
            int4 crec = ent_clip[k];
            float cov;
            if (f.path.clip_gpath[gp] >= 0 && (uint32_t)crec.x != kInvalid && (uint32_t)crec.z != kInvalid) {
                float md = buf_value(bufs[k][0], px, py), ms = buf_value(bufs[k][1], px, py);
                float mm = fminf(fabsf(md + (float)crec.y), fabsf(ms + (float)crec.w));
                cov = resolve_coverage(mm + (float)bd, even_odd);
            } else if ((uint32_t)rec.y != kInvalid) {
                cov = resolve_coverage(buf_value(bufs[k][0], px, py) + (float)bd, even_odd);
            } else {
                cov = resolve_coverage((float)bd, even_odd);
            }
            uint32_t paint = f.path.paint[gp];
            float pa = (float)(paint >> 24) * (1.0f / 255.0f);
            float a = pa * cov;
            if (MODE == 0) {
                float pr = (float)(paint & 0xffu) * (1.0f / 255.0f);
                float pg = (float)((paint >> 8) & 0xffu) * (1.0f / 255.0f);
                float pb = (float)((paint >> 16) & 0xffu) * (1.0f / 255.0f);
                float ia = 1.0f - a;
                d0 = pr * a + d0 * ia; d1 = pg * a + d1 * ia; d2 = pb * a + d2 * ia; d3 = a + d3 * ia;
            } else {
                d3 = a + d3 * (1.0f - a);
            }
        }
        __syncthreads();
    }
    if (X >= sc.width || Y >= sc.height || X < 0 || Y < 0) return;
    uint64_t o = sc.out_offset + (uint64_t)Y * (uint64_t)sc.width + (uint64_t)X;
    if (MODE == 0) {
        auto q = [](float v) { return (uint32_t)__float2uint_rn(fminf(fmaxf(v, 0.0f), 1.0f) * 255.0f); };
        ((uint32_t*)out)[o] = q(d0) | (q(d1) << 8) | (q(d2) << 16) | (q(d3) << 24);
    } else if (MODE == 1) {
        ((uint8_t*)out)[o] = (uint8_t)__float2uint_rn(fminf(fmaxf(d3, 0.0f), 1.0f) * 255.0f);
    } else {
        ((float*)out)[o] = d3;
    }
}

void launch_composite(const FrameDev& f, int mode, void* out, const float4& bg, cudaStream_t s) {
    if (f.screen_count == 0) return;
    if (mode == 0) { count_launch(); k_composite<0><<<f.screen_count, kCompThreads, 0, s>>>(f, out, bg); }
    else if (mode == 1) { count_launch(); k_composite<1><<<f.screen_count, kCompThreads, 0, s>>>(f, out, bg); }
    else { count_launch(); k_composite<2><<<f.screen_count, kCompThreads, 0, s>>>(f, out, bg); }
}

// ---------------------------------------------------------------------------
// readback of raw alpha masks and resolved tile coverage (parity checks)
// ---------------------------------------------------------------------------
__global__ void k_alpha_masks(FrameDev f, float* out) {
    __shared__ CovBuf bufs[8];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint64_t A = f.counters->alpha_tiles;
    uint32_t a = blockIdx.x * 8 + wid;
    if (a >= A) return;
    warp_accumulate_tile(f, a, bufs[wid]);
    __syncwarp();
    for (int k = lane; k < 256; k += 32) out[(uint64_t)a * 256 + k] = buf_value(bufs[wid], k & 15, k >> 4);
}

__global__ void k_tile_cov(FrameDev f, float* out) {
    __shared__ CovBuf bufs[8][2];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint64_t T = f.counters->tiles;
    uint32_t g = blockIdx.x * 8 + wid;
    if (g >= T) return;
    int4 rec = f.tiles[g];
    uint32_t gp = path_of_tile(f, g);
    uint32_t ctrl = ((uint32_t)rec.w >> 16) & 0xffu;
    bool even_odd = (ctrl & 0x2u) != 0;
    int8_t bd = tile_backdrop(rec);
    bool combine = false;
    int4 crec = make_int4(0, 0, 0, 0);
    if (!f.path.is_clip[gp] && f.path.clip_gpath[gp] >= 0) {
        crec = f.clips[g];
        combine = (uint32_t)crec.x != kInvalid && (uint32_t)crec.z != kInvalid;
    }
    if (combine) {
        warp_accumulate_tile(f, (uint32_t)crec.x, bufs[wid][0]);
        warp_accumulate_tile(f, (uint32_t)crec.z, bufs[wid][1]);
    } else if ((uint32_t)rec.y != kInvalid) {
        warp_accumulate_tile(f, (uint32_t)rec.y, bufs[wid][0]);
    }
    __syncwarp();
    for (int k = lane; k < 256; k += 32) {
        int x = k & 15, y = k >> 4;
        float c;
        if (combine) {
            float mm = fminf(fabsf(buf_value(bufs[wid][0], x, y) + (float)crec.y),
                             fabsf(buf_value(bufs[wid][1], x, y) + (float)crec.w));
            c = resolve_coverage(mm + (float)bd, even_odd);
        } else if ((uint32_t)rec.y != kInvalid) {
            c = resolve_coverage(buf_value(bufs[wid][0], x, y) + (float)bd, even_odd);
        } else {
            c = resolve_coverage((float)bd, even_odd);
        }
        out[(uint64_t)g * 256 + k] = c;
    }
}

void launch_masks(const FrameDev& f, float* alpha_masks, float* tile_cov, cudaStream_t s) {
    if (alpha_masks) { count_launch(); k_alpha_masks<<<(f.tile_cap + 7) / 8 + 1, 256, 0, s>>>(f, alpha_masks); }
    if (tile_cov) { count_launch(); k_tile_cov<<<(f.tile_cap + 7) / 8 + 1, 256, 0, s>>>(f, tile_cov); }
}

}  // namespace pf

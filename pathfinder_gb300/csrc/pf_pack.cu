// pf_pack.cu — scene packing at upload, on the device.
//
// The reference walks its paths on the CPU when it builds a scene: per draw
// path its paint, fill rule, blend mode and clip
// (SceneBuilder::prepare_draw_path_for_gpu_binning, renderer/src/builder.rs:1058-1094;
// prepare_clip_path_for_gpu_binning, renderer/src/builder.rs:1181-1204), and per
// path the contours it packs into the segment buffers (SegmentsD3D11::add_path,
// renderer/src/builder.rs:804-830). Here the caller's path records go to the
// device as they are and these kernels build the per-path tables, the contour
// order and the clip-chain facts from them, so that an upload costs the host
// O(scenes) work rather than O(paths). Invalid records and indices are
// reported through PackInfo::status and the upload is refused; every index a
// later kernel reads is clamped in range first, so a refused upload reads and
// writes nothing out of bounds.

#include "pf_kernels.cuh"
#include "../../include/pathfinder_cuda.h"

namespace pf {

namespace {

// The scene holding global index i of a per-scene ranged array: the last
// scene whose base is <= i (scenes with nothing in the array share their
// base with the next scene and are skipped by taking the last).
template <typename Base>
__device__ __forceinline__ uint32_t scene_at(const ScenePackDev* __restrict__ sc, uint32_t n, uint32_t i, Base base) {
    uint32_t lo = 0, hi = n;  // first scene with base > i is in [lo, hi]
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (base(sc[mid]) <= i) lo = mid + 1;
        else hi = mid;
    }
    return lo > 0 ? lo - 1 : 0;
}

__global__ void k_pack_starts(const uint32_t* __restrict__ raw, uint32_t* __restrict__ starts,
                              const ScenePackDev* __restrict__ sc, uint32_t nsc, uint32_t nb, uint32_t point_total,
                              PackInfo* info) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j > nb) return;
    if (j == nb) {  // the end of the last contour of the batch
        starts[j] = point_total;
        return;
    }
    const uint32_t k = scene_at(sc, nsc, j, [](const ScenePackDev& s) { return s.contour_base; });
    const ScenePackDev s = sc[k];
    const uint32_t c = j - s.contour_base;  // boundary c of the scene: 0..contour_count
    const uint32_t v = raw[j];
    // contour c owns [v, next): ordered and inside the scene's points
    bool bad = c < s.contour_count && (v > raw[j + 1] || raw[j + 1] > s.point_count);
    if (c == s.contour_count && s.contour_count > 0 && v > s.point_count) bad = true;
    if (bad) atomicOr(&info->status, kStatusMalformed);
    starts[j] = s.point_base + (bad ? 0u : (v > s.point_count ? 0u : v));
}

// The tables of path gp; returns its contour references (0 when invalid).
__device__ uint32_t pack_path(const PFCUDAPath* __restrict__ paths, uint32_t gp, const ScenePackDev* __restrict__ sc,
                              uint32_t nsc, const uint8_t* __restrict__ overlay_opaque, const PathTablesDev& t,
                              PackInfo* info) {
    const uint32_t k = scene_at(sc, nsc, gp, [](const ScenePackDev& s) { return s.first_path; });
    const ScenePackDev s = sc[k];
    const uint32_t i = gp - s.first_path;
    const bool c = i < s.nclip;
    const PFCUDAPath p = paths[gp];
    bool bad = (uint64_t)p.first_contour + p.contour_count > s.contour_count;
    bad = bad || p.fill_rule > 1 || p.blend_mode >= PF_BLEND_MODE_COUNT;
    bad = bad || (!c && p.overlay > s.overlay_count);
    bad = bad || (p.clip_path >= 0 && (uint32_t)p.clip_path >= s.nclip);
    bad = bad || (c && p.clip_path == (int32_t)i);  // a clip path clipping itself
    if (bad) atomicOr(&info->status, kStatusMalformed);
    const uint32_t refs = bad ? 0u : p.contour_count;
    t.ncont[gp] = refs;
    t.paint[gp] = (uint32_t)p.paint.r | ((uint32_t)p.paint.g << 8) | ((uint32_t)p.paint.b << 16) |
                  ((uint32_t)p.paint.a << 24);
    t.local[gp] = c ? i : i - s.nclip;
    t.scene_of[gp] = k;
    t.clip[gp] = (!bad && p.clip_path >= 0) ? (int32_t)(s.first_path + (uint32_t)p.clip_path) : -1;
    t.rule[gp] = bad ? 0 : p.fill_rule;
    t.is_clip[gp] = c ? 1 : 0;
    if (c) {
        t.draw_index[gp] = kInvalid;
        t.blend[gp] = 0;
        t.overlay[gp] = 0;
        t.occludes[gp] = 0;
        return refs;
    }
    const uint32_t d = s.draw_base + (i - s.nclip);
    const uint32_t blend = bad ? 0u : p.blend_mode;
    const uint32_t ov = (bad || p.overlay == 0) ? 0u : s.overlay_base + p.overlay;  // global overlay + 1
    t.draw_index[gp] = d;
    t.alpha[d] = (float)p.paint.a / 255.0f;
    t.blend[gp] = (uint8_t)blend;
    t.overlay[gp] = ov;
    // BuiltDrawPath::occludes (renderer/src/builder.rs:80-94): opaque paint and
    // BlendMode::occludes_backdrop (content/src/effects.rs:202-230)
    const bool opaque = p.paint.a == 255 && (ov == 0 || overlay_opaque[ov - 1]);
    t.occludes[gp] = (opaque && (blend == PF_BLEND_MODE_SRC_OVER || blend == PF_BLEND_MODE_CLEAR)) ? 1 : 0;
    if (blend != PF_BLEND_MODE_SRC_OVER) atomicOr(&info->flags, kPackBlendModes);
    return refs;
}

// One thread per path (blocks of whole warps: the reference total is summed per warp).
__global__ void k_pack_paths(const PFCUDAPath* __restrict__ paths, uint32_t P, const ScenePackDev* __restrict__ sc,
                             uint32_t nsc, const uint8_t* __restrict__ overlay_opaque, PathTablesDev t,
                             PackInfo* info) {
    const uint32_t gp = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long refs = gp < P ? pack_path(paths, gp, sc, nsc, overlay_opaque, t, info) : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) refs += __shfl_down_sync(0xffffffffu, refs, o);
    if ((threadIdx.x & 31) == 0 && refs) atomicAdd((unsigned long long*)&info->refs, refs);
}

// One warp per path: its contour references in path order.
// Each path writes its own validated count of references (a total past 2^32
// would wrap first_ord; the host refuses that upload, and no write leaves cap).
__global__ void k_pack_order(const PFCUDAPath* __restrict__ paths, uint32_t P, const ScenePackDev* __restrict__ sc,
                             const uint32_t* __restrict__ scene_of, const uint32_t* __restrict__ ncont,
                             const uint32_t* __restrict__ first_ord, uint32_t cap, uint32_t* __restrict__ ord_contour,
                             uint32_t* __restrict__ ord_path) {
    const uint32_t gp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    if (gp >= P) return;
    const uint32_t a = first_ord[gp], n = ncont[gp];  // 0 for an invalid record
    const uint32_t base = sc[scene_of[gp]].contour_base + paths[gp].first_contour;
    for (uint32_t q = lane; q < n; q += 32) {
        const uint64_t o = (uint64_t)a + q;
        if (o >= cap) break;
        ord_contour[o] = base + q;
        ord_path[o] = gp;
    }
}

// Clip chains (a clip path clipped by another, the D3D11 level's clip levels,
// renderer/src/builder.rs:1124-1220): a chain longer than the scene's clip
// paths is a cycle.
__global__ void k_pack_chains(const int32_t* __restrict__ clip, const uint8_t* __restrict__ is_clip,
                              const uint32_t* __restrict__ scene_of, const ScenePackDev* __restrict__ sc,
                              uint32_t P, PackInfo* info) {
    const uint32_t gp = blockIdx.x * blockDim.x + threadIdx.x;
    if (gp >= P) return;
    const uint32_t nclip = sc[scene_of[gp]].nclip;
    uint32_t len = 0;
    for (int32_t q = clip[gp]; q >= 0; q = clip[(uint32_t)q]) {
        if (++len > nclip) {
            atomicOr(&info->status, kStatusMalformed);
            break;
        }
    }
    if (len) atomicMax(&info->chain_max, len);
    if (is_clip[gp] && clip[gp] >= 0) atomicOr(&info->flags, kPackNestedClips);
}

__global__ void k_pack_ranges(const ScenePackDev* __restrict__ sc, uint32_t nsc, const uint32_t* __restrict__ first_ord,
                              const uint32_t* __restrict__ seg_base, const uint64_t* d_nord, uint32_t cap,
                              uint32_t* __restrict__ ranges) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nsc) return;
    const uint64_t nord = *d_nord;
    const uint32_t n = nord < cap ? (uint32_t)nord : cap;  // seg_base holds n + 1 entries
    const ScenePackDev s = sc[k];
    const uint32_t a = min(first_ord[s.first_path], n), b = min(first_ord[s.first_path + s.nclip + s.ndraw], n);
    ranges[2 * k] = seg_base[a];
    ranges[2 * k + 1] = seg_base[b];
}

inline uint32_t blocks_for(uint64_t threads, uint32_t per_block) {
    return (uint32_t)((threads + per_block - 1) / per_block);
}

}  // namespace

void launch_pack_starts(const uint32_t* raw, uint32_t* starts, const ScenePackDev* scenes, uint32_t scene_count,
                        uint32_t boundary_count, uint32_t point_total, PackInfo* info, cudaStream_t s) {
    count_launch();
    k_pack_starts<<<blocks_for((uint64_t)boundary_count + 1, 256), 256, 0, s>>>(raw, starts, scenes, scene_count,
                                                                               boundary_count, point_total, info);
}

void launch_pack_paths(const PFCUDAPath* paths, uint32_t path_count, const ScenePackDev* scenes,
                       uint32_t scene_count, const uint8_t* overlay_opaque, const PathTablesDev& t, PackInfo* info,
                       cudaStream_t s) {
    if (path_count == 0) return;
    count_launch();
    k_pack_paths<<<blocks_for(path_count, 256), 256, 0, s>>>(paths, path_count, scenes, scene_count, overlay_opaque, t,
                                                            info);
}

void launch_pack_order(const PFCUDAPath* paths, uint32_t path_count, const ScenePackDev* scenes,
                       const uint32_t* scene_of, const uint32_t* ncont, const uint32_t* first_ord, uint32_t cap,
                       uint32_t* ord_contour, uint32_t* ord_path, cudaStream_t s) {
    if (path_count == 0) return;
    count_launch();
    k_pack_order<<<blocks_for((uint64_t)path_count * 32, 256), 256, 0, s>>>(paths, path_count, scenes, scene_of, ncont,
                                                                           first_ord, cap, ord_contour, ord_path);
}

void launch_pack_chains(const int32_t* clip, const uint8_t* is_clip, const uint32_t* scene_of,
                        const ScenePackDev* scenes, uint32_t path_count, PackInfo* info, cudaStream_t s) {
    if (path_count == 0) return;
    count_launch();
    k_pack_chains<<<blocks_for(path_count, 256), 256, 0, s>>>(clip, is_clip, scene_of, scenes, path_count, info);
}

void launch_pack_ranges(const ScenePackDev* scenes, uint32_t scene_count, const uint32_t* first_ord,
                        const uint32_t* seg_base, const uint64_t* d_nord, uint32_t cap, uint32_t* ranges,
                        cudaStream_t s) {
    if (scene_count == 0) return;
    count_launch();
    k_pack_ranges<<<blocks_for(scene_count, 128), 128, 0, s>>>(scenes, scene_count, first_ord, seg_base, d_nord, cap,
                                                              ranges);
}

}  // namespace pf

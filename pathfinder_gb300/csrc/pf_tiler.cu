// pf_tiler.cu — scene packing, bound, and the two tiling passes of the CUDA
// level.  Built with -fmad=false: the tiling arithmetic must match the
// reference CPU tiler bit for bit (see pf_device.cuh).
//
// Stage map (reference -> here):
//   SegmentsD3D11::add_path (renderer/src/builder.rs:804-841) and
//   ContourIter::next (content/src/outline.rs:1024-1065)  -> k_contour_seg*
//   Tiler::new bounds / BuiltPath::new tile rect
//   (renderer/src/tiler.rs:40-66, builder.rs:415-485)     -> k_bound, path scans
//   process_segment (tiler.rs:166-184)                     -> k_flatten_count, k_flatten_emit
//   process_line_segment/add_fill/adjust_alpha_tile_backdrop
//   (tiler.rs:191-308, builder.rs:509-616)                 -> k_bin_count, k_bin_emit
#include "pf_kernels.cuh"

#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

namespace pf {

static std::atomic<uint64_t> g_launches{0};
uint64_t launch_counter() { return g_launches.load(); }
void count_launch(uint32_t n) { g_launches += n; }
bool& pdl_switch() { static thread_local bool on = false; return on; }

int resident_blocks_of(const void* kernel, int threads) {
    struct Entry { int dev; const void* kernel; int threads, blocks; };
    static std::mutex m;
    static std::vector<Entry> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    std::lock_guard<std::mutex> g(m);
    for (const Entry& e : cache)
        if (e.dev == dev && e.kernel == kernel && e.threads == threads) return e.blocks;
    int v = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kernel, threads, 0) != cudaSuccess || v <= 0) v = 1;
    cache.push_back(Entry{dev, kernel, threads, v});
    return v;
}

uint32_t device_sm_count() {
    constexpr int kMaxDevices = 64;
    static std::atomic<uint32_t> cache[kMaxDevices] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 1;
    uint32_t v = cache[dev].load(std::memory_order_relaxed);
    if (v) return v;
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 1;
    cache[dev].store((uint32_t)n, std::memory_order_relaxed);
    return (uint32_t)n;
}

// ---------------------------------------------------------------------------
// warp / block scan helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t warp_inclusive_scan(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Exclusive block scan for blockDim.x == NT (multiple of 32); returns the
// block total in *total.
template <int NT>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[NT / 32];
    __shared__ uint32_t block_total;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t inc = warp_inclusive_scan(v);
    if (lane == 31) warp_sums[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = lane < NT / 32 ? warp_sums[lane] : 0;
        uint32_t si = warp_inclusive_scan(s);
        if (lane < NT / 32) warp_sums[lane] = si - s;
        if (lane == NT / 32 - 1) block_total = si;
    }
    __syncthreads();
    uint32_t r = inc - v + warp_sums[wid];
    *total = block_total;
    __syncthreads();
    return r;
}

// Sum over the block (blockDim.x == NT), valid in thread 0.
template <int NT>
__device__ __forceinline__ uint32_t block_sum(uint32_t v) {
    __shared__ uint32_t warp_part[NT / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) warp_part[wid] = v;
    __syncthreads();
    uint32_t t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < NT / 32; w++) t += warp_part[w];
    __syncthreads();  // the next call reuses warp_part
    return t;
}

// The sum of v over the block, in every thread.
template <int NT>
__device__ __forceinline__ uint32_t block_sum_all(uint32_t v) {
    __shared__ uint32_t sum;
    const uint32_t t = block_sum<NT>(v);
    if (threadIdx.x == 0) sum = t;
    __syncthreads();
    const uint32_t r = sum;
    __syncthreads();  // the next call rewrites `sum`
    return r;
}

// ---------------------------------------------------------------------------
// generic exclusive scan (reduce, scan partials, down-sweep)
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 256, kScanItems = 8, kScanChunk = kScanThreads * kScanItems;

// Element count: the device-side total clamped to the buffer capacity (an
// overflowing frame is flagged elsewhere and re-run), or the host count.
__device__ __forceinline__ uint32_t scan_count(const uint64_t* d_n, uint32_t n_host) {
    if (!d_n) return n_host;
    uint64_t n = *d_n;
    return n < (uint64_t)n_host ? (uint32_t)n : n_host;
}

__device__ __forceinline__ uint32_t scan_in(const uint32_t* in, uint32_t i, uint32_t n, int mode) {
    if (i >= n) return 0;
    uint32_t v = in[i];
    return mode == 1 ? (v != 0u ? 1u : 0u) : v;
}

// A thread's kScanItems consecutive values from `first` (a multiple of
// kScanItems): two 16-byte accesses when the run lies inside [0, n) and the
// array is 16-byte aligned, else one value at a time.
static_assert(kScanItems == 8, "load8 / store8 move eight values");
__device__ __forceinline__ void load8(const uint32_t* in, uint32_t first, uint32_t n, int mode, uint32_t (&v)[8]) {
    if (first + 8 <= n && ((uintptr_t)in & 15u) == 0) {
        const uint4 a = *reinterpret_cast<const uint4*>(in + first);
        const uint4 b = *reinterpret_cast<const uint4*>(in + first + 4);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
        if (mode == 1) {
#pragma unroll
            for (int k = 0; k < 8; k++) v[k] = v[k] != 0u ? 1u : 0u;
        }
    } else {
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = scan_in(in, first + k, n, mode);
    }
}

__device__ __forceinline__ void store8(uint32_t* out, uint32_t first, uint32_t n, const uint32_t (&e)[8]) {
    if (first + 8 <= n && ((uintptr_t)out & 15u) == 0) {
        *reinterpret_cast<uint4*>(out + first) = make_uint4(e[0], e[1], e[2], e[3]);
        *reinterpret_cast<uint4*>(out + first + 4) = make_uint4(e[4], e[5], e[6], e[7]);
    } else {
#pragma unroll
        for (int k = 0; k < 8; k++)
            if (first + k < n) out[first + k] = e[k];
    }
}

__global__ void k_scan_reduce(const uint32_t* __restrict__ in, const uint64_t* d_n, uint32_t n_host, int mode,
                              uint32_t* __restrict__ partials) {
    pdl_enter();
    uint32_t n = scan_count(d_n, n_host);
    uint32_t base = blockIdx.x * kScanChunk;
    if (base >= n) return;
    uint32_t v[kScanItems], s = 0;
    load8(in, base + threadIdx.x * kScanItems, n, mode, v);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) s += v[k];
    const uint32_t total = block_sum<kScanThreads>(s);
    if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

__global__ void k_scan_partials(uint32_t* partials, const uint64_t* d_n, uint32_t n_host, uint32_t* out,
                                uint64_t* total_out) {
    pdl_enter();
    uint32_t n = scan_count(d_n, n_host);
    uint32_t nb = (n + kScanChunk - 1) / kScanChunk;
    uint32_t carry = 0;
    for (uint32_t b0 = 0; b0 < nb; b0 += 1024) {
        uint32_t i = b0 + threadIdx.x;
        uint32_t v = i < nb ? partials[i] : 0;
        uint32_t total;
        uint32_t ex = block_exclusive_scan<1024>(v, &total);
        if (i < nb) partials[i] = ex + carry;
        carry += total;
    }
    if (threadIdx.x == 0) {
        out[n] = carry;
        if (total_out) *total_out = carry;
    }
}

__global__ void k_scan_down(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, const uint64_t* d_n,
                            uint32_t n_host, int mode, const uint32_t* __restrict__ partials) {
    pdl_enter();
    uint32_t n = scan_count(d_n, n_host);
    uint32_t base = blockIdx.x * kScanChunk;
    if (base >= n) return;
    // each thread owns kScanItems consecutive items
    uint32_t v[kScanItems];
    uint32_t s = 0;
    uint32_t first = base + threadIdx.x * kScanItems;
    load8(in, first, n, mode, v);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) s += v[k];
    uint32_t total;
    uint32_t ex = block_exclusive_scan<kScanThreads>(s, &total) + partials[blockIdx.x];
    uint32_t e[kScanItems];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        e[k] = ex;
        ex += v[k];
    }
    store8(out, first, n, e);
}

// ---------------------------------------------------------------------------
// single-pass scans (decoupled look-back): a block scans its 2,048-value tile,
// publishes the tile's sum (kTileAggregate), takes the sum of everything
// before it from its predecessors' words back to the nearest running total
// (kTileInclusive), publishes its own running total and writes its outputs.
// Blocks take their tile from a ticket in the order they start, so every
// predecessor has started and publishes its sum before it looks back itself:
// the waits end.  They are bounded all the same (kStatusScanStall).
// ---------------------------------------------------------------------------
constexpr unsigned long long kTileAggregate = 1ull << 62, kTileInclusive = 2ull << 62;
constexpr unsigned long long kTileValue = (1ull << 62) - 1ull;
constexpr uint32_t kLookBackLimit = 1u << 22;

__device__ __forceinline__ unsigned long long load_tile_word(const unsigned long long* p) {
    return *reinterpret_cast<const volatile unsigned long long*>(p);
}
__device__ __forceinline__ void store_tile_word(unsigned long long* p, unsigned long long v) {
    *reinterpret_cast<volatile unsigned long long*>(p) = v;
}

// Exclusive prefix of tile t whose sum is `sum` (one warp; every lane gets it).
__device__ __forceinline__ unsigned long long look_back(unsigned long long* words, uint32_t t, unsigned long long sum,
                                                        uint32_t* status) {
    const uint32_t lane = threadIdx.x & 31;
    if (lane == 0) store_tile_word(&words[t], kTileAggregate | sum);
    unsigned long long prefix = 0;
    uint32_t j = t;  // tiles [0, j) are still to add
    uint32_t polls = 0;
    while (j > 0) {
        const unsigned long long w = lane < j ? load_tile_word(&words[j - 1 - lane]) : kTileInclusive;
        const uint32_t incl = __ballot_sync(0xffffffffu, (w & ~kTileValue) == kTileInclusive);
        const uint32_t none = __ballot_sync(0xffffffffu, (w & ~kTileValue) == 0ull);
        const int first = incl ? __ffs(incl) - 1 : 32;  // the nearest running total
        const uint32_t span = first < 31 ? (2u << first) - 1u : 0xffffffffu;
        if (none & span) {  // a predecessor has not published yet
            if (++polls >= kLookBackLimit) {
                if (lane == 0 && status) atomicOr(status, kStatusScanStall);
                break;
            }
            continue;
        }
        unsigned long long v = ((span >> lane) & 1u) ? (w & kTileValue) : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        prefix += v;
        if (first < 32) break;
        j -= 32;
    }
    if (lane == 0) store_tile_word(&words[t], kTileInclusive | ((prefix + sum) & kTileValue));
    return prefix;
}

// NL lanes of the same length; lb[0] is the ticket, lane l's tile words
// start at lb + 1 + l * nb.
template <int NL>
__global__ void __launch_bounds__(kScanThreads) k_scan_onepass(ScanLanes L, const uint64_t* d_n, uint32_t n_cap,
                                                               unsigned long long* lb, uint32_t nb, uint32_t* status) {
    pdl_enter();
    __shared__ uint32_t tile_sh;
    __shared__ unsigned long long prefix_sh;
    if (threadIdx.x == 0) tile_sh = atomicAdd(reinterpret_cast<unsigned int*>(lb), 1u);
    __syncthreads();
    const uint32_t t = tile_sh;
    const uint32_t n = scan_count(d_n, n_cap);
    const uint32_t tiles = (n + kScanChunk - 1) / kScanChunk;
    if (t >= (tiles ? tiles : 1u)) return;  // (n == 0: tile 0 writes the zero totals)
    const uint32_t first = t * kScanChunk + threadIdx.x * kScanItems;
#pragma unroll
    for (int l = 0; l < NL; l++) {
        uint32_t v[kScanItems], s = 0;
        load8(L.in[l], first, n, L.mode[l], v);
#pragma unroll
        for (int k = 0; k < kScanItems; k++) s += v[k];
        uint32_t total;
        uint32_t ex = block_exclusive_scan<kScanThreads>(s, &total);
        if (threadIdx.x < 32) {
            const unsigned long long p = look_back(lb + 1 + (size_t)l * nb, t, total, status);
            if (threadIdx.x == 0) prefix_sh = p;
        }
        __syncthreads();
        const unsigned long long p = prefix_sh;
        ex += (uint32_t)p;
        uint32_t e[kScanItems];
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            e[k] = ex;
            ex += v[k];
        }
        store8(L.out[l], first, n, e);
        if (L.incl[l]) {
#pragma unroll
            for (int k = 0; k < kScanItems; k++) e[k] += v[k];
            store8(L.incl[l], first, n, e);
        }
        if (threadIdx.x == 0 && t + 1 >= tiles) {  // the last tile: the total
            L.out[l][n] = (uint32_t)(p + total);
            if (L.total[l]) *L.total[l] = p + total;
        }
        __syncthreads();  // prefix_sh is reused by the next lane
    }
}

// The single-pass form when the scratch has a look-back region with room and
// the scan has at most kOnePassTiles tiles: on longer scans every block is
// resident at once, and each walks back over many predecessors whose running
// totals are not known yet (the three-pass form is faster there).
constexpr uint32_t kOnePassTiles = 64;
template <int NL>
static bool launch_scan_onepass(const ScanLanes& lanes, const uint64_t* d_n, uint32_t n_cap, ScanTemp& tmp,
                                cudaStream_t s) {
    uint32_t nb = (n_cap + kScanChunk - 1) / kScanChunk;
    if (nb == 0) nb = 1;
    if (nb > kOnePassTiles) return false;
    const uint64_t words = 1 + (uint64_t)NL * nb;
    if (!tmp.lookback || tmp.lookback_used + words > tmp.lookback_cap) return false;
    unsigned long long* lb = tmp.lookback + tmp.lookback_used;
    tmp.lookback_used += (uint32_t)words;
    count_launch();
    pdl_launch(k_scan_onepass<NL>, nb, kScanThreads, 0, s, lanes, d_n, n_cap, lb, nb, tmp.status);
    return true;
}

template <int NL>
__global__ void k_scanm_reduce(ScanLanes L, const uint64_t* d_n, uint32_t n_cap, uint32_t* __restrict__ partials);
template <int NL>
__global__ void k_scanm_down_fused(ScanLanes L, const uint64_t* d_n, uint32_t n_cap,
                                   const uint32_t* __restrict__ partials);
constexpr uint32_t kFusedScanBlocks = 2048;  // the most blocks a two-launch scan takes

void launch_scan(const uint32_t* in, uint32_t* out, const uint64_t* d_n, uint32_t n_host, uint32_t n_cap, int mode,
                 uint64_t* total_out, ScanTemp& tmp, cudaStream_t s) {
    uint32_t nb = (n_cap + kScanChunk - 1) / kScanChunk;
    if (nb == 0) nb = 1;
    if (d_n) n_host = n_cap;  // device count is clamped to the capacity
    {
        ScanLanes one{};
        one.count = 1;
        one.in[0] = in; one.out[0] = out; one.total[0] = total_out; one.mode[0] = mode;
        if (launch_scan_onepass<1>(one, d_n, n_host, tmp, s)) return;
    }
    if (nb <= kFusedScanBlocks) {  // reduce, then down-sweeps that sum their own prefixes
        ScanLanes one{};
        one.count = 1;
        one.in[0] = in; one.out[0] = out; one.total[0] = total_out; one.mode[0] = mode;
        { count_launch(); pdl_launch(k_scanm_reduce<1>, nb, kScanThreads, 0, s, one, d_n, n_host, tmp.partials); }
        { count_launch(); pdl_launch(k_scanm_down_fused<1>, nb, kScanThreads, 0, s, one, d_n, n_host, tmp.partials); }
        return;
    }
    { count_launch(); pdl_launch(k_scan_reduce, nb, kScanThreads, 0, s, in, d_n, n_host, mode, tmp.partials); }
    { count_launch(); pdl_launch(k_scan_partials, 1, 1024, 0, s, tmp.partials, d_n, n_host, out, total_out); }
    { count_launch(); pdl_launch(k_scan_down, nb, kScanThreads, 0, s, in, out, d_n, n_host, mode, tmp.partials); }
}

cudaError_t launch_scan_checked(const uint32_t* in, uint32_t* out, uint32_t n, ScanTemp& tmp, cudaStream_t s) {
    uint32_t nb = (n + kScanChunk - 1) / kScanChunk;
    if (nb == 0) nb = 1;
    const uint64_t* d_n = nullptr;
    uint64_t* total_out = nullptr;
    int mode = 0;
    uint32_t* partials = tmp.partials;
    void* a_reduce[] = {(void*)&in, (void*)&d_n, (void*)&n, (void*)&mode, (void*)&partials};
    void* a_part[] = {(void*)&partials, (void*)&d_n, (void*)&n, (void*)&out, (void*)&total_out};
    void* a_down[] = {(void*)&in, (void*)&out, (void*)&d_n, (void*)&n, (void*)&mode, (void*)&partials};
    cudaError_t e;
    count_launch(3);
    if ((e = cudaLaunchKernel((const void*)k_scan_reduce, dim3(nb), dim3(kScanThreads), a_reduce, 0, s))) return e;
    if ((e = cudaLaunchKernel((const void*)k_scan_partials, dim3(1), dim3(1024), a_part, 0, s))) return e;
    return cudaLaunchKernel((const void*)k_scan_down, dim3(nb), dim3(kScanThreads), a_down, 0, s);
}

// ---------------------------------------------------------------------------
// fused scans: up to kMaxScanLanes arrays of the same length in one
// reduce / partials / down-sweep set (the per-tile fill offsets, alpha ids and
// column backdrop prefixes share their length)
// ---------------------------------------------------------------------------
// NL lanes, indexed at compile time (a runtime lane index would copy the
// lane table to local memory).
template <int NL>
__global__ void k_scanm_reduce(ScanLanes L, const uint64_t* d_n, uint32_t n_cap, uint32_t* __restrict__ partials) {
    pdl_enter();
    const uint32_t n = scan_count(d_n, n_cap);
    const uint32_t base = blockIdx.x * kScanChunk;
    if (base >= n) return;
    const uint32_t nb = (n_cap + kScanChunk - 1) / kScanChunk;
#pragma unroll
    for (int l = 0; l < NL; l++) {
        uint32_t v[kScanItems], s = 0;
        load8(L.in[l], base + threadIdx.x * kScanItems, n, L.mode[l], v);
#pragma unroll
        for (int k = 0; k < kScanItems; k++) s += v[k];
        const uint32_t total = block_sum<kScanThreads>(s);
        if (threadIdx.x == 0) partials[l * nb + blockIdx.x] = total;
    }
}

template <int NL>
__global__ void k_scanm_partials(ScanLanes L, const uint64_t* d_n, uint32_t n_cap, uint32_t* partials) {
    pdl_enter();
    const uint32_t n = scan_count(d_n, n_cap);
    const uint32_t nb = (n + kScanChunk - 1) / kScanChunk, nbc = (n_cap + kScanChunk - 1) / kScanChunk;
#pragma unroll
    for (int l = 0; l < NL; l++) {
        uint32_t carry = 0;
        uint32_t* p = partials + l * nbc;
        for (uint32_t b0 = 0; b0 < nb; b0 += 1024) {
            uint32_t i = b0 + threadIdx.x;
            uint32_t v = i < nb ? p[i] : 0;
            uint32_t total;
            uint32_t ex = block_exclusive_scan<1024>(v, &total);
            if (i < nb) p[i] = ex + carry;
            carry += total;
        }
        if (threadIdx.x == 0) {
            L.out[l][n] = carry;
            if (L.total[l]) *L.total[l] = carry;
        }
    }
}

template <int NL>
__global__ void k_scanm_down(ScanLanes L, const uint64_t* d_n, uint32_t n_cap, const uint32_t* __restrict__ partials) {
    pdl_enter();
    const uint32_t n = scan_count(d_n, n_cap);
    const uint32_t base = blockIdx.x * kScanChunk;
    if (base >= n) return;
    const uint32_t nb = (n_cap + kScanChunk - 1) / kScanChunk;
    const uint32_t first = base + threadIdx.x * kScanItems;
#pragma unroll
    for (int l = 0; l < NL; l++) {
        uint32_t v[kScanItems];
        uint32_t s = 0;
        load8(L.in[l], first, n, L.mode[l], v);
#pragma unroll
        for (int k = 0; k < kScanItems; k++) s += v[k];
        uint32_t total;
        uint32_t ex = block_exclusive_scan<kScanThreads>(s, &total) + partials[l * nb + blockIdx.x];
        uint32_t e[kScanItems];
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            e[k] = ex;
            ex += v[k];
        }
        store8(L.out[l], first, n, e);
        if (L.incl[l]) {
#pragma unroll
            for (int k = 0; k < kScanItems; k++) e[k] += v[k];
            store8(L.incl[l], first, n, e);
        }
    }
}

// Down-sweep that sums its block's prefix from the blocks' partial sums
// itself (each block reads fewer than kFusedScanBlocks of them, from L2), so a
// scan of that many blocks needs no launch that scans the partials.  The
// last block with values writes the totals; with no values, block 0 does.
template <int NL>
__global__ void k_scanm_down_fused(ScanLanes L, const uint64_t* d_n, uint32_t n_cap,
                                   const uint32_t* __restrict__ partials) {
    pdl_enter();
    const uint32_t n = scan_count(d_n, n_cap);
    const uint32_t base = blockIdx.x * kScanChunk;
    const uint32_t nbc = (n_cap + kScanChunk - 1) / kScanChunk, nb = (n + kScanChunk - 1) / kScanChunk;
    if (n == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
#pragma unroll
            for (int l = 0; l < NL; l++) {
                L.out[l][0] = 0;
                if (L.total[l]) *L.total[l] = 0;
            }
        }
        return;
    }
    if (base >= n) return;
    const uint32_t first = base + threadIdx.x * kScanItems;
#pragma unroll
    for (int l = 0; l < NL; l++) {
        uint32_t ps = 0;
        for (uint32_t j = threadIdx.x; j < blockIdx.x; j += kScanThreads) ps += partials[l * nbc + j];
        const uint32_t prefix = block_sum_all<kScanThreads>(ps);
        uint32_t v[kScanItems];
        uint32_t sv = 0;
        load8(L.in[l], first, n, L.mode[l], v);
#pragma unroll
        for (int k = 0; k < kScanItems; k++) sv += v[k];
        uint32_t total;
        uint32_t ex = block_exclusive_scan<kScanThreads>(sv, &total) + prefix;
        uint32_t e[kScanItems];
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            e[k] = ex;
            ex += v[k];
        }
        store8(L.out[l], first, n, e);
        if (L.incl[l]) {
#pragma unroll
            for (int k = 0; k < kScanItems; k++) e[k] += v[k];
            store8(L.incl[l], first, n, e);
        }
        if (blockIdx.x == nb - 1 && threadIdx.x == 0) {
            L.out[l][n] = prefix + total;
            if (L.total[l]) *L.total[l] = prefix + total;
        }
    }
}

template <int NL>
static void launch_scan_lanes(const ScanLanes& lanes, const uint64_t* d_n, uint32_t n_cap, ScanTemp& tmp,
                              cudaStream_t s) {
    uint32_t nb = (n_cap + kScanChunk - 1) / kScanChunk;
    if (nb == 0) nb = 1;
    if (nb <= kFusedScanBlocks) {
        { count_launch(); pdl_launch(k_scanm_reduce<NL>, nb, kScanThreads, 0, s, lanes, d_n, n_cap, tmp.partials); }
        { count_launch(); pdl_launch(k_scanm_down_fused<NL>, nb, kScanThreads, 0, s, lanes, d_n, n_cap, tmp.partials); }
        return;
    }
    { count_launch(); pdl_launch(k_scanm_reduce<NL>, nb, kScanThreads, 0, s, lanes, d_n, n_cap, tmp.partials); }
    { count_launch(); pdl_launch(k_scanm_partials<NL>, 1, 1024, 0, s, lanes, d_n, n_cap, tmp.partials); }
    { count_launch(); pdl_launch(k_scanm_down<NL>, nb, kScanThreads, 0, s, lanes, d_n, n_cap, tmp.partials); }
}

void launch_scan_multi(const ScanLanes& lanes, const uint64_t* d_n, uint32_t n_cap, ScanTemp& tmp, cudaStream_t s) {
    if (lanes.count == 1 && launch_scan_onepass<1>(lanes, d_n, n_cap, tmp, s)) return;
    if (lanes.count == 2 && launch_scan_onepass<2>(lanes, d_n, n_cap, tmp, s)) return;
    if (lanes.count == 3 && launch_scan_onepass<3>(lanes, d_n, n_cap, tmp, s)) return;
    if (lanes.count == 1) launch_scan_lanes<1>(lanes, d_n, n_cap, tmp, s);
    else if (lanes.count == 2) launch_scan_lanes<2>(lanes, d_n, n_cap, tmp, s);
    else launch_scan_lanes<3>(lanes, d_n, n_cap, tmp, s);
}

// ---------------------------------------------------------------------------
// transform (Contour::transform, content/src/outline.rs:884-893;
// Transform2F * Vector2F, geometry/src/transform2d.rs:123-129, :312-318)
// ---------------------------------------------------------------------------
__global__ void k_transform(const float2* __restrict__ in, float2* __restrict__ out, uint32_t n, float m00,
                            float m01, float m10, float m11, float vx, float vy) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float2 p = in[i];
        float hx = fmul(m00, p.x), hy = fmul(m10, p.x), hz = fmul(m01, p.y), hw = fmul(m11, p.y);
        out[i] = make_float2(fadd(fadd(hx, hz), vx), fadd(fadd(hy, hw), vy));
    }
}

void launch_transform(const float2* in, float2* out, uint32_t n, const float* m6, cudaStream_t s) {
    if (n == 0) return;
    uint32_t blocks = (n + 255) / 256;
    const uint32_t cap = device_sm_count() * 16;
    if (blocks > cap) blocks = cap;
    { count_launch(); k_transform<<<blocks, 256, 0, s>>>(in, out, n, m6[0], m6[1], m6[2], m6[3], m6[4], m6[5]); }
}

// ---------------------------------------------------------------------------
// segment packing: one warp per contour (in global path order)
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool is_endpoint(const uint8_t* flags, uint32_t i) {
    return (flags[i] & 3u) == 0;
}

__global__ void k_contour_segcount(const uint32_t* __restrict__ ord_contour, const uint64_t* d_n, uint32_t cap,
                                   const uint32_t* __restrict__ starts, uint32_t ncont,
                                   const uint8_t* __restrict__ flags, uint32_t* __restrict__ seg_count,
                                   uint32_t* status) {
    uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= scan_count(d_n, cap)) return;
    uint32_t c = ord_contour[k];
    if (c >= ncont) {
        if (lane == 0) {
            atomicOr(status, kStatusMalformed);
            seg_count[k] = 0;
        }
        return;
    }
    uint32_t a = starts[c], b = starts[c + 1];
    uint32_t n = b > a ? b - a : 0;
    uint32_t count = 0;
    bool bad = false;
    for (uint32_t i0 = 0; i0 < n; i0 += 32) {
        uint32_t i = i0 + lane;
        bool start = i < n && (i == 0 || is_endpoint(flags, a + i));
        if (start && i + 1 < n && !is_endpoint(flags, a + i + 1)) {
            // curve: needs its end point inside the contour
            if (i + 2 >= n) bad = true;
            else if (!is_endpoint(flags, a + i + 2) && i + 3 >= n) bad = true;
        }
        count += __popc(__ballot_sync(0xffffffffu, start));
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(status, kStatusMalformed);
    if (lane == 0) seg_count[k] = count;
}

__global__ void k_contour_segemit(const uint32_t* __restrict__ ord_contour, const uint32_t* __restrict__ ord_path,
                                  const uint64_t* d_n, uint32_t cap, const uint32_t* __restrict__ starts,
                                  uint32_t ncont, const uint8_t* __restrict__ flags,
                                  const uint32_t* __restrict__ seg_base, SegRec* __restrict__ segs) {
    uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= scan_count(d_n, cap)) return;
    uint32_t c = ord_contour[k], gp = ord_path[k];
    if (c >= ncont) return;  // counted as no segments
    uint32_t a = starts[c], b = starts[c + 1];
    uint32_t n = b > a ? b - a : 0;
    uint32_t out = seg_base[k];
    for (uint32_t i0 = 0; i0 < n; i0 += 32) {
        uint32_t i = i0 + lane;
        bool start = i < n && (i == 0 || is_endpoint(flags, a + i));
        uint32_t m = __ballot_sync(0xffffffffu, start);
        if (start) {
            SegRec r;
            r.x = (int)(a + i);
            r.w = (int)gp;
            if (i + 1 >= n) { r.y = (int)a; r.z = (int)kSegLine; }
            else if (is_endpoint(flags, a + i + 1)) { r.y = (int)(a + i + 1); r.z = (int)kSegLine; }
            else if (i + 2 < n && is_endpoint(flags, a + i + 2)) { r.y = (int)(a + i + 2); r.z = (int)kSegQuad; }
            else if (i + 3 < n) { r.y = (int)(a + i + 3); r.z = (int)kSegCubic; }
            else { r.y = (int)a; r.z = (int)kSegLine; }  // malformed (flagged by k_contour_segcount)
            segs[out + __popc(m & ((1u << lane) - 1u))] = r;
        }
        out += __popc(m);
    }
}

void launch_contour_segcount(const uint32_t* ord_contour, const uint64_t* d_n, uint32_t cap, const uint32_t* starts,
                             uint32_t contour_total, const uint8_t* flags, uint32_t* seg_count, uint32_t* status,
                             cudaStream_t s) {
    if (cap == 0) return;
    const uint32_t blocks = (uint32_t)(((uint64_t)cap * 32 + 255) / 256);
    count_launch();
    k_contour_segcount<<<blocks, 256, 0, s>>>(ord_contour, d_n, cap, starts, contour_total, flags, seg_count, status);
}

void launch_contour_segemit(const uint32_t* ord_contour, const uint32_t* ord_path, const uint64_t* d_n, uint32_t cap,
                            const uint32_t* starts, uint32_t contour_total, const uint8_t* flags,
                            const uint32_t* seg_base, SegRec* segs, cudaStream_t s) {
    if (cap == 0) return;
    const uint32_t blocks = (uint32_t)(((uint64_t)cap * 32 + 255) / 256);
    count_launch();
    k_contour_segemit<<<blocks, 256, 0, s>>>(ord_contour, ord_path, d_n, cap, starts, contour_total, flags, seg_base,
                                             segs);
}

// ---------------------------------------------------------------------------
// bound: one warp per path
// ---------------------------------------------------------------------------
__global__ void k_bound(FrameDev f, const uint32_t* __restrict__ ord_contour, const uint32_t* __restrict__ starts) {
    pdl_enter();
    const uint32_t wi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wi >= f.path_count) return;
    const uint32_t gp = f.path_begin + wi;
    float mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
    bool any = false;
    uint32_t k0 = f.path.first_ord_contour[gp], k1 = f.path.first_ord_contour[gp + 1];
    for (uint32_t k = k0; k < k1; k++) {
        uint32_t c = ord_contour[k];
        uint32_t a = starts[c], b = starts[c + 1];
        if (b > a) any = true;
        // four loads in flight per lane; each lane still folds its points
        // in the same order (i, i + 32, i + 64, ...)
        for (uint32_t i = a + lane; i < b; i += 128) {
            float2 p[4];
#pragma unroll
            for (int u = 0; u < 4; u++) p[u] = i + 32u * u < b ? f.pts[i + 32u * u] : make_float2(0.0f, 0.0f);
#pragma unroll
            for (int u = 0; u < 4; u++) {
                if (i + 32u * u >= b) break;
                mnx = smin(mnx, p[u].x); mny = smin(mny, p[u].y);
                mxx = smax(mxx, p[u].x); mxy = smax(mxy, p[u].y);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mnx = smin(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
        mny = smin(mny, __shfl_xor_sync(0xffffffffu, mny, o));
        mxx = smax(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mxy = smax(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
    }
    if (lane != 0) return;
    const SceneDev& sc = f.scenes[f.path.scene[gp]];
    float bx0 = 0.0f, by0 = 0.0f, bx1 = 0.0f, by1 = 0.0f;
    if (any) {
        // RectF::intersection (geometry/src/rect.rs:116-139); default rect when disjoint
        float4 v = sc.view_box;
        if (mnx < v.z && mny < v.w && v.x < mxx && v.y < mxy) {
            bx0 = smax(mnx, v.x); by0 = smax(mny, v.y);
            bx1 = smin(mxx, v.z); by1 = smin(mxy, v.w);
        }
    }
    if (!f.path.is_clip[gp] && blend_is_destructive(f.path.blend[gp])) {
        // a destructive blend mode tiles the whole view box (renderer/src/builder.rs:430-434)
        const float4 v = sc.view_box;
        bx0 = v.x; by0 = v.y; bx1 = v.z; by1 = v.w;
    }
    // round_rect_out_to_tile_bounds (renderer/src/tiles.rs:64-66)
    const float q = 1.0f / 16.0f;
    int4 r;
    r.x = cvt_rne(floorf(fmul(bx0, q))); r.y = cvt_rne(floorf(fmul(by0, q)));
    r.z = cvt_rne(ceilf(fmul(bx1, q)));  r.w = cvt_rne(ceilf(fmul(by1, q)));
    f.path.tile_rect[gp] = r;
    // scan inputs: tiles and above-rect columns of the path (DenseTileMap
    // and backdrops vector of BuiltPath::new, renderer/src/builder.rs:441-456)
    int w = r.z - r.x, h = r.w - r.y;
    f.path_tiles[gp] = (w > 0 && h > 0) ? (uint32_t)w * (uint32_t)h : 0u;
    f.path_cols[gp] = w > 0 ? (uint32_t)w : 0u;
}

void launch_bound(const FrameDev& f, const uint32_t* ord_contour, const uint32_t* starts, cudaStream_t s) {
    if (f.path_count == 0) return;
    uint32_t blocks = (f.path_count * 32 + 255) / 256;
    { count_launch(); pdl_launch(k_bound, blocks, 256, 0, s, f, ord_contour, starts); }
}

// A path's binning context from its tile rect, its scanned offsets and its
// scene's view box.
__device__ __forceinline__ PathCtx path_ctx(const FrameDev& f, uint32_t gp) {
    PathCtx pc;
    int4 r = f.path.tile_rect[gp];
    pc.minx = r.x; pc.miny = r.y; pc.maxx = r.z; pc.maxy = r.w;
    pc.tile_base = f.path.tile_offset[gp];
    pc.col_base = f.path.col_offset[gp];
    float4 v = f.scenes[f.path.scene[gp]].view_box;
    pc.vminx = v.x; pc.vmaxx = v.z; pc.vmaxy = v.w;
    pc.pad[0] = pc.pad[1] = pc.pad[2] = 0u;
    return pc;
}

// Zero the per-tile accumulators and the per-screen-tile z-buffer and counts
// of this frame, and write each path's binning context; block 0 also checks
// the path scans' totals against the capacities (one kernel instead of a
// check kernel and two memsets).
__global__ void k_zero_tiles(FrameDev f) {
    pdl_enter();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < f.path_count; i += gridDim.x * blockDim.x)
        f.path_bin[f.path_begin + i] = path_ctx(f, f.path_begin + i);
    uint64_t T = f.counters->tiles, C = f.counters->columns;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (T > f.tile_cap) {
            atomicOr(&f.counters->status, kStatusTileCapacity);
            f.counters->needed_tiles = T;
        }
        if (C > f.col_cap) atomicOr(&f.counters->status, kStatusColumnCapacity);
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= f.screen_count; i += gridDim.x * blockDim.x) {
        f.zbuf[i] = 0;
        f.screen_cnt[i] = 0;
    }
    if (T > f.tile_cap || C > f.col_cap) return;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < T || i < C;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if (i < T) { f.tile_fill_count[i] = 0; f.tile_delta[i] = 0; }
        if (i < C) f.col_backdrop[i] = 0;
    }
}

void launch_path_scan(const FrameDev& f, ScanTemp& tmp, cudaStream_t s) {
    ScanLanes lanes{};
    lanes.count = 2;
    lanes.in[0] = f.path_tiles + f.path_begin; lanes.out[0] = f.path.tile_offset + f.path_begin;
    lanes.total[0] = &f.counters->tiles;
    lanes.in[1] = f.path_cols + f.path_begin; lanes.out[1] = f.path.col_offset + f.path_begin;
    lanes.total[1] = &f.counters->columns;
    launch_scan_multi(lanes, nullptr, f.path_count, tmp, s);
    { count_launch(); pdl_launch(k_zero_tiles, f.sms * 8, 256, 0, s, f); }
}

// Launch bounds: the ordered flattening passes run at 32 registers a thread
// (64 warps an SM, a few spilled values), the one-pass flattening and the
// binning passes at 40 (48 warps); the extra warps hide their gather and
// atomic latency (measured: 36 or 32 registers spill the binning passes' walk
// state and slow them, and spill the one-pass flattening's line placement).
// ---------------------------------------------------------------------------
// flattening (process_segment's recursion, renderer/src/tiler.rs:166-184).
// Ordered frames write the lines in emission order (input segments in path
// order, each segment's lines depth first); plain frames write each
// segment's lines depth first within its block's ranges (k_flatten_count).
//
// A warp takes 32 segments and tests their subdivision level by level: at
// level d the nodes still to test (children of nodes that were not flat) of
// all 32 segments are spread over the lanes, each lane computing its node
// from the root with exactly the splits the recursion performs.  A flat node
// is a leaf: leaf masks record, on a grid of 2^kLeafLevels parameter slots,
// where each leaf starts, so the count is the mask's population and the
// depth-first order is the order of the slots.  The emit pass spreads the
// leaves of 32 segments over the lanes the same way.  A segment with a node
// still not flat at depth kLeafLevels is flattened by the depth-first walk
// (flatten_segment) instead, by its own lane.
// ---------------------------------------------------------------------------
constexpr int kLeafLevels = 6;
constexpr uint32_t kFlattenMaxWarps = 8;  // flatten_threads <= 256

// Lane owning item i of a warp's items: the first lane whose inclusive count
// exceeds i (incl: the lane's inclusive count).
__device__ __forceinline__ uint32_t warp_owner(uint32_t incl, uint32_t i) {
    uint32_t j = 0;
#pragma unroll
    for (uint32_t step = 16; step > 0; step >>= 1) {
        const uint32_t v = __shfl_sync(0xffffffffu, incl, j + step - 1);
        if (v <= i) j += step;
    }
    return j;
}

// Position of the k-th (from 0) set bit of m; m has more than k set bits.
__device__ __forceinline__ uint32_t nth_set_bit64(unsigned long long m, uint32_t k) {
    uint32_t pos = 0;
#pragma unroll
    for (int w = 32; w >= 1; w >>= 1) {
        const unsigned long long low = m & ((1ull << w) - 1ull);
        const uint32_t c = (uint32_t)__popcll(low);
        if (k >= c) {
            k -= c;
            m >>= w;
            pos += (uint32_t)w;
        } else {
            m = low;
        }
    }
    return pos;
}

struct FlattenWarp {
    Cubic root[32];                    // each lane's segment as a cubic (a line as its base)
    unsigned long long leaves[32];     // leaf start slots of each segment
    unsigned long long next[32];       // nodes of the next level to test
    unsigned long long multi[32];      // leaves whose line crosses a tile boundary (one-pass form)
    uint32_t deep;                     // segments deeper than kLeafLevels
};

// Whether a line reaches beyond the tile of its start (the binning's walk
// takes more than its one-step path for it).  The one-pass flattening places
// such lines apart from the others so that each warp of the binning passes
// mostly walks lines of one kind.
__device__ __forceinline__ bool line_multi_tile(const Line& l) {
    const float r = 1.0f / 16.0f;
    return floorf(l.fx * r) != floorf(l.tx * r) || floorf(l.fy * r) != floorf(l.ty * r);
}

// Line k of a leaf mask: the leaf from its start slot to the next leaf's (or
// the end); its split path and depth.
__device__ __forceinline__ void leaf_of_mask(unsigned long long m, uint32_t k, uint32_t* addr, int* depth) {
    const uint32_t start = nth_set_bit64(m, k);
    const unsigned long long above = start >= 63u ? 0ull : (m >> (start + 1u));
    const uint32_t next = above ? start + (uint32_t)__ffsll((long long)above) : 64u;
    const int d = kLeafLevels - (31 - __clz((int)(next - start)));
    *depth = d;
    *addr = start >> (kLeafLevels - d);
}

// Flattening.  ORDERED (frames whose line order is read: record read-back
// and differentiable frames) is the count pass: leaf masks and line counts
// for the emit pass, which places each segment's lines in depth-first order
// after a scan over the warps.  Otherwise (plain frames, whose later stages
// sum per tile with integer atomics or order by tile, so that no output
// depends on the order of the lines) the same kernel writes the lines: each
// block takes its range of lines within one tile from the front of the line
// array (counter `lines`) and its range of longer lines from the back
// (counter `lines_back`), one atomic each, and places them in depth-first
// order within those ranges, with no scan and no emit pass.
template <bool ORDERED>
__global__ void __launch_bounds__(256, ORDERED ? 8 : 6) k_flatten_count(FrameDev f) {
    pdl_enter();
    // one FlattenWarp per warp of the block, sized at launch (so that blocks
    // of fewer warps hold less shared memory and more of them fit an SM)
    extern __shared__ __align__(16) unsigned char flatten_smem[];
    __shared__ uint32_t warp_base[kFlattenMaxWarps][2];
    __shared__ unsigned long long block_base[2];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    FlattenWarp& w = reinterpret_cast<FlattenWarp*>(flatten_smem)[wib];
    const uint32_t s0 = (blockIdx.x * (blockDim.x >> 5) + wib) * 32u;
    if (ORDERED && s0 >= f.seg_count) return;  // whole warps (the other form's warps meet at barriers)
    const uint32_t s = s0 + lane;
    unsigned long long active = 0;  // nodes of the current level to test
    unsigned long long leaves = 0;
    uint32_t path = 0;
    if (s < f.seg_count) {
        // level 0 by the segment's own lane: a line, or a curve flat as a
        // whole, is one leaf; otherwise both halves are tested at level 1
        Cubic c;
        const SegRec sr = f.segs[f.seg_begin + s];
        const int kind = segment_root(f.pts, sr, c, &f.counters->status);
        path = (uint32_t)sr.w;
        if (kind == kRootLine || (kind == kRootCurve && cubic_is_flat(c))) leaves = 1;
        else if (kind == kRootCurve) active = 3;
        w.root[lane] = c;
    }
    w.leaves[lane] = leaves;
    w.next[lane] = 0;
    if (!ORDERED) w.multi[lane] = (leaves && line_multi_tile(w.root[lane].base)) ? 1ull : 0ull;
    if (lane == 0) w.deep = 0;
    __syncwarp();
    for (int d = 1; d <= kLeafLevels; d++) {
        // the nodes to test come in sibling pairs (both children of a node
        // that was not flat): an item is a pair, its parent recomputed from
        // the root and split once, as the recursion splits it
        const unsigned long long pairs = active & 0x5555555555555555ull;
        const uint32_t cnt = (uint32_t)__popcll(pairs);
        const uint32_t incl = warp_inclusive_scan(cnt);
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        if (total == 0) break;
        for (uint32_t i0 = 0; i0 < total; i0 += 32) {
            const uint32_t i = i0 + lane;
            const uint32_t j = warp_owner(incl, i);
            const uint32_t first = __shfl_sync(0xffffffffu, incl - cnt, j);
            const unsigned long long aj = __shfl_sync(0xffffffffu, pairs, j);
            if (i < total) {
                const uint32_t a0 = nth_set_bit64(aj, i - first);  // the left child's address
                Cubic half[2];
                cubic_split_half(subdivision_node(w.root[j], a0 >> 1, d - 1), half[0], half[1]);
                // both children's bits, then one update of each mask
                unsigned long long leaf_bits = 0, multi_bits = 0, next_bits = 0;
                bool deeper = false;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const uint32_t a = a0 + (uint32_t)h;
                    const Cubic& c = half[h];
                    if (cubic_is_flat(c)) {
                        const unsigned long long bit = 1ull << (a << (kLeafLevels - d));
                        leaf_bits |= bit;
                        if (!ORDERED && line_multi_tile(c.base)) multi_bits |= bit;
                    } else if (d < kLeafLevels) {
                        next_bits |= 3ull << (2u * a);
                    } else {
                        deeper = true;
                    }
                }
                if (leaf_bits) atomicOr(&w.leaves[j], leaf_bits);
                if (multi_bits) atomicOr(&w.multi[j], multi_bits);
                if (next_bits) atomicOr(&w.next[j], next_bits);
                if (deeper) atomicOr(&w.deep, 1u << j);
            }
        }
        __syncwarp();
        active = w.next[lane];
        w.next[lane] = 0;
        __syncwarp();
    }
    uint32_t n = 0, n1 = 0;  // lines, and of those the ones beyond one tile (one-pass form)
    unsigned long long multi = 0;
    const bool deep = s < f.seg_count && ((w.deep >> lane) & 1u);
    if (s < f.seg_count) {
        leaves = w.leaves[lane];
        if (deep) {
            flatten_segment(f.pts, f.segs[f.seg_begin + s], [&](const Line& ln, uint32_t, int) {
                n++;
                if (!ORDERED && line_multi_tile(ln)) n1++;
            }, &f.counters->status);
            leaves = 0;  // no mask: the segment is walked again for its lines
        } else {
            n = (uint32_t)__popcll(leaves);
            if (!ORDERED) {
                multi = w.multi[lane] & leaves;
                n1 = (uint32_t)__popcll(multi);
            }
        }
        if (ORDERED) {
            f.seg_line_count[s] = n;
            f.seg_leaves[s] = leaves;
        }
    }
    if (ORDERED) {
        // the emit pass places the warp's lines after those of the warps
        // before it (a scan of one value per warp)
        const uint32_t warp_lines = __reduce_add_sync(0xffffffffu, n);
        if (lane == 0) f.seg_warp_lines[s0 / 32u] = warp_lines;
        return;
    }
    // the block's two ranges of lines, then each warp's part of them
    const uint32_t n0 = n - n1;
    const uint32_t incl0 = warp_inclusive_scan(n0), incl1 = warp_inclusive_scan(n1);
    if (lane == 31) {
        warp_base[wib][0] = incl0;
        warp_base[wib][1] = incl1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t0 = 0, t1 = 0;
        for (uint32_t k = 0; k < (blockDim.x >> 5); k++) {
            const uint32_t v0 = warp_base[k][0], v1 = warp_base[k][1];
            warp_base[k][0] = t0;
            warp_base[k][1] = t1;
            t0 += v0;
            t1 += v1;
        }
        block_base[0] = t0 ? atomicAdd((unsigned long long*)&f.counters->lines, (unsigned long long)t0) : 0ull;
        block_base[1] = t1 ? atomicAdd((unsigned long long*)&f.counters->lines_back, (unsigned long long)t1) : 0ull;
    }
    __syncthreads();
    if (s0 >= f.seg_count) return;
    // one-tile line r of the segment: front position base0 + r; longer line
    // r: position base1 + r counted down from the end of the array
    const unsigned long long base0 = block_base[0] + warp_base[wib][0] + incl0 - n0;
    const unsigned long long base1 = block_base[1] + warp_base[wib][1] + incl1 - n1;
    auto put = [&](bool far, unsigned long long r, const Line& ln, uint32_t pth) {
        if (r >= f.line_cap) return;
        const unsigned long long l = far ? (unsigned long long)f.line_cap - 1ull - r : r;
        f.lines[l] = make_float4(ln.fx, ln.fy, ln.tx, ln.ty);
        f.line_path[l] = pth;
    };
    // one leaf at level 0: the root's base line, by its own lane
    if (n != 0 && leaves == 1ull) put(multi != 0, multi ? base1 : base0, w.root[lane].base, path);
    // several leaves: the leaves of the warp's segments spread over the lanes
    const uint32_t nl = leaves > 1ull ? n : 0u;
    const uint32_t incl = warp_inclusive_scan(nl);
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    for (uint32_t i0 = 0; i0 < total; i0 += 32) {
        const uint32_t i = i0 + lane;
        const uint32_t j = warp_owner(incl, i);
        const uint32_t k = i - __shfl_sync(0xffffffffu, incl - nl, j);
        const unsigned long long lj = __shfl_sync(0xffffffffu, leaves, j);
        const unsigned long long mj = __shfl_sync(0xffffffffu, multi, j);
        const unsigned long long b0j = __shfl_sync(0xffffffffu, base0, j);
        const unsigned long long b1j = __shfl_sync(0xffffffffu, base1, j);
        const uint32_t pj = __shfl_sync(0xffffffffu, path, j);
        if (i < total) {
            uint32_t addr;
            int d;
            leaf_of_mask(lj, k, &addr, &d);
            // the leaf's rank among the segment's leaves of its kind
            const uint32_t start = addr << (kLeafLevels - d);
            const unsigned long long before = (1ull << start) - 1ull;
            const uint32_t r1 = (uint32_t)__popcll(mj & before);
            const bool far = (mj >> start) & 1ull;
            put(far, far ? b1j + r1 : b0j + (k - r1), subdivision_node(w.root[j], addr, d).base, pj);
        }
    }
    // deeper segments: walked again by their own lanes
    if (deep) {
        unsigned long long r0 = base0, r1 = base1;
        flatten_segment(f.pts, f.segs[f.seg_begin + s], [&](const Line& ln, uint32_t, int) {
            const bool far = line_multi_tile(ln);
            put(far, far ? r1++ : r0++, ln, path);
        }, &f.counters->status);
    }
}

// DIFF also records each line's segment and curve-parameter interval: the leaf
// at split path `addr` of depth d covers t in [addr, addr + 1) / 2^d.  The
// adjoint holds these subdivisions fixed.
template <bool DIFF>
__global__ void __launch_bounds__(256, 8) k_flatten_emit(FrameDev f) {
    pdl_enter();
    __shared__ Cubic roots[kFlattenMaxWarps][32];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t s0 = (blockIdx.x * (blockDim.x >> 5) + wib) * 32u;
    if (s0 == 0 && lane == 0 && f.counters->lines > f.line_cap) {  // the flattening scan's total
        atomicOr(&f.counters->status, kStatusLineCapacity);
        f.counters->needed_lines = f.counters->lines;
    }
    if (s0 >= f.seg_count || f.counters->lines > f.line_cap) return;  // whole warps
    const uint32_t s = s0 + lane;
    uint32_t n = 0, path = 0;
    unsigned long long leaves = 0;
    Cubic c{};
    const uint32_t warp_base = f.seg_warp_base[s0 / 32u];
    if (s < f.seg_count) {
        // the segment's reads issued together
        const SegRec sr = f.segs[f.seg_begin + s];
        n = f.seg_line_count[s];
        const unsigned long long lv = f.seg_leaves[s];
        if (n) {
            segment_root(f.pts, sr, c, &f.counters->status);
            leaves = lv;
            path = (uint32_t)sr.w;
        }
    }
    // the segment's first line: the warp's base plus the lines of its lanes before it
    const uint32_t base = warp_base + warp_inclusive_scan(n) - n;
    const bool walk = n != 0 && leaves == 0;
    if (n != 0 && leaves > 1ull) roots[wib][lane] = c;  // leaves spread over the warp below
    if (n != 0 && leaves == 1ull) {  // one leaf at level 0: the root's base line, by its own lane
        f.lines[base] = make_float4(c.base.fx, c.base.fy, c.base.tx, c.base.ty);
        f.line_path[base] = path;
        if constexpr (DIFF) {
            f.line_seg[base] = f.seg_begin + s;
            f.line_t[base] = make_float2(0.0f, 1.0f);
        }
    }
    const uint32_t nl = walk || leaves == 1ull ? 0u : n;
    const uint32_t incl = warp_inclusive_scan(nl);
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    __syncwarp();
    for (uint32_t i0 = 0; i0 < total; i0 += 32) {
        const uint32_t i = i0 + lane;
        const uint32_t j = warp_owner(incl, i);
        const uint32_t k = i - __shfl_sync(0xffffffffu, incl - nl, j);
        const unsigned long long lj = __shfl_sync(0xffffffffu, leaves, j);
        const uint32_t bj = __shfl_sync(0xffffffffu, base, j), pj = __shfl_sync(0xffffffffu, path, j);
        if (i < total) {
            // leaf k: from its start slot to the next leaf's (or the end)
            const uint32_t start = nth_set_bit64(lj, k);
            const unsigned long long above = start >= 63u ? 0ull : (lj >> (start + 1u));
            const uint32_t next = above ? start + (uint32_t)__ffsll((long long)above) : 64u;
            const int d = kLeafLevels - (31 - __clz((int)(next - start)));
            const uint32_t addr = start >> (kLeafLevels - d);
            const Cubic c = subdivision_node(roots[wib][j], addr, d);
            const uint32_t l = bj + k;
            f.lines[l] = make_float4(c.base.fx, c.base.fy, c.base.tx, c.base.ty);
            f.line_path[l] = pj;
            if constexpr (DIFF) {
                const float step = ldexpf(1.0f, -d), t0 = (float)addr * step;
                f.line_seg[l] = f.seg_begin + s0 + j;
                f.line_t[l] = make_float2(t0, t0 + step);
            }
        }
    }
    if (!walk) return;
    const uint32_t sg = f.seg_begin + s;
    uint32_t l = base;
    flatten_segment(f.pts, f.segs[sg], [&](const Line& ln, uint32_t addr, int d) {
        f.lines[l] = make_float4(ln.fx, ln.fy, ln.tx, ln.ty);
        f.line_path[l] = path;
        if constexpr (DIFF) {
            const float step = ldexpf(1.0f, -d), t0 = (float)addr * step;
            f.line_seg[l] = sg;
            f.line_t[l] = make_float2(t0, t0 + step);
        }
        l++;
    }, &f.counters->status);
}

// The D3D11 level's uniform dicing: one thread per input segment.
__global__ void __launch_bounds__(256, 6) k_dice_count(FrameDev f) {
    pdl_enter();
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= f.seg_count) return;
    uint32_t n = 0;
    bool limited = false;
    const DiceSeg dsg = dice_seg(f.pts, f.segs[f.seg_begin + s]);
    if (dice_finite(dsg)) n = dice_count(dsg, &limited);
    else atomicOr(&f.counters->status, kStatusMalformed);  // no pieces for non-finite input
    if (limited) atomicOr(&f.counters->status, kStatusDepthLimit);
    f.seg_line_count[s] = n;
}

__global__ void __launch_bounds__(256, 6) k_dice_emit(FrameDev f) {
    pdl_enter();
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0 && f.counters->lines > f.line_cap) {  // the dicing scan's total against the capacity
        atomicOr(&f.counters->status, kStatusLineCapacity);
        f.counters->needed_lines = f.counters->lines;
    }
    if (s >= f.seg_count || f.counters->lines > f.line_cap) return;
    const SegRec sr = f.segs[f.seg_begin + s];
    uint32_t l = f.seg_line_base[s];
    // uniform pieces, ends rounded to 1/256 px
    const DiceSeg d = dice_seg(f.pts, sr);
    bool limited = false;
    const uint32_t n = dice_finite(d) ? dice_count(d, &limited) : 0u;
    float2 a = make_float2(dice_q(d.p0.x), dice_q(d.p0.y));
    for (uint32_t k = 1; k <= n; k++, l++) {
        const float2 b = dice_point(d, k, n);
        f.lines[l] = make_float4(a.x, a.y, b.x, b.y);
        f.line_path[l] = (uint32_t)sr.w;
        a = b;
    }
}

static size_t flatten_smem_bytes(int threads) { return (size_t)(threads / 32) * sizeof(FlattenWarp); }

void launch_flatten(const FrameDev& f, ScanTemp& tmp, cudaStream_t s) {
    if (f.seg_count == 0) return;
    const int ft = f.tune.flatten_threads;
    const bool dice = f.d3d11 && !f.diff;
    // dicing: a thread per segment; flattening: a warp per 32 segments
    const uint32_t blocks = dice ? (f.seg_count + ft - 1) / ft
                                 : (uint32_t)(((uint64_t)f.seg_count + 31) / 32 * 32 + ft - 1) / ft;
    count_launch();
    if (dice) {
        pdl_launch(k_dice_count, blocks, ft, 0, s, f);
    } else if (!f.diff && f.fill_e == nullptr) {  // line order free: one pass
        pdl_launch(k_flatten_count<false>, blocks, ft, flatten_smem_bytes(ft), s, f);
        return;
    } else {
        pdl_launch(k_flatten_count<true>, blocks, ft, flatten_smem_bytes(ft), s, f);
    }
    if (dice) {
        launch_scan(f.seg_line_count, f.seg_line_base, nullptr, f.seg_count, f.seg_count, 0, &f.counters->lines, tmp,
                    s);
    } else {  // one value per warp of 32 segments
        const uint32_t warps = (f.seg_count + 31) / 32;
        launch_scan(f.seg_warp_lines, f.seg_warp_base, nullptr, warps, warps, 0, &f.counters->lines, tmp, s);
    }
    count_launch();
    if (dice) pdl_launch(k_dice_emit, blocks, ft, 0, s, f);
    else if (f.diff) pdl_launch(k_flatten_emit<true>, blocks, ft, 0, s, f);
    else pdl_launch(k_flatten_emit<false>, blocks, ft, 0, s, f);
}

// ---------------------------------------------------------------------------
// binning: one thread per flattened line (process_line_segment, add_fill,
// adjust_alpha_tile_backdrop: renderer/src/tiler.rs:191-308,
// renderer/src/builder.rs:509-616)
// ---------------------------------------------------------------------------
// The frame's lines: the front range [0, lines) and, from a one-pass
// flattening, the back range of lines_back lines ending at the array's end.
// Line i of the frame (i < total) is at i below `front`, else at i + `skip`.
struct LineRanges {
    uint32_t total, front, skip;
    __device__ __forceinline__ uint32_t at(uint32_t i) const { return i < front ? i : i + skip; }
};
__device__ __forceinline__ LineRanges line_ranges(const FrameDev& f) {
    const uint64_t L0 = f.counters->lines, L1 = f.counters->lines_back;
    if (L0 + L1 > f.line_cap) return LineRanges{0u, 0u, 0u};
    return LineRanges{(uint32_t)(L0 + L1), (uint32_t)L0, f.line_cap - (uint32_t)(L0 + L1)};
}
__device__ __forceinline__ uint32_t line_total(const FrameDev& f) { return line_ranges(f).total; }

struct CountSink {
    const PathCtx* pc;
    uint32_t* tile_fill_count;
    int32_t* tile_delta;
    int32_t* col_backdrop;
    uint32_t n;
    template <class Rec>
    __device__ __forceinline__ void fill(Rec, uint32_t g) {
        n++;
        atomicAdd(&tile_fill_count[g], 1u);  // lanes rarely share a tile: aggregation costs more
    }
    __device__ __forceinline__ void backdrop(int32_t tx, int32_t ty, int32_t d) {
        // ObjectBuilder::adjust_alpha_tile_backdrop (renderer/src/builder.rs:595-616)
        int32_t w = pc->maxx - pc->minx, h = pc->maxy - pc->miny;
        int32_t ox = tx - pc->minx, oy = ty - pc->miny;
        if (ox < 0 || ox >= w || oy >= h) return;
        if (oy < 0) atomicAdd(&col_backdrop[pc->col_base + (uint32_t)ox], d);
        else atomicAdd(&tile_delta[pc->tile_base + (uint32_t)(oy * w + ox)], d);  // row-major, as the tiles
    }
};

template <int MODE>
__global__ void __launch_bounds__(512, 3) k_bin_count(FrameDev f) {
    pdl_enter();
    if (blockIdx.x == 0 && threadIdx.x == 0) {  // the flattening's total against the capacity
        const uint64_t L = f.counters->lines + f.counters->lines_back;
        if (L > f.line_cap) {
            atomicOr(&f.counters->status, kStatusLineCapacity);
            f.counters->needed_lines = L;
        }
    }
    if (f.counters->tiles > f.tile_cap || f.counters->columns > f.col_cap) return;
    const LineRanges lr = line_ranges(f);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < lr.total; i += gridDim.x * blockDim.x) {
        const uint32_t l = lr.at(i);
        const float4 ln = f.lines[l];
        const PathCtx pc = f.path_bin[f.line_path[l]];
        CountSink sink{&pc, f.tile_fill_count, f.tile_delta, f.col_backdrop, 0};
        dda_line<MODE, true>(pc, Line{ln.x, ln.y, ln.z, ln.w}, sink, f.dda_limit, &f.counters->status);
        if (f.fill_e != nullptr) f.line_fill_count[l] = sink.n;  // the emission-index scan's input
    }
}

// ORDER also writes each fill's emission index (only frames run for record
// read-back do: the order of fills within a tile changes no output).
// The tile scan leaves each tile's fill end (offset + count) in its count
// word: a fill's slot is that cursor, decremented, so one atomic gives it.
// The store of each fill waits one fill: the cursor's value comes back from
// L2 while the DDA computes the next fill (flush() stores the last one).
// The sink reads the frame's pointers from the kernel parameter itself.
template <bool ORDER>
struct EmitSink {
    const FrameDev* f;
    uint32_t e;
    bool pending = false;
    uint32_t p_end = 0, p_e = 0;
    uint2 p_rec = make_uint2(0u, 0u);
    __device__ __forceinline__ void store_pending() {
        const uint32_t slot = p_end - 1u;
        if (slot < f->fill_cap) {
            f->fills[slot] = p_rec;
            if (ORDER) f->fill_e[slot] = p_e;
        }
    }
    __device__ __forceinline__ void fill(uint2 rec, uint32_t g) {
        const uint32_t end = atomicSub(&f->tile_fill_count[g], 1u);
        if (pending) store_pending();
        pending = true;
        p_end = end; p_rec = rec; p_e = e;
        if (ORDER) e++;
    }
    __device__ __forceinline__ void flush() {
        if (pending) store_pending();
        pending = false;
    }
    __device__ __forceinline__ void backdrop(int32_t, int32_t, int32_t) {}
};

// FP32 fills of differentiable frames (no emission index: nothing reads it).
struct EmitSinkF {
    float4* fills;
    uint32_t* cursor;  // each tile's fill end, counted down
    uint32_t fill_cap;
    __device__ __forceinline__ void fill(float4 rec, uint32_t g) {
        const uint32_t slot = atomicSub(&cursor[g], 1u) - 1u;
        if (slot < fill_cap) fills[slot] = rec;
    }
    __device__ __forceinline__ void flush() {}
    __device__ __forceinline__ void backdrop(int32_t, int32_t, int32_t) {}
};

template <int MODE, bool ORDER>
__global__ void __launch_bounds__(512, 3) k_bin_emit(const __grid_constant__ FrameDev f) {
    pdl_enter();
    if (blockIdx.x == 0 && threadIdx.x == 0) {  // the binning scans' totals against the capacities
        if (f.counters->fills > f.fill_cap) {
            atomicOr(&f.counters->status, kStatusFillCapacity);
            f.counters->needed_fills = f.counters->fills;
        }
        if (f.counters->alpha_tiles > f.tile_cap) atomicOr(&f.counters->status, kStatusAlphaCapacity);
    }
    if (f.counters->tiles > f.tile_cap || f.counters->columns > f.col_cap) return;
    if (f.counters->fills > f.fill_cap) return;
    const LineRanges lr = line_ranges(f);
    // one sink for all of the thread's lines: a fill's store waits for the
    // thread's next fill, whichever line it comes from
    EmitSink<ORDER> sink{&f, 0u};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < lr.total; i += gridDim.x * blockDim.x) {
        const uint32_t l = lr.at(i);
        // the line's reads issued together; frames that write emission
        // indices skip lines without fills by their count (the others walk
        // them: they emit nothing)
        const uint32_t nfill = ORDER ? f.line_fill_count[l] : 1u;
        const float4 ln = f.lines[l];
        const uint32_t gp = f.line_path[l];
        if (nfill == 0) continue;
        const PathCtx pc = f.path_bin[gp];
        if constexpr (MODE == kFillF32) {
            EmitSinkF sinkf{f.fills_f, f.tile_fill_count, f.fill_cap};
            dda_line<MODE>(pc, Line{ln.x, ln.y, ln.z, ln.w}, sinkf, f.dda_limit, &f.counters->status);
        } else {
            if (ORDER) sink.e = f.line_fill_base[l];
            dda_line<MODE>(pc, Line{ln.x, ln.y, ln.z, ln.w}, sink, f.dda_limit, &f.counters->status);
        }
    }
    if constexpr (MODE != kFillF32) sink.flush();
}

// The binning pass's fill conversion for the frame.
static int fill_mode(const FrameDev& f) { return f.diff ? kFillF32 : (f.d3d11 ? kFillD3D11 : kFillCpu); }

void launch_bin_count(const FrameDev& f, cudaStream_t s) {
    count_launch();
    const uint32_t blocks = f.sms * f.tune.bin_blocks_per_sm;
    const int m = fill_mode(f);
    if (m == kFillF32) pdl_launch(k_bin_count<kFillF32>, blocks, f.tune.bin_threads, 0, s, f);
    else if (m == kFillD3D11) pdl_launch(k_bin_count<kFillD3D11>, blocks, f.tune.bin_threads, 0, s, f);
    else pdl_launch(k_bin_count<kFillCpu>, blocks, f.tune.bin_threads, 0, s, f);
}

// The emit pass runs beside propagation and visibility in a frame's graph,
// and alone in frames run in order: four waves of resident blocks (measured
// on the 4K frame with lines sorted by kind: 0.093 ms alone against 0.108 at
// two waves and 0.104 at one, the graph's frame the same at all three).
template <class K>
static uint32_t emit_blocks(const FrameDev& f, K kernel, int threads) {
    return f.sms * 4u * (uint32_t)std::max(resident_blocks(kernel, threads), 1);
}

void launch_bin_emit(const FrameDev& f, cudaStream_t s) {
    count_launch();
    const int m = fill_mode(f);
    const int t = f.tune.bin_threads;
    const bool order = f.fill_e != nullptr;
    if (m == kFillF32) pdl_launch(k_bin_emit<kFillF32, false>, emit_blocks(f, k_bin_emit<kFillF32, false>, t), t, 0, s, f);
    else if (m == kFillD3D11 && order)
        pdl_launch(k_bin_emit<kFillD3D11, true>, emit_blocks(f, k_bin_emit<kFillD3D11, true>, t), t, 0, s, f);
    else if (m == kFillD3D11)
        pdl_launch(k_bin_emit<kFillD3D11, false>, emit_blocks(f, k_bin_emit<kFillD3D11, false>, t), t, 0, s, f);
    else if (order) pdl_launch(k_bin_emit<kFillCpu, true>, emit_blocks(f, k_bin_emit<kFillCpu, true>, t), t, 0, s, f);
    else pdl_launch(k_bin_emit<kFillCpu, false>, emit_blocks(f, k_bin_emit<kFillCpu, false>, t), t, 0, s, f);
}

}  // namespace pf

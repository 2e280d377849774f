// pf_noalloc.cu — the exclusive scan for callers that cannot allocate.
//
// Some callers of this library cannot call cudaMalloc while they work: a
// real-time frame loop where cudaMalloc's implicit device synchronisation
// would stall the frame, a host whose device memory is owned by its own pool
// allocator, or code that runs while another module captures a CUDA graph.
// PFCUDAExclusiveScanNoAlloc gives them the scan that turns per-tile fill
// counts into fill offsets without any allocation: its scratch (one partial
// sum per 2,048-value block) lives in the fixed array below, which every GPU
// that loads the library holds until the process exits (32 KiB per device).
//
// Limits and sharing:
//   * at most kNoAllocMaxCount (16,777,216) values per call; larger calls are
//     rejected with PF_CUDA_ERR_CAPACITY before anything is launched;
//   * every call shares the one array, so calls that overlap on the GPU (on
//     different streams, or from different host threads) race and corrupt
//     each other's results: serialise them;
//   * nothing in the array needs to start at zero: each partial sum a call
//     reads was written earlier by the same call, so the previous call's
//     contents are never used;
//   * the array's device address is looked up once per device and kept for
//     the life of the process: a device reset (cudaDeviceReset) in the host
//     process makes it stale, so the library must not outlive one;
//   * the returned status is that of this call's own launches (taken from
//     each launch's return value): an error that unrelated earlier work left
//     pending in the runtime is neither reported nor cleared.
#include "pf_kernels.cuh"
#include "../../include/pathfinder_cuda.h"

#include <mutex>

namespace {

constexpr uint32_t kNoAllocMaxCount = 1u << 24;
constexpr uint32_t kNoAllocBlock = 2048;  // values per scan block (pf_tiler.cu)
constexpr uint32_t kNoAllocPartials = kNoAllocMaxCount / kNoAllocBlock + 2;

// Fixed scratch of the allocation-free scan.  In host code this name is only
// a host-side stand-in for the device symbol, never a device address: the
// address kernels receive comes from cudaGetSymbolAddress below.
static __device__ __align__(256) uint32_t g_noalloc_scan_scratch[kNoAllocPartials];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
uint32_t* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once
// per device (the first call on a device does this set-up).
cudaError_t scratch_for_current_device(uint32_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scan_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = (uint32_t*)p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int32_t PFCUDAExclusiveScanNoAlloc(const uint32_t* in, uint32_t* out, uint32_t n, void* stream) {
    if (!out || (!in && n)) return PF_CUDA_ERR_INVALID;
    if (n > kNoAllocMaxCount) return PF_CUDA_ERR_CAPACITY;
    uint32_t* scratch = nullptr;
    cudaError_t e = scratch_for_current_device(&scratch);
    if (e != cudaSuccess) return e == cudaErrorNoDevice ? PF_CUDA_ERR_NO_DEVICE : PF_CUDA_ERR_LAUNCH;
    pf::ScanTemp tmp{scratch, kNoAllocPartials};
    e = pf::launch_scan_checked(in, out, n, tmp, (cudaStream_t)stream);
    return e == cudaSuccess ? PF_CUDA_OK : PF_CUDA_ERR_LAUNCH;
}

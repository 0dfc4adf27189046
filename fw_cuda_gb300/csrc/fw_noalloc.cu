// APSP entry point for callers that cannot allocate device memory.
//
// fw_apsp_i32 allocates its panel workspace with cudaMalloc on first use, and
// fw_apsp_i32_ws wants the caller to provide one. Some callers can do
// neither: a process whose memory pool already owns every free byte of the
// GPU (a serving runtime that reserves device memory up front), code that must
// not trigger the implicit device synchronisation of cudaMalloc/cudaFree, or
// a plugin host that gives its plugins no allocator at all. For them,
// fw_apsp_i32_noalloc takes its workspace from the fixed array below, which
// is part of the library's device image: every GPU that loads the library
// holds these 8 MiB until the process exits, and no call allocates anything.
//
// The array covers the blocked sweep's two 128-row panels at n <= 8192 (and
// the per-pivot sweep's four snapshot rows at the same n); larger graphs are
// rejected with FW_ERR_INVALID_ARGUMENT. Every call on every stream shares the
// one array and it keeps whatever the previous call left in it; each call
// writes every word it later reads, so nothing needs clearing, but two calls
// whose work overlaps on the GPU (different streams, or different host
// threads) race on it and must be serialised by the caller.
//
// Host code cannot use the array's name as a device address (on the host it
// names a shadow variable), so the device address is looked up once per
// device with cudaGetSymbolAddress, with that device current, by the first
// call on that device. Make that first call before any stream capture.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "fw103.h"
#include "fw_internal.h"

namespace {

constexpr int64_t kNoAllocMaxN = 8192;
// Two panels of 128 rows with a leading dimension of kNoAllocMaxN.
constexpr size_t kNoAllocScratchInts = 2 * 128 * static_cast<size_t>(kNoAllocMaxN);

static __device__ __align__(256) int32_t g_fw_noalloc_scratch[kNoAllocScratchInts];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the array on the current device (set-up on first use).
int scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fw::cuda_error(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return fw::set_error(FW_ERR_INVALID_ARGUMENT, "device ordinal " + std::to_string(dev) + " out of range");
    std::lock_guard<std::mutex> lk(g_setup_mutex);
    if (g_scratch_addr[dev] == nullptr) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_fw_noalloc_scratch);
        if (e != cudaSuccess) return fw::cuda_error(e, "cudaGetSymbolAddress(g_fw_noalloc_scratch)");
        if (p == nullptr) return fw::set_error(FW_ERR_CUDA, "cudaGetSymbolAddress returned a null address");
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return FW_OK;
}

}  // namespace

extern "C" int fw_apsp_i32_noalloc(int32_t* d_D, int64_t n, int tile, int kappa, int variant,
                                   fw_stream_t stream) {
    // The two-block schedule of kappa > 4 needs twice the panel workspace;
    // kappa only selects the schedule, not the result, so cap it here.
    if (kappa > 4) kappa = 4;
    // The packed fast path needs an n x n 16-bit copy; here the int32 sweep runs.
    if (variant == FW_VARIANT_AUTO) variant = FW_VARIANT_MULTI_LAYER;
    if (n > kNoAllocMaxN)
        return fw::set_error(FW_ERR_INVALID_ARGUMENT,
                             "fw_apsp_i32_noalloc: n = " + std::to_string(n) +
                                 " exceeds the fixed scratch limit of n <= " + std::to_string(kNoAllocMaxN) +
                                 "; use fw_apsp_i32 or fw_apsp_i32_ws for larger graphs");
    const size_t need = fw::min_workspace_bytes(n, kappa, variant);
    if (need > sizeof(g_fw_noalloc_scratch))
        return fw::set_error(FW_ERR_INVALID_ARGUMENT, "fw_apsp_i32_noalloc: workspace of " + std::to_string(need) +
                                                          " bytes exceeds the fixed scratch array");
    if (d_D == nullptr) return fw::set_error(FW_ERR_INVALID_ARGUMENT, "d_D is NULL");
    void* scratch = nullptr;
    if (int rc = scratch_address(&scratch)) return rc;
    // Passing exactly the minimum keeps the single-stream schedule (the
    // look-ahead would also create a side stream on first use).
    return fw_apsp_i32_ws(d_D, n, tile, kappa, variant, scratch, need, stream);
}

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
// The array covers the call's 256-byte status block and the blocked sweep's
// two 128-row panels at n <= 8192 (or the per-pivot sweep's four snapshot
// rows at the same n); larger graphs are rejected with
// FW_ERR_INVALID_ARGUMENT. FW_VARIANT_AUTO runs the int32 multi-layer sweep
// here (the packed path needs an n x n copy of the matrix), and kappa > 4 runs
// as kappa 4 (the two-block pass needs twice the panels); neither changes the
// result. Every call on every stream shares the
// one array and it keeps whatever the previous call left in it; each call
// writes every word it later reads, so nothing needs clearing, but two calls
// whose work overlaps on the GPU (different streams, or different host
// threads) race on it and must be serialised by the caller.
//
// Host code cannot use the array's name as a device address (on the host it
// names a shadow variable), so the device address is looked up once per
// device with cudaGetSymbolAddress, with that device current, by the first
// call on that device. Make that first call before any stream capture. The
// address belongs to the device's context: after cudaDeviceReset the next
// call sees a new context and looks the address up again.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <mutex>
#include <string>

#include "fw103.h"
#include "fw_internal.h"

namespace {

constexpr int64_t kNoAllocMaxN = 8192;
// The status block, then two panels of 128 rows with a leading dimension of
// kNoAllocMaxN.
constexpr size_t kNoAllocScratchInts = fw::kStatusBytes / 4 + 2 * 128 * static_cast<size_t>(kNoAllocMaxN);

static __device__ __align__(256) int32_t g_fw_noalloc_scratch[kNoAllocScratchInts];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
struct ScratchAddr {
    CUcontext ctx = nullptr;  // the context the address was looked up in
    void* ptr = nullptr;
};
ScratchAddr g_scratch_addr[kMaxDevices];

// The driver's cuCtxGetCurrent, through the runtime's entry-point query (the
// library does not link libcuda itself).
PFN_cuCtxGetCurrent_v4000 ctx_get_current() {
    static PFN_cuCtxGetCurrent_v4000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// Device address of the array on the current device: looked up once per
// device and context (set-up on the first call, again after a device reset).
int scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fw::cuda_error(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return fw::set_error(FW_ERR_INVALID_ARGUMENT, "device ordinal " + std::to_string(dev) + " out of range");
    // Makes the device's primary context current (and creates it after a reset).
    e = cudaSetDevice(dev);
    if (e != cudaSuccess) return fw::cuda_error(e, "cudaSetDevice");
    CUcontext ctx = nullptr;
    const auto get_ctx = ctx_get_current();
    if (!get_ctx || get_ctx(&ctx) != CUDA_SUCCESS || ctx == nullptr)
        return fw::set_error(FW_ERR_CUDA, "cuCtxGetCurrent is not available or returned no context");
    std::lock_guard<std::mutex> lk(g_setup_mutex);
    ScratchAddr& a = g_scratch_addr[dev];
    if (a.ptr == nullptr || a.ctx != ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_fw_noalloc_scratch);
        if (e != cudaSuccess) return fw::cuda_error(e, "cudaGetSymbolAddress(g_fw_noalloc_scratch)");
        if (p == nullptr) return fw::set_error(FW_ERR_CUDA, "cudaGetSymbolAddress returned a null address");
        a.ctx = ctx;
        a.ptr = p;
    }
    *out = a.ptr;
    return FW_OK;
}

}  // namespace

extern "C" int fw_apsp_i32_noalloc(int32_t* d_D, int64_t n, int tile, int kappa, int variant,
                                   fw_stream_t stream) {
    // The two-block schedule of kappa > 4 needs twice the panel workspace;
    // kappa only selects the schedule, not the result, so cap it here.
    if (kappa > 4) kappa = 4;
    // The packed fast path needs an n x n 16-bit copy; here the int32 sweep runs.
    const bool was_auto = variant == FW_VARIANT_AUTO;
    if (was_auto) variant = FW_VARIANT_MULTI_LAYER;
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
    // An earlier AUTO report of this stream no longer describes its last call.
    if (was_auto) fw::forget_auto_report(reinterpret_cast<cudaStream_t>(stream));
    // Passing exactly the minimum keeps the single-stream schedule (the
    // look-ahead would also create a side stream on first use), and the
    // per-pivot sweep launches directly instead of replaying a graph.
    return fw::apsp_i32_ws(d_D, n, tile, kappa, variant, scratch, need, stream, false, false);
}

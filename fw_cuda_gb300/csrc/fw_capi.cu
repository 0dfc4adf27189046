// C ABI of libfw103.so (declared in include/fw103.h): argument checks, status
// codes, the per-(device, stream) workspace cache, per-kernel timing and the
// host-side graph generator.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <random>
#include <string>
#include <utility>
#include <vector>

#include "fw103.h"
#include "fw_internal.h"

namespace fw {
namespace {

thread_local std::string t_last_error;

// ----------------------------------------------------------------- workspace
struct WsEntry {
    void* ptr = nullptr;
    size_t bytes = 0;
};
std::mutex g_ws_mutex;
std::map<std::pair<int, cudaStream_t>, WsEntry> g_ws;
// Device address of the packed path's `done` word of the last FW_VARIANT_AUTO
// call per (device, stream), for fw_apsp_auto_report.
std::map<std::pair<int, cudaStream_t>, const unsigned int*> g_auto_done;
// Device address of the status word of the last call per (device, stream)
// that has one (the blocked, next-hop and fp32 sweeps), for fw_check_faults.
std::map<std::pair<int, cudaStream_t>, unsigned int*> g_last_status;

// Host-side fault injection for tests (fw_debug_inject), per host thread.
thread_local int t_inject = 0;

// ----------------------------------------------------------------- profiling
struct ProfState {
    std::atomic<bool> on{false};
    std::vector<cudaEvent_t> pool;
    size_t next = 0;
    struct Rec {
        int kc;
        cudaEvent_t a, b;
        double relax;
        int64_t launches;
    };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> open;  // one pending start event per class
};
std::mutex g_prof_mutex;
ProfState g_prof;
const char* const kClassNames[KC_COUNT] = {"fw_diag",          "fw_panel",        "fw_remainder",
                                           "fw_pivot_step",    "fw_batched",      "fw_forward_f32",
                                           "fw_backward_f32",  "fw_p16_diag",     "fw_p16_panel",
                                           "fw_p16_remainder", "fw_paths_i32",    "fw_ooc_update",
                                           "fw_stripe"};

cudaEvent_t prof_event() {
    if (g_prof.next == g_prof.pool.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        g_prof.pool.push_back(e);
    }
    return g_prof.pool[g_prof.next++];
}

}  // namespace

int set_error(int status, const std::string& msg) {
    t_last_error = msg;
    return status;
}

int cuda_error(cudaError_t e, const char* what) {
    return set_error(FW_ERR_CUDA, std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

void prof_begin(KernelClass kc, cudaStream_t s) {
    if (!g_prof.on) return;
    std::lock_guard<std::mutex> lk(g_prof_mutex);
    cudaEvent_t e = prof_event();
    if (!e) return;
    cudaEventRecord(e, s);
    g_prof.open[kc] = e;
}

void prof_end(KernelClass kc, cudaStream_t s, double relaxations, int64_t launches) {
    if (!g_prof.on) return;
    std::lock_guard<std::mutex> lk(g_prof_mutex);
    cudaEvent_t a = g_prof.open[kc];
    cudaEvent_t b = prof_event();
    if (!a || !b) return;
    cudaEventRecord(b, s);
    g_prof.recs.push_back({kc, a, b, relaxations, launches});
    g_prof.open[kc] = nullptr;
}

void* workspace_get(cudaStream_t s, size_t bytes) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        set_error(FW_ERR_CUDA, "cudaGetDevice failed");
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_ws_mutex);
    WsEntry& w = g_ws[{dev, s}];
    if (w.bytes >= bytes && w.ptr) return w.ptr;
    if (w.ptr) {
        // The old buffer may still be in use by work queued on `s`.
        cudaStreamSynchronize(s);
        cudaFree(w.ptr);
        w.ptr = nullptr;
        w.bytes = 0;
        // an FW_VARIANT_AUTO report and a status word of this stream pointed into it
        g_auto_done.erase({dev, s});
        g_last_status.erase({dev, s});
    }
    void* p = nullptr;
    const cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error(FW_ERR_NO_MEMORY, "workspace allocation of " + std::to_string(bytes) +
                                        " bytes failed: " + cudaGetErrorString(e));
        return nullptr;
    }
    w.ptr = p;
    w.bytes = bytes;
    return p;
}

// Zeroes the call's status block on `s` and records its first word as the
// stream's last status word.
int status_begin(cudaStream_t s, void* status_block) {
    FW_CUDA_TRY(cudaMemsetAsync(status_block, 0, kStatusBytes, s));
    int dev = 0;
    FW_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_ws_mutex);
    g_last_status[{dev, s}] = static_cast<unsigned int*>(status_block);
    return FW_OK;
}

// Test hook: a pending FW_INJECT_CALL_FAULT makes the call's status word
// nonzero after its kernels, as a missed copy would.
int status_end(cudaStream_t s, void* status_block) {
    if (t_inject & FW_INJECT_CALL_FAULT) {
        t_inject &= ~FW_INJECT_CALL_FAULT;
        FW_CUDA_TRY(cudaMemsetAsync(status_block, 0x01, 1, s));
    }
    return FW_OK;
}

bool take_packed_fault_injection() {
    const bool on = (t_inject & FW_INJECT_PACKED_FAULT) != 0;
    t_inject &= ~FW_INJECT_PACKED_FAULT;
    return on;
}

const unsigned int* last_call_status(cudaStream_t s) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_ws_mutex);
    auto it = g_last_status.find({dev, s});
    return it == g_last_status.end() ? nullptr : it->second;
}

void forget_auto_report(cudaStream_t s) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    std::lock_guard<std::mutex> lk(g_ws_mutex);
    g_auto_done.erase({dev, s});
}

namespace {
std::mutex g_aux_mutex;
std::map<std::pair<int, cudaStream_t>, AuxStream> g_aux;
}  // namespace

int aux_stream_get(cudaStream_t s, AuxStream* out) {
    int dev = 0;
    FW_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_aux_mutex);
    AuxStream& a = g_aux[{dev, s}];
    if (!a.side) {
        int least = 0, greatest = 0;
        FW_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        FW_CUDA_TRY(cudaStreamCreateWithFlags(&a.side, cudaStreamNonBlocking));
        FW_CUDA_TRY(cudaStreamCreateWithPriority(&a.hi, cudaStreamNonBlocking, greatest));
        FW_CUDA_TRY(cudaEventCreateWithFlags(&a.fork, cudaEventDisableTiming));
        for (int i = 0; i < 2; ++i) {
            FW_CUDA_TRY(cudaEventCreateWithFlags(&a.panels[i], cudaEventDisableTiming));
            FW_CUDA_TRY(cudaEventCreateWithFlags(&a.bulk[i], cudaEventDisableTiming));
        }
    }
    *out = a;
    return FW_OK;
}

int normalise_kappa(int kappa) { return (kappa <= 0 || kappa > 16) ? 4 : kappa; }

}  // namespace fw

using namespace fw;

namespace {

int check_apsp_args(const int32_t* d_D, int64_t n, int variant) {
    if (d_D == nullptr) return set_error(FW_ERR_INVALID_ARGUMENT, "d_D is NULL");
    if (n < 1) return set_error(FW_ERR_INVALID_ARGUMENT, "n must be >= 1, got " + std::to_string(n));
    // 64-bit offsets throughout; the per-pivot sweep puts one row per grid.y.
    const int64_t nmax = (variant == FW_VARIANT_BASELINE) ? 65535 : 262144;
    if (n > nmax)
        return set_error(FW_ERR_INVALID_ARGUMENT,
                         "n = " + std::to_string(n) + " exceeds " + std::to_string(nmax) + " for this variant");
    if (variant != FW_VARIANT_BASELINE && variant != FW_VARIANT_TILING && variant != FW_VARIANT_MULTI_LAYER &&
        variant != FW_VARIANT_AUTO)
        return set_error(FW_ERR_INVALID_ARGUMENT, "unknown variant " + std::to_string(variant));
    if ((reinterpret_cast<uintptr_t>(d_D) & 15u) != 0)
        return set_error(FW_ERR_INVALID_ARGUMENT, "d_D must be 16-byte aligned (cudaMalloc memory is)");
    return FW_OK;
}

}  // namespace

extern "C" {

const char* fw_last_error_string(void) { return t_last_error.c_str(); }

const char* fw_version(void) { return "fw103 0.1.0 (sm_103a)"; }

// The blocked variants run fastest with two panel buffers (look-ahead, or the
// two-block pass of kappa > 4); one buffer is the minimum for kappa <= 4.
size_t fw_workspace_bytes_i32(int64_t n, int tile, int kappa, int variant) {
    (void)tile;
    (void)kappa;
    if (n < 1) return 0;
    if (variant == FW_VARIANT_BASELINE) return kStatusBytes + pivot_workspace_bytes(n);
    const size_t blocked = blocked_workspace_bytes(n, 2);
    const size_t body =
        variant == FW_VARIANT_AUTO ? ((blocked + 255) & ~size_t(255)) + p16_workspace_bytes(n) : blocked;
    // Small graphs run the stripe sweep when the workspace holds it.
    const size_t stripe = stripe_workspace_bytes(n);
    return kStatusBytes + (stripe > body ? stripe : body);
}

}  // extern "C"

namespace fw {
size_t min_workspace_bytes(int64_t n, int kappa, int variant) {
    if (n < 1) return 0;
    if (variant == FW_VARIANT_BASELINE) return kStatusBytes + pivot_workspace_bytes(n);
    const size_t blocked = blocked_workspace_bytes(n, blocks_per_pass(variant, kappa, n));
    if (variant == FW_VARIANT_AUTO)
        return kStatusBytes + ((blocked_workspace_bytes(n, 2) + 255) & ~size_t(255)) + p16_workspace_bytes(n);
    return kStatusBytes + blocked;
}

int apsp_i32_ws(int32_t* d_D, int64_t n, int tile, int kappa, int variant, void* d_workspace,
                size_t workspace_bytes, fw_stream_t stream, bool may_allocate, bool allow_stripe) {
    if (int rc = check_apsp_args(d_D, n, variant)) return rc;
    (void)tile;  // fixed geometry, as in the reference (src/fw_tiling_gpu.cu:254-257)
    const size_t need = min_workspace_bytes(n, kappa, variant);
    if (d_workspace == nullptr || workspace_bytes < need)
        return set_error(FW_ERR_INVALID_ARGUMENT,
                         "workspace of " + std::to_string(need) + " bytes required, got " +
                             std::to_string(workspace_bytes));
    if ((reinterpret_cast<uintptr_t>(d_workspace) & 255u) != 0)
        return set_error(FW_ERR_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // Layout: the status block (kStatusBytes; its first word counts the
    // call's missed tile copies), then the sweep's own workspace.
    void* status = d_workspace;
    char* body = static_cast<char*>(d_workspace) + kStatusBytes;
    const size_t body_bytes = workspace_bytes - kStatusBytes;
    unsigned int* faults = static_cast<unsigned int*>(status);
    if (int rc = status_begin(s, status)) return rc;
    int rc = FW_OK;
    // For n <= 2048 the blocked variants and AUTO take the stripe sweep (one
    // cooperative launch; faster there than the packed path) when the
    // workspace has fw_workspace_bytes_i32() bytes; a smaller caller workspace
    // keeps the 128-wide blocked sweep, or the packed path for AUTO.
    if (allow_stripe && variant != FW_VARIANT_BASELINE && stripe_workspace_bytes(n) > 0 &&
        body_bytes >= stripe_workspace_bytes(n) && body_bytes >= blocked_workspace_bytes(n, 2)) {
        bool ran = false;
        rc = stripe_solve(d_D, n, body, s, faults, &ran);
        if (rc) return rc;
        if (ran) {
            if (variant == FW_VARIANT_AUTO) {
                // fw_apsp_auto_report reads a word of this call's status
                // block that status_begin zeroed: the packed path did not run.
                int dev = 0;
                cudaGetDevice(&dev);
                std::lock_guard<std::mutex> lk(g_ws_mutex);
                g_auto_done[{dev, s}] = faults + 1;
            }
            return status_end(s, status);
        }
    }
    if (variant == FW_VARIANT_BASELINE) {
        rc = pivot_solve(d_D, n, body, s, may_allocate);
    } else if (variant == FW_VARIANT_AUTO) {
        const size_t blocked = (blocked_workspace_bytes(n, 2) + 255) & ~size_t(255);
        const unsigned int* done = nullptr;
        rc = p16_solve(d_D, n, body + blocked, s, &done, take_packed_fault_injection());
        if (rc) return rc;
        {
            int dev = 0;
            cudaGetDevice(&dev);
            std::lock_guard<std::mutex> lk(g_ws_mutex);
            g_auto_done[{dev, s}] = done;
        }
        // The int32 fallback behind the flag runs the two-block schedule on
        // one stream: its remainder launches are persistent, so that they
        // cost little when the packed result is taken.
        rc = blocked_solve(d_D, n, 2, body, blocked, s, done, faults);
    } else {
        rc = blocked_solve(d_D, n, blocks_per_pass(variant, kappa, n), body, body_bytes, s, nullptr, faults);
    }
    if (rc) return rc;
    return status_end(s, status);
}
}  // namespace fw

extern "C" {

int fw_apsp_i32_ws(int32_t* d_D, int64_t n, int tile, int kappa, int variant, void* d_workspace,
                   size_t workspace_bytes, fw_stream_t stream) {
    return apsp_i32_ws(d_D, n, tile, kappa, variant, d_workspace, workspace_bytes, stream, true);
}

int fw_apsp_i32(int32_t* d_D, int64_t n, int tile, int kappa, int variant, fw_stream_t stream) {
    if (int rc = check_apsp_args(d_D, n, variant)) return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const size_t need = fw_workspace_bytes_i32(n, tile, kappa, variant);
    void* ws = workspace_get(s, need);
    if (!ws) return FW_ERR_NO_MEMORY;
    return fw_apsp_i32_ws(d_D, n, tile, kappa, variant, ws, need, stream);
}

int fw_check_faults(fw_stream_t stream, unsigned int* count) {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const unsigned int* word = last_call_status(s);
    if (!word) return set_error(FW_ERR_INVALID_ARGUMENT, "fw_check_faults: no call with a status word on this device "
                                                         "and stream (or its library workspace was replaced)");
    FW_CUDA_TRY(cudaStreamSynchronize(s));
    unsigned int v = 0;
    FW_CUDA_TRY(cudaMemcpy(&v, word, sizeof(v), cudaMemcpyDeviceToHost));
    if (count) *count = v;
    if (v)
        return set_error(FW_ERR_TIMEOUT, std::to_string(v) +
                                             " tile copies did not arrive within their bounded wait; the call's "
                                             "result is not valid");
    return FW_OK;
}

int fw_debug_inject(int kinds) {
    if (kinds & ~(FW_INJECT_CALL_FAULT | FW_INJECT_PACKED_FAULT))
        return set_error(FW_ERR_INVALID_ARGUMENT, "fw_debug_inject: unknown kind " + std::to_string(kinds));
    t_inject = kinds;
    return FW_OK;
}

int fw_apsp_auto_report(fw_stream_t stream, int* used_packed) {
    if (!used_packed) return set_error(FW_ERR_INVALID_ARGUMENT, "used_packed is NULL");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int dev = 0;
    FW_CUDA_TRY(cudaGetDevice(&dev));
    const unsigned int* done = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_ws_mutex);
        auto it = g_auto_done.find({dev, s});
        if (it != g_auto_done.end()) done = it->second;
    }
    if (!done) return set_error(FW_ERR_INVALID_ARGUMENT, "no FW_VARIANT_AUTO call on this device and stream");
    FW_CUDA_TRY(cudaStreamSynchronize(s));
    unsigned int v = 0;
    FW_CUDA_TRY(cudaMemcpy(&v, done, sizeof(v), cudaMemcpyDeviceToHost));
    *used_packed = v ? 1 : 0;
    return FW_OK;
}

int fw_apsp_paths_i32(int32_t* d_D, int32_t* d_nh, int64_t n, int64_t batch, fw_stream_t stream) {
    if (!d_D || !d_nh) return set_error(FW_ERR_INVALID_ARGUMENT, "fw_apsp_paths_i32: NULL pointer");
    if (n < 1 || n > 65535 || batch < 1 || batch > 65535)
        return set_error(FW_ERR_INVALID_ARGUMENT, "fw_apsp_paths_i32: need 1 <= n <= 65535 and 1 <= batch <= 65535");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    void* ws = workspace_get(s, kStatusBytes + f32_workspace_bytes(n, batch));
    if (!ws) return FW_ERR_NO_MEMORY;
    if (int rc = status_begin(s, ws)) return rc;
    if (int rc = i32_paths(d_D, d_nh, n, batch, static_cast<char*>(ws) + kStatusBytes, s,
                           static_cast<unsigned int*>(ws)))
        return rc;
    return status_end(s, ws);
}

int fw_path_length_i32(const int32_t* h_nh, int64_t n, int64_t i, int64_t j, int32_t* h_path, int64_t cap) {
    if (!h_nh || n < 1 || i < 0 || j < 0 || i >= n || j >= n)
        return -set_error(FW_ERR_INVALID_ARGUMENT, "fw_path_length_i32: bad arguments");
    if (h_nh[i * n + j] < 0) return 0;
    int64_t len = 0, u = i;
    if (h_path && cap > 0) h_path[0] = (int32_t)i;
    len = 1;
    while (u != j) {
        const int64_t v = h_nh[u * n + j];
        if (v < 0 || v >= n || len > n) return -set_error(FW_ERR_INVALID_ARGUMENT, "next hops do not form a path");
        if (h_path && len < cap) h_path[len] = (int32_t)v;
        ++len;
        u = v;
    }
    return (int)len;
}

int fw_forward_f32(float* d_D, int32_t* d_nh, int64_t n, int64_t batch, fw_stream_t stream) {
    if (!d_D || !d_nh) return set_error(FW_ERR_INVALID_ARGUMENT, "fw_forward_f32: NULL pointer");
    if (n < 1 || n > 65535 || batch < 1 || batch > 65535)
        return set_error(FW_ERR_INVALID_ARGUMENT, "fw_forward_f32: need 1 <= n <= 65535 and 1 <= batch <= 65535");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    void* ws = workspace_get(s, kStatusBytes + f32_workspace_bytes(n, batch));
    if (!ws) return FW_ERR_NO_MEMORY;
    if (int rc = status_begin(s, ws)) return rc;
    if (int rc = f32_forward(d_D, d_nh, n, batch, static_cast<char*>(ws) + kStatusBytes, s,
                             static_cast<unsigned int*>(ws)))
        return rc;
    return status_end(s, ws);
}

int fw_backward(const float* d_dLdD, const int32_t* d_nh, float* d_dLdW, int64_t n, int64_t batch,
                int32_t* d_bad_walks, fw_stream_t stream) {
    if (!d_dLdD || !d_nh || !d_dLdW) return set_error(FW_ERR_INVALID_ARGUMENT, "fw_backward: NULL pointer");
    if (n < 1 || n > 16384 || batch < 1 || batch > 65535)
        return set_error(FW_ERR_INVALID_ARGUMENT, "fw_backward: need 1 <= n <= 16384 and 1 <= batch <= 65535");
    return f32_backward(d_dLdD, d_nh, d_dLdW, n, batch, d_bad_walks, reinterpret_cast<cudaStream_t>(stream));
}

int fw_generate_graph_i32(int32_t* h_out, int64_t n, double density, uint32_t seed, int32_t wmin, int32_t wmax) {
    if (h_out == nullptr) return set_error(FW_ERR_INVALID_ARGUMENT, "h_out is NULL");
    if (n < 1) return set_error(FW_ERR_INVALID_ARGUMENT, "n must be >= 1");
    if (!(density >= 0.0 && density <= 1.0)) return set_error(FW_ERR_INVALID_ARGUMENT, "density must be in [0, 1]");
    if (wmin > wmax) return set_error(FW_ERR_INVALID_ARGUMENT, "wmin > wmax");
    std::mt19937 gen(seed != 0 ? seed : std::random_device{}());
    std::uniform_int_distribution<int32_t> weight(wmin, wmax);
    std::bernoulli_distribution edge(density);
    const size_t nn = static_cast<size_t>(n);
    for (size_t i = 0; i < nn; ++i) {
        int32_t* row = h_out + i * nn;
        for (size_t j = 0; j < nn; ++j) {
            row[j] = (i == j) ? 0 : (edge(gen) ? weight(gen) : FW_INF);
        }
    }
    return FW_OK;
}

int fw_profile_begin(void) {
    std::lock_guard<std::mutex> lk(g_prof_mutex);
    g_prof.on = true;
    g_prof.next = 0;
    g_prof.recs.clear();
    g_prof.open.assign(KC_COUNT, nullptr);
    return FW_OK;
}

int fw_profile_end(fw_kernel_stats* out, int cap, int* count) {
    std::lock_guard<std::mutex> lk(g_prof_mutex);
    g_prof.on = false;
    std::vector<fw_kernel_stats> agg(KC_COUNT);
    for (int k = 0; k < KC_COUNT; ++k) {
        std::memset(&agg[k], 0, sizeof(fw_kernel_stats));
        std::snprintf(agg[k].name, sizeof(agg[k].name), "%s", kClassNames[k]);
    }
    int status = FW_OK;
    for (const auto& r : g_prof.recs) {
        if (cudaEventSynchronize(r.b) != cudaSuccess) {
            status = cuda_error(cudaGetLastError(), "cudaEventSynchronize");
            continue;
        }
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) {
            status = cuda_error(cudaGetLastError(), "cudaEventElapsedTime");
            continue;
        }
        agg[r.kc].launches += r.launches;
        agg[r.kc].total_ms += ms;
        agg[r.kc].relaxations += r.relax;
    }
    g_prof.recs.clear();
    g_prof.next = 0;
    int m = 0;
    for (int k = 0; k < KC_COUNT; ++k) {
        if (agg[k].launches == 0) continue;
        if (out && m < cap) out[m] = agg[k];
        ++m;
    }
    if (count) *count = m;
    return status;
}

int fw_measure_relax_peak(double* dpx_only, double* mixed, fw_stream_t stream) {
    return measure_relax_peak(dpx_only, mixed, reinterpret_cast<cudaStream_t>(stream));
}

int fw_measure_int32_rates(double* rates, int count, fw_stream_t stream) {
    if (!rates || count < 1) return set_error(FW_ERR_INVALID_ARGUMENT, "fw_measure_int32_rates: no output");
    return measure_int32_rates(rates, count, reinterpret_cast<cudaStream_t>(stream));
}

int fw_measure_relax_peak_packed(double* dpx_only, double* mixed, fw_stream_t stream) {
    return measure_relax_peak_packed(dpx_only, mixed, reinterpret_cast<cudaStream_t>(stream));
}

}  // extern "C"

// Host-side internals shared by the fw103 translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <string>

#include "fw103.h"

namespace fw {

// Records `msg` as this thread's last error and returns `status`.
int set_error(int status, const std::string& msg);

// Maps a CUDA error to FW_ERR_CUDA with a message naming `what`.
int cuda_error(cudaError_t e, const char* what);

#define FW_CUDA_TRY(call)                                              \
    do {                                                               \
        cudaError_t _e = (call);                                       \
        if (_e != cudaSuccess) return ::fw::cuda_error(_e, #call);     \
    } while (0)

#define FW_LAUNCH_CHECK(what)                                          \
    do {                                                               \
        cudaError_t _e = cudaGetLastError();                           \
        if (_e != cudaSuccess) return ::fw::cuda_error(_e, what);      \
    } while (0)

// Runs `fn` (returning a status) once per device, from any thread: kernel
// attributes such as the dynamic shared-memory limit belong to the current
// device's context, so a process that drives several GPUs sets them on each.
struct PerDeviceOnce {
    std::mutex mu;
    uint64_t done = 0;  // bit d: done on device d (devices >= 64 run it every time)
};

template <class Fn>
int once_per_device(PerDeviceOnce& once, Fn&& fn) {
    int dev = 0;
    FW_CUDA_TRY(cudaGetDevice(&dev));
    const uint64_t bit = (dev >= 0 && dev < 64) ? (uint64_t(1) << dev) : 0;
    std::lock_guard<std::mutex> lk(once.mu);
    if (once.done & bit) return FW_OK;
    const int rc = fn();
    if (rc == FW_OK) once.done |= bit;
    return rc;
}

// Kernel classes timed by fw_profile_begin/fw_profile_end.
enum KernelClass {
    KC_DIAG = 0,
    KC_PANEL,
    KC_REMAINDER,
    KC_PIVOT_STEP,
    KC_BATCHED,
    KC_FWD_F32,
    KC_BWD_F32,
    KC_P16_DIAG,
    KC_P16_PANEL,
    KC_P16_REMAINDER,
    KC_PATHS_I32,
    KC_OOC_UPDATE,
    KC_STRIPE,
    KC_COUNT
};

// Brackets one launch with events when profiling is on (no-ops otherwise).
// `relaxations` is the algorithmic work the launch performs.
void prof_begin(KernelClass kc, cudaStream_t s);
// `launches`: the kernel launches the bracket stands for (a replayed graph
// of several counts them all).
void prof_end(KernelClass kc, cudaStream_t s, double relaxations, int64_t launches = 1);

// Every workspace of an asynchronous sweep entry point starts with a status
// block of this size; its first word counts the call's tile copies that
// missed their bounded wait (fw_check_faults reads it).
constexpr size_t kStatusBytes = 256;

// Zeroes the status block on `s` and records it as the stream's last one;
// status_end applies a pending FW_INJECT_CALL_FAULT test injection.
int status_begin(cudaStream_t s, void* status_block);
int status_end(cudaStream_t s, void* status_block);
// Device address of the status word of the last call on (current device, s),
// or nullptr.
const unsigned int* last_call_status(cudaStream_t s);
// Whether a FW_INJECT_PACKED_FAULT test injection is pending (and clears it).
bool take_packed_fault_injection();
// Drops the stream's FW_VARIANT_AUTO report (a later call did not run AUTO).
void forget_auto_report(cudaStream_t s);

// Per-(device, stream) workspace owned by the library: at least `bytes`,
// 256-byte aligned, kept for later calls. Returns nullptr (and sets the last
// error) when allocation fails.
void* workspace_get(cudaStream_t s, size_t bytes);

// Two non-blocking streams and their events tied to the caller's (device,
// stream), created on first use and kept: the look-ahead schedules run the
// bulk remainder of pivot block t on `side` while `hi` carries the chain the
// next block waits for (block t's update of block t+1's row and column, then
// block t+1's closure and panels); its highest priority lets its few CTAs
// take SMs as soon as remainder CTAs retire.
struct AuxStream {
    cudaStream_t side = nullptr;  // bulk remainder (default priority)
    cudaStream_t hi = nullptr;    // the chain (highest priority)
    cudaEvent_t fork = nullptr;   // the caller's stream up to the solve
    cudaEvent_t panels[2] = {};   // block t's panels are ready (t & 1)
    cudaEvent_t bulk[2] = {};     // block t's bulk remainder is done (t & 1)
};
int aux_stream_get(cudaStream_t s, AuxStream* out);

// Normalised arguments of the blocked sweep.
int normalise_kappa(int kappa);

// Blocked-sweep launchers (fw_apsp_i32.cu).
int blocks_per_pass(int variant, int kappa, int64_t n);
size_t blocked_workspace_bytes(int64_t n, int blocks);
// `skip`, when not null, is a device flag: nonzero makes every kernel of the
// sweep return at once (the packed fast path already produced the result).
// `faults`, when not null, is the call's status word: every tile copy that
// misses its bounded wait adds one (the result is then not valid).
// With ws_bytes >= blocked_workspace_bytes(n, 2) the single-block schedule
// runs with a one-block look-ahead (two panel buffers).
int blocked_solve(int32_t* d_D, int64_t n, int blocks, void* ws, size_t ws_bytes, cudaStream_t s,
                  const unsigned int* skip = nullptr, unsigned int* faults = nullptr);
// Smallest workspace fw_apsp_i32_ws accepts for these arguments.
size_t min_workspace_bytes(int64_t n, int kappa, int variant);

// Stripe sweep (fw_stripe.cu): the blocked sweep with 8-wide pivot blocks in
// one cooperative launch, the matrix held in registers, for 1 <= n <= 2048.
constexpr int64_t kStripeMaxN = 2048;
// Workspace of the stripe sweep (0 when n is outside its range).
size_t stripe_workspace_bytes(int64_t n);
// Runs the stripe sweep when n is in range and the device can hold its
// cooperative grid; *ran tells whether it did (if not, nothing was enqueued).
// `faults`: the call's status word (flag waits that ran out add to it).
int stripe_solve(int32_t* d_D, int64_t n, void* ws, cudaStream_t s, unsigned int* faults, bool* ran);

// Exact packed 16-bit fast path (fw_packed16.cu).
size_t p16_workspace_bytes(int64_t n);
// inject_copy_fault (tests): mark the packed status as if a tile copy had
// missed its wait, so that the decode refuses and the int32 sweep runs.
int p16_solve(int32_t* D, int64_t n, void* ws, cudaStream_t s, const unsigned int** done_flag,
              bool inject_copy_fault = false);
size_t pivot_workspace_bytes(int64_t n);
// may_allocate = false: plain launches only (no CUDA graph is captured,
// which would allocate driver resources).
int pivot_solve(int32_t* d_D, int64_t n, void* ws, cudaStream_t s, bool may_allocate = true);
// fw_apsp_i32_ws; may_allocate = false for callers that must allocate nothing;
// allow_stripe = false keeps small graphs of the blocked variants on the
// blocked sweep.
int apsp_i32_ws(int32_t* d_D, int64_t n, int tile, int kappa, int variant, void* d_workspace,
                size_t workspace_bytes, fw_stream_t stream, bool may_allocate, bool allow_stripe = true);

// Differentiable fp32 forward / backward (fw_diff.cu).
size_t f32_workspace_bytes(int64_t n, int64_t batch);
int f32_forward(float* D, int* nh, int64_t n, int64_t batch, void* ws, cudaStream_t s, unsigned* faults);
int f32_backward(const float* G, const int* nh, float* dW, int64_t n, int64_t batch, int* d_bad, cudaStream_t s);
// int32 sweep that also records next hops (same kernels as the fp32 form).
int i32_paths(int* D, int* nh, int64_t n, int64_t batch, void* ws, cudaStream_t s, unsigned* faults);

// Remainder tile copies of the next-hop forward that missed their bounded
// wait (fw_diff.cu; part of fw_copy_faults).
unsigned int nh_copy_faults();
// The same for the out-of-core update kernel (fw_ooc.cu).
unsigned int ooc_copy_faults();

// Out-of-core sweep over a host-resident matrix (fw_ooc.cu); W and H are
// validated multiples of 128.
size_t ooc_device_bytes(int64_t n, int64_t W, int64_t H);
int ooc_solve(int32_t* h_D, int64_t n, int64_t W, int64_t H, cudaStream_t s);

// Register-only relaxation-rate kernels (fw_peak.cu).
int measure_relax_peak(double* dpx_only, double* mixed, cudaStream_t s);
// Per-class int32 rates (fw_measure_int32_rates; kInt32RateCount entries).
constexpr int kInt32RateCount = 9;
int measure_int32_rates(double* rates, int count, cudaStream_t s);
int measure_relax_peak_packed(double* dpx_only, double* mixed, cudaStream_t s);

}  // namespace fw

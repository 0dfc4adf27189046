// Stripe sweep: the blocked Floyd-Warshall sweep for n <= 2048 in ONE
// cooperative launch, with the whole matrix held in registers.
//
// For small matrices the 128-wide blocked sweep (fw_apsp_i32.cu) is bound by
// its critical path, not by arithmetic: every pivot block is a chain of
// kernels (row/column update, a 128-pivot closure on one SM, the panels), and
// at n = 1024 eight such chains take most of the solve. Here the pivot blocks
// are 8 wide and the hand-over between them is a flag in L2, not a kernel
// boundary:
//
//   * the matrix is cut into stripes of 8 rows; stripe z is held in registers
//     by CTA z % G (slot z / G; S <= 2 slots per CTA), every thread holding
//     the stripe's 8 rows of its 4 columns (one 16-byte vector per row);
//   * stage z applies the 8 pivots of stripe z. Its owner closes the 8 x 8
//     diagonal block Dg in one warp (shuffles), turns the stripe into
//     R' = min(R, Dg* (x) R) (a min-plus product, because Dg* is closed),
//     writes R' to the workspace and releases flag z;
//   * every other stripe takes stage z as D = min(D, C (x) R'), where C is the
//     stripe's own 8 columns of the pivots as they were BEFORE the stage.
//     With Dg* closed, C' (x) R' = C (x) R' for C' = min(C, C (x) Dg*), and on
//     the pivot columns themselves the update yields C', so one uniform
//     min-plus product per stripe is exactly the blocked sweep's
//     column-panel + remainder update (src/fw_tiling_gpu.cu:253-284 does the
//     same three phases with 32-wide tiles and one launch per phase);
//   * the owner of stripe z + 1 updates that stripe with stage z before
//     anything else and publishes it at once, so the chain the solve waits on
//     is one stripe update, one 8-pivot closure and one stripe panel per
//     stage; the other stripes' updates overlap it.
//
// Stripes therefore see the stages in pivot order, which is the blocked sweep
// with 8-wide pivot blocks: with no negative cycle every value is an exact path
// length or INF and the result is the k-i-j sweep's, bit for bit
// (src/fw_baseline_cpu.cpp:6-15).
//
// Waits. A consumer's thread 0 polls flag z with ld.acquire.gpu, bounded by
// the global timer; a wait that runs out adds one to the call's status word,
// and the CTA leaves (its stripes unwritten; the status word says the result
// is not valid). CTAs only wait for lower stages, stage 0 needs no wait, and
// the cooperative launch guarantees that every CTA is resident, so a correct
// build never waits long; the bound only keeps a fault from hanging the GPU.
#include <cuda_runtime.h>

#include <string>

#include "fw_common.cuh"
#include "fw_internal.h"

namespace fw {

namespace {

constexpr int kStripeRows = 8;  // rows per stripe = pivots per stage
constexpr int kStripeVec = 4;   // columns per thread
constexpr int kStripeMaxSlots = 2;
// A flag wait gives up after this long (a correct solve waits microseconds).
constexpr unsigned long long kStripeWaitNs = 2000000000ull;
// ... and after this many polls whatever the timer says (each poll is an L2
// round trip of a few hundred nanoseconds).
constexpr unsigned kStripeMaxPolls = 1u << 24;

template <int S>
struct StripeCfg;
template <>
struct StripeCfg<1> {
    static constexpr int kMaxThreads = 320;
};
template <>
struct StripeCfg<2> {
    static constexpr int kMaxThreads = 512;  // 128 registers: two stripes without spills
};

// Micro-tile columns (of the thread's 4) whose pivot pairs use two DPX
// add-mins (form A of relax2); the others use two FMA-pipe multiply-adds and
// a three-way DPX min.
constexpr unsigned kStripeColsA = (1u << 0) | (1u << 2);

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Polls *flag until it is nonzero; false once `limit_ns` have passed.
__device__ bool wait_flag(const unsigned* flag, unsigned long long limit_ns) {
    if (ld_acquire_gpu(flag)) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned it = 1; it < kStripeMaxPolls; ++it) {
        if (ld_acquire_gpu(flag)) return true;
        if ((it & 63u) == 0 && global_ns() - t0 > limit_ns) return false;
    }
    return false;
}

__device__ __forceinline__ int4 ld_cg4(const int* p) { return __ldcg(reinterpret_cast<const int4*>(p)); }

__device__ __forceinline__ int lane_of(const int4& v, int e) {
    return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w;
}

// acc = min(acc, C (x) P) for one stripe: C the stripe's 8 values of the
// stage's pivot columns per row (shared memory, row-major [8][8]), P the
// stage's 8 published pivot rows at this thread's 4 columns (global, read
// through L2). ONE_SHOT issues all 8 row loads at once (one L2 round trip on
// the critical path); otherwise they come in two halves of 4 rows, which
// keeps the registers of a two-stripe CTA low.
template <bool ONE_SHOT>
__device__ __forceinline__ void stripe_update(int (&acc)[kStripeRows][kStripeVec], const int* cs, const int* prow,
                                              int ldw, int one) {
    constexpr int kRowsPerLoad = ONE_SHOT ? kStripeRows : kStripeRows / 2;
#pragma unroll
    for (int kh = 0; kh < kStripeRows; kh += kRowsPerLoad) {
        int4 p[kRowsPerLoad];
#pragma unroll
        for (int kk = 0; kk < kRowsPerLoad; ++kk) p[kk] = ld_cg4(prow + (int64_t)(kh + kk) * ldw);
#pragma unroll
        for (int r = 0; r < kStripeRows; ++r) {
#pragma unroll
            for (int k4 = 0; k4 < kRowsPerLoad; k4 += 4) {
                const int4 c = *reinterpret_cast<const int4*>(cs + r * kStripeRows + kh + k4);
#pragma unroll
                for (int e = 0; e < kStripeVec; ++e) {
                    const bool fa = ((kStripeColsA >> e) & 1u) != 0;
                    int v = relax2(fa, acc[r][e], c.x, lane_of(p[k4], e), c.y, lane_of(p[k4 + 1], e), one);
                    acc[r][e] = relax2(fa, v, c.z, lane_of(p[k4 + 2], e), c.w, lane_of(p[k4 + 3], e), one);
                }
            }
        }
    }
}

// Closes this CTA's stripe z (held in acc) and publishes it: Dg (the stripe's
// pivot columns, held by threads 2z and 2z + 1) -> shared memory, closure by
// the warp of those threads, the panel R' = min(R, Dg* (x) R) (PAIRS: from a copy of R, pivot
// pairs on both pipes; otherwise an in-place sweep without the copy's
// registers), R' -> the workspace, then flag z. Called by every thread of
// the CTA.
template <bool PAIRS>
__device__ __forceinline__ void stripe_close_publish(int (&acc)[kStripeRows][kStripeVec], int z, int* dgt,
                                                     int* piv, int ldw, unsigned* flags, int one) {
    const int t = threadIdx.x;
    // The warp that holds Dg (threads 2z and 2z + 1, one warp) closes it:
    // dgt[k][i] = Dg[i][k] (the block transposed, so that column k of Dg* is
    // one row), then per pivot lane (i, j), i < 4, relaxes Dg[i][j] (lo) and
    // Dg[i + 4][j] (hi) from shuffled copies of row and column k.
    if ((t >> 5) == ((2 * z) >> 5)) {
        if ((t >> 1) == z) {
            const int h = (t & 1) * kStripeVec;
#pragma unroll
            for (int e = 0; e < kStripeVec; ++e)
#pragma unroll
                for (int r = 0; r < kStripeRows; ++r) dgt[(h + e) * kStripeRows + r] = acc[r][e];
        }
        __syncwarp();
        const int lane = t & 31, i = lane >> 3, j = lane & 7;
        int lo = dgt[j * kStripeRows + i], hi = dgt[j * kStripeRows + i + 4];
#pragma unroll
        for (int k = 0; k < kStripeRows; ++k) {
            const int a_lo = __shfl_sync(0xffffffffu, lo, (i << 3) | k);
            const int a_hi = __shfl_sync(0xffffffffu, hi, (i << 3) | k);
            const int b = k < 4 ? __shfl_sync(0xffffffffu, lo, (k << 3) | j)
                                : __shfl_sync(0xffffffffu, hi, ((k - 4) << 3) | j);
            lo = __viaddmin_s32(a_lo, b, lo);
            hi = __viaddmin_s32(a_hi, b, hi);
        }
        __syncwarp();
        dgt[j * kStripeRows + i] = lo;
        dgt[j * kStripeRows + i + 4] = hi;
    }
    __syncthreads();
    if constexpr (PAIRS) {
        // R' = min(R, Dg* (x) R) from a copy of R, two pivots per step over
        // both integer pipes (relax2).
        int rr[kStripeRows][kStripeVec];
#pragma unroll
        for (int r = 0; r < kStripeRows; ++r)
#pragma unroll
            for (int e = 0; e < kStripeVec; ++e) rr[r][e] = acc[r][e];
#pragma unroll
        for (int r = 0; r < kStripeRows; ++r) {
            // row r of Dg*: dgt[k][r] for k = 0..7
            int g[kStripeRows];
#pragma unroll
            for (int k = 0; k < kStripeRows; ++k) g[k] = dgt[k * kStripeRows + r];
#pragma unroll
            for (int k = 0; k < kStripeRows; k += 2)
#pragma unroll
                for (int e = 0; e < kStripeVec; ++e)
                    acc[r][e] = relax2(((kStripeColsA >> e) & 1u) != 0, acc[r][e], g[k], rr[k][e], g[k + 1],
                                       rr[k + 1][e], one);
        }
    } else {
        // R' = min(R, Dg* (x) R), in place over the pivots: pivot k relaxes
        // every row through row k (exact, because Dg* is closed: every value
        // it can produce is at least min(R, Dg* (x) R), and pivot k alone
        // reaches Dg*[i][k] + R[k]).
#pragma unroll
        for (int k = 0; k < kStripeRows; ++k) {
            const int4 g0 = *reinterpret_cast<const int4*>(dgt + k * kStripeRows);
            const int4 g1 = *reinterpret_cast<const int4*>(dgt + k * kStripeRows + 4);
            const int g[kStripeRows] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
            int rk[kStripeVec];
#pragma unroll
            for (int e = 0; e < kStripeVec; ++e) rk[e] = acc[k][e];
#pragma unroll
            for (int r = 0; r < kStripeRows; ++r)
#pragma unroll
                for (int e = 0; e < kStripeVec; ++e) acc[r][e] = __viaddmin_s32(g[r], rk[e], acc[r][e]);
        }
    }
    // The diagonal block itself is Dg*, as the closure left it (the same
    // values the sweep above produces there unless a cycle is negative; with
    // one, this keeps a graph of n <= 8 equal to the k-sequential closure).
    if ((t >> 1) == z) {
        const int h = (t & 1) * kStripeVec;
#pragma unroll
        for (int e = 0; e < kStripeVec; ++e)
#pragma unroll
            for (int r = 0; r < kStripeRows; ++r) acc[r][e] = dgt[(h + e) * kStripeRows + r];
    }
    int* dst = piv + (int64_t)z * kStripeRows * ldw + kStripeVec * t;
#pragma unroll
    for (int r = 0; r < kStripeRows; ++r)
        *reinterpret_cast<int4*>(dst + (int64_t)r * ldw) = make_int4(acc[r][0], acc[r][1], acc[r][2], acc[r][3]);
    // The barrier orders every thread's row stores before thread 0's release
    // store of the flag, and the release (gpu scope, cumulative) makes them
    // visible to any CTA that acquires the flag.
    __syncthreads();
    if (t == 0) st_release_gpu(flags + z, 1u);
}

template <int S, bool VEC>
__global__ void __launch_bounds__(StripeCfg<S>::kMaxThreads, 1)
    fw_stripe_kernel(int* __restrict__ D, int n, int ns, int ldw, int* __restrict__ piv, unsigned* __restrict__ flags,
                     unsigned* __restrict__ faults, int one, unsigned long long wait_ns) {
    __shared__ __align__(16) int cs[2][S][kStripeRows * kStripeRows];
    __shared__ __align__(16) int dgt[kStripeRows * kStripeRows];
    const int G = gridDim.x, cta = blockIdx.x, t = threadIdx.x;
    const int c0 = kStripeVec * t;
    int acc[S][kStripeRows][kStripeVec];
#pragma unroll
    for (int q = 0; q < S; ++q) {
        const int z = cta + q * G;
#pragma unroll
        for (int r = 0; r < kStripeRows; ++r) {
            const int row = z * kStripeRows + r;
            const bool in = z < ns && row < n;
            const int* src = D + (int64_t)row * n + c0;
            if (VEC) {
                int4 v = make_int4(kInf, kInf, kInf, kInf);
                if (in && c0 < n) v = *reinterpret_cast<const int4*>(src);
                acc[q][r][0] = v.x; acc[q][r][1] = v.y; acc[q][r][2] = v.z; acc[q][r][3] = v.w;
            } else {
#pragma unroll
                for (int e = 0; e < kStripeVec; ++e) acc[q][r][e] = (in && c0 + e < n) ? src[e] : kInf;
            }
        }
    }
    if (cta == 0) stripe_close_publish<S == 1>(acc[0], 0, dgt, piv, ldw, flags, one);
    for (int s = 0; s < ns; ++s) {
        const int buf = s & 1;
        const int own_s = (s % G == cta) ? s / G : -1;  // slot holding pivot stripe s
        const int nx = s + 1;
        const int own_n = (nx < ns && nx % G == cta) ? nx / G : -1;  // slot holding stripe s + 1
        // The stage's pivot columns of every other slot, before the stage.
        if ((t >> 1) == s) {
            const int h = (t & 1) * kStripeVec;
#pragma unroll
            for (int q = 0; q < S; ++q) {
                if (q == own_s) continue;
#pragma unroll
                for (int r = 0; r < kStripeRows; ++r)
                    *reinterpret_cast<int4*>(&cs[buf][q][r * kStripeRows + h]) =
                        make_int4(acc[q][r][0], acc[q][r][1], acc[q][r][2], acc[q][r][3]);
            }
        }
        int missed = 0;
        if (own_s < 0 && t == 0 && !wait_flag(flags + s, wait_ns)) {
            atomicAdd(faults, 1u);
            missed = 1;
        }
        // The stage barrier, which also tells every thread whether the wait ran out.
        if (__syncthreads_or(missed)) return;
        const int* prow = piv + (int64_t)s * kStripeRows * ldw + c0;
        // The next stage's stripe first: the rest of the solve waits for it.
#pragma unroll
        for (int q = 0; q < S; ++q) {
            if (q != own_n) continue;
            stripe_update<S == 1>(acc[q], cs[buf][q], prow, ldw, one);
            stripe_close_publish<S == 1>(acc[q], nx, dgt, piv, ldw, flags, one);
        }
#pragma unroll
        for (int q = 0; q < S; ++q) {
            if (q == own_s || q == own_n || cta + q * G >= ns) continue;
            stripe_update<S == 1>(acc[q], cs[buf][q], prow, ldw, one);
        }
    }
#pragma unroll
    for (int q = 0; q < S; ++q) {
        const int z = cta + q * G;
        if (z >= ns) continue;
#pragma unroll
        for (int r = 0; r < kStripeRows; ++r) {
            const int row = z * kStripeRows + r;
            if (row >= n || c0 >= n) continue;
            int* dst = D + (int64_t)row * n + c0;
            if (VEC) {
                *reinterpret_cast<int4*>(dst) = make_int4(acc[q][r][0], acc[q][r][1], acc[q][r][2], acc[q][r][3]);
            } else {
#pragma unroll
                for (int e = 0; e < kStripeVec; ++e)
                    if (c0 + e < n) dst[e] = acc[q][r][e];
            }
        }
    }
}

struct StripeGeom {
    int ns;   // stripes
    int thr;  // threads per CTA (4 columns each)
    int ldw;  // leading dimension of the published rows
};

StripeGeom stripe_geom(int64_t n) {
    StripeGeom g;
    g.ns = (int)((n + kStripeRows - 1) / kStripeRows);
    // 2 * ns threads cover the 8 * ns columns of the padded matrix.
    g.thr = 32 * ((2 * g.ns + 31) / 32);
    g.ldw = kStripeVec * g.thr;
    return g;
}

// *launched = false (and FW_OK) when the device refuses the cooperative grid
// (for instance when another process limits the SMs this one may use).
template <int S, bool VEC>
int stripe_launch(int32_t* D, int64_t n, const StripeGeom& g, int grid, int* piv, unsigned* flags, unsigned* faults,
                  cudaStream_t s, bool* launched) {
    *launched = false;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)g.thr);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    prof_begin(KC_STRIPE, s);
    const cudaError_t e = cudaLaunchKernelEx(&cfg, fw_stripe_kernel<S, VEC>, (int*)D, (int)n, g.ns, g.ldw, piv, flags,
                                             faults, 1, kStripeWaitNs);
    if (e == cudaErrorCooperativeLaunchTooLarge) {
        cudaGetLastError();
        return FW_OK;
    }
    if (e != cudaSuccess) return cuda_error(e, "fw_stripe_kernel (cooperative launch)");
    prof_end(KC_STRIPE, s, (double)n * (double)n * (double)n);
    *launched = true;
    return FW_OK;
}

// CTAs of this kernel that fit on the device at once (cooperative limit).
template <int S, bool VEC>
int resident_ctas(int threads, int* out) {
    int dev = 0, sms = 0, coop = 0, per_sm = 0;
    FW_CUDA_TRY(cudaGetDevice(&dev));
    FW_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    FW_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    FW_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fw_stripe_kernel<S, VEC>, threads, 0));
    *out = coop ? per_sm * sms : 0;
    return FW_OK;
}

template <bool VEC>
int stripe_solve_impl(int32_t* D, int64_t n, void* ws, cudaStream_t s, unsigned* faults, bool* ran) {
    const StripeGeom g = stripe_geom(n);
    int* piv = static_cast<int*>(ws);
    unsigned* flags = reinterpret_cast<unsigned*>(static_cast<char*>(ws) +
                                                  (((size_t)g.ns * kStripeRows * g.ldw * sizeof(int) + 255) & ~size_t(255)));
    int cap1 = 0;
    if (int rc = resident_ctas<1, VEC>(g.thr, &cap1)) return rc;
    if (g.ns <= cap1 && g.thr <= StripeCfg<1>::kMaxThreads) {
        FW_CUDA_TRY(cudaMemsetAsync(flags, 0, (size_t)g.ns * sizeof(unsigned), s));
        return stripe_launch<1, VEC>(D, n, g, g.ns, piv, flags, faults, s, ran);
    }
    int cap2 = 0;
    if (int rc = resident_ctas<2, VEC>(g.thr, &cap2)) return rc;
    if (g.thr <= StripeCfg<2>::kMaxThreads && cap2 > 0 && g.ns <= kStripeMaxSlots * cap2) {
        const int grid = g.ns < cap2 ? g.ns : cap2;
        FW_CUDA_TRY(cudaMemsetAsync(flags, 0, (size_t)g.ns * sizeof(unsigned), s));
        return stripe_launch<2, VEC>(D, n, g, grid, piv, flags, faults, s, ran);
    }
    return FW_OK;  // does not fit this device: the caller runs the blocked sweep
}

}  // namespace

// Word 0: the flag fw_debug_flag_wait waits on (nothing sets it before the
// first wait); word 1: the probe's outcome.
__device__ unsigned int g_flag_probe[2];

namespace {

// Test kernel of fw_debug_flag_wait: the stripe sweep's bounded flag wait on a
// flag that nothing sets, then, once thread 0 has set it, the same wait again.
__global__ void fw_flag_probe_kernel(unsigned long long limit_ns, unsigned* __restrict__ probe) {
    if (threadIdx.x != 0) return;
    const bool got = wait_flag(probe, limit_ns);
    st_release_gpu(probe, 1u);
    const bool after = wait_flag(probe, limit_ns);
    probe[1] = (got ? 0u : 1u) | (after ? 2u : 0u);
}

}  // namespace

size_t stripe_workspace_bytes(int64_t n) {
    if (n < 1 || n > kStripeMaxN) return 0;
    const StripeGeom g = stripe_geom(n);
    return (((size_t)g.ns * kStripeRows * g.ldw * sizeof(int) + 255) & ~size_t(255)) +
           (((size_t)g.ns * sizeof(unsigned) + 255) & ~size_t(255));
}

int stripe_solve(int32_t* D, int64_t n, void* ws, cudaStream_t s, unsigned* faults, bool* ran) {
    *ran = false;
    if (n < 1 || n > kStripeMaxN) return FW_OK;
    return (n % 4) == 0 ? stripe_solve_impl<true>(D, n, ws, s, faults, ran)
                        : stripe_solve_impl<false>(D, n, ws, s, faults, ran);
}

}  // namespace fw

extern "C" int fw_debug_flag_wait(int64_t limit_us, fw_stream_t stream) {
    if (limit_us < 1 || limit_us > 1000000)
        return fw::set_error(FW_ERR_INVALID_ARGUMENT, "fw_debug_flag_wait: limit_us must be in [1, 1000000]");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned int* probe = nullptr;
    FW_CUDA_TRY(cudaGetSymbolAddress(reinterpret_cast<void**>(&probe), fw::g_flag_probe));
    FW_CUDA_TRY(cudaMemsetAsync(probe, 0, 2 * sizeof(unsigned int), s));
    fw::fw_flag_probe_kernel<<<1, 32, 0, s>>>((unsigned long long)limit_us * 1000ull, probe);
    FW_LAUNCH_CHECK("fw_flag_probe_kernel");
    FW_CUDA_TRY(cudaStreamSynchronize(s));
    unsigned int v = 0;
    FW_CUDA_TRY(cudaMemcpy(&v, probe + 1, sizeof(v), cudaMemcpyDeviceToHost));
    if (!(v & 2u))
        return fw::set_error(FW_ERR_INTERNAL, "fw_debug_flag_wait: a flag that was set was not seen");
    if (v & 1u)
        return fw::set_error(FW_ERR_TIMEOUT, "fw_debug_flag_wait: the bounded flag wait gave up after " +
                                                 std::to_string(limit_us) + " us (nothing set the flag)");
    return FW_OK;
}

// Out-of-core int32 Floyd-Warshall: the matrix stays in host memory and
// streams through the GPU in row stripes, for matrices larger than the
// device's memory. No counterpart in the reference, which caps n at
// MAX_N = 32769 (include/constants.h:5) and copies the whole matrix to the
// device before a solve (src/gpu_memory.cu:13-16).
//
// One pass per W pivots P = [p0, p0 + W) (W a multiple of 128):
//   1. R = D[P][:] and the column stripe D[:][P] are copied to the device; the
//      column stripe is transposed into CT (CT[k][i] = D[i][p0 + k]).
//   2. Dg = D[P][P] is closed by the in-core sweep (Dg*).
//   3. R2 = min(R, Dg* (x) R) and CT2 = min(CT, Dg*^T (x) CT) — the row and
//      column panels of the pass, as min-plus products (Dg* is closed, so
//      neither depends on a k order).
//   4. Every row stripe D[I][:] goes host -> device; its tiles outside the
//      rows and columns of P become min(D[I][J], CT2[:, I]^T (x) R2[:, J]),
//      its columns in P take the column panel (CT2 transposed back) and its
//      rows in P the row panel R2; then it goes back. These are the values
//      of the in-core sweep after the same pivots, so the result is
//      bit-identical to it and to the k-i-j sweep of
//      src/fw_baseline_cpu.cpp:6-15, and the relaxations done are n^3 plus
//      the W^3 of each diagonal closure.
// Three stripe buffers rotate over a copy-in stream, the caller's stream
// (compute) and a copy-out stream, so the host transfers of one stripe
// overlap the update of the next. A pass moves 8 n^2 bytes over the host link
// for W n^2 relaxations, so the pass width sets the compute-to-transfer ratio.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "fw_common.cuh"
#include "fw_internal.h"
#include "fw_tile.cuh"
#include "fw_tma.cuh"

namespace fw {

// Update-kernel tile copies that missed their bounded wait (see fw_copy_faults).
__device__ unsigned int g_ooc_copy_faults = 0;

namespace {

// Form-A columns of the stripe update (see kColsA).
constexpr unsigned kOocColsA = cols_below(5);

__global__ void fw_ooc_fill_kernel(int* __restrict__ p, int64_t count) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = kInf;
}

// dst[k][i] = src[i][k] for i < rows, k < cols (32 x 32 tiles through shared
// memory; the +1 column keeps the transposed reads free of bank conflicts).
__global__ void fw_ooc_transpose_kernel(const int* __restrict__ src, int64_t lds, int* __restrict__ dst, int64_t ldd,
                                        int64_t rows, int64_t cols) {
    __shared__ int t[32][33];
    const int64_t i0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int64_t i = i0 + y, k = k0 + threadIdx.x;
        if (i < rows && k < cols) t[y][threadIdx.x] = src[i * lds + k];
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int64_t k = k0 + y, i = i0 + threadIdx.x;
        if (i < rows && k < cols) dst[k * ldd + i] = t[threadIdx.x][y];
    }
}

// The thread's 8 x 8 micro-tile of the 128 x 128 tile at (r0, c0) of an
// M x N matrix with leading dimension ldc; INF outside.
template <bool VEC>
__device__ __forceinline__ void ooc_load_acc(int (&acc)[8][8], const int* __restrict__ C, int64_t ldc, int64_t M,
                                             int64_t N, int64_t r0, int64_t c0, int tx, int ty) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int64_t gr = r0 + own_row(ty, r);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int64_t gc = c0 + h * 64 + tx * 4;
            if (VEC) {
                int4 t = make_int4(kInf, kInf, kInf, kInf);
                if (gr < M && gc < N) t = *reinterpret_cast<const int4*>(C + gr * ldc + gc);
                acc[r][h * 4 + 0] = t.x; acc[r][h * 4 + 1] = t.y;
                acc[r][h * 4 + 2] = t.z; acc[r][h * 4 + 3] = t.w;
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    acc[r][h * 4 + e] = (gr < M && gc + e < N) ? C[gr * ldc + gc + e] : kInf;
            }
        }
    }
}

template <bool VEC>
__device__ __forceinline__ void ooc_store_acc(const int (&acc)[8][8], int* __restrict__ C, int64_t ldc, int64_t M,
                                              int64_t N, int64_t r0, int64_t c0, int tx, int ty) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int64_t gr = r0 + own_row(ty, r);
        if (gr >= M) continue;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int64_t gc = c0 + h * 64 + tx * 4;
            if (VEC) {
                if (gc < N)
                    *reinterpret_cast<int4*>(C + gr * ldc + gc) =
                        make_int4(acc[r][h * 4 + 0], acc[r][h * 4 + 1], acc[r][h * 4 + 2], acc[r][h * 4 + 3]);
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (gc + e < N) C[gr * ldc + gc + e] = acc[r][h * 4 + e];
            }
        }
    }
}

// Tile rows [x0, x1) (or columns) left out of an update.
struct TileGap {
    int64_t x0, x1;
};
__device__ __forceinline__ int64_t skip_gap(int64_t idx, const TileGap& g) { return idx < g.x0 ? idx : idx + (g.x1 - g.x0); }

// C[i][j] = min(C[i][j], min_k A[k][i] + B[k][j]) for i < M, j < N and
// k < 32 * nslab, over the 128 x 128 tiles outside the row gap and the column
// gap. A and B are k-major panels behind 2-D tensor maps whose extents cover
// whole 128-wide tiles (INF where there is no value); their 32-row slabs
// arrive by TMA into the 3-stage ring, one mbarrier per stage, the stage and
// parity count running across the tiles a persistent CTA takes. The main loop
// is the in-core remainder's. A copy that misses its bounded wait is counted
// in `faults` (the call's status word) and g_ooc_copy_faults; the CTA then
// waits for the copies it issued and leaves that tile and the rest of its
// share as they were.
template <bool VEC>
__global__ void __launch_bounds__(kThreads, 2)
    fw_ooc_update_kernel(int* __restrict__ C, int64_t ldc, int64_t M, int64_t N,
                         const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, int nslab,
                         TileGap rgap, TileGap cgap, int one, unsigned* __restrict__ faults) {
    extern __shared__ __align__(128) int smem[];
    __shared__ __align__(8) uint64_t bars[kStages];
    __shared__ int s_ok;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    if (tid == 0) {
        s_ok = (smem_u32(smem) & 127u) == 0;
        for (int i = 0; i < kStages; ++i) mbar_init(&bars[i], 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (!s_ok) {  // no copy can be issued: the CTA's tiles keep their values
        if (tid == 0) count_copy_fault(&g_ooc_copy_faults, faults);
        return;
    }
    int g = 0;
    const int64_t tn = (N + kTile - 1) / kTile - (cgap.x1 - cgap.x0);
    const int64_t ntiles = ((M + kTile - 1) / kTile - (rgap.x1 - rgap.x0)) * tn;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t r0 = skip_gap(t / tn, rgap) * kTile, c0 = skip_gap(t % tn, cgap) * kTile;
        auto issue = [&](int j) {
            if (tid == 0) {
                const int stg = (g + j) % kStages;
                int* dst = smem + stg * kStageInts;
                mbar_expect_tx(&bars[stg], (uint32_t)kStageInts * 4);
                tma_load_2d(dst, &mapA, (int)r0, j * kSlab, &bars[stg]);
                tma_load_2d(dst + kSlabInts, &mapB, (int)c0, j * kSlab, &bars[stg]);
            }
        };
        int acc[8][8];
        ooc_load_acc<VEC>(acc, C, ldc, M, N, r0, c0, tx, ty);
#pragma unroll
        for (int j = 0; j < kStages - 1; ++j)
            if (j < nslab) issue(j);
        for (int kb = 0; kb < nslab; ++kb) {
            const int stg = (g + kb) % kStages;
            // every thread is past slab kb - 1 (its stage can be refilled), and
            // all agree whether slab kb arrived
            if (!ring_wait_all(&bars[stg], (uint32_t)(((g + kb) / kStages) & 1))) {
                if (tid == 0) count_copy_fault(&g_ooc_copy_faults, faults);
                ring_drain(bars, kStages, g + kb, g + min(kb + kStages - 2, nslab - 1));
                return;
            }
            if (kb + kStages - 1 < nslab) issue(kb + kStages - 1);
            const int* st = smem + stg * kStageInts;
            relax_slab<kOocColsA>(acc, st, st + kSlabInts, tx, ty, one);
        }
        g += nslab;
        ooc_store_acc<VEC>(acc, C, ldc, M, N, r0, c0, tx, ty);
        __syncthreads();  // the next tile's prologue refills the ring
    }
}

constexpr int kStripeBuffers = 3;

// Adds the status word of one in-core sweep into the call's own.
__global__ void fw_ooc_add_status_kernel(const unsigned* __restrict__ src, unsigned* __restrict__ dst) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *dst += *src;
}

// Device buffers, streams and events of one call; released by the destructor
// on every return path.
struct OocState {
    int* R = nullptr;     // Wp x ldp: the pass's pivot rows, INF padded
    int* R2 = nullptr;    // Wp x ldp: row panel
    int* CT = nullptr;    // Wp x ldp: pivot columns, transposed
    int* CT2 = nullptr;   // Wp x ldp: column panel, transposed
    int* Cst = nullptr;   // n x Wp: pivot columns as copied from the host
    int* Dg = nullptr;    // w x w: diagonal block, contiguous, closed in place
    int* DgK = nullptr;   // Wp x Wp: Dg* row-major, INF padded
    int* DgT = nullptr;   // Wp x Wp: Dg* transposed, INF padded
    unsigned* faults = nullptr;  // the call's status word: missed tile copies
    int* buf[kStripeBuffers] = {};
    cudaStream_t in = nullptr, out = nullptr;
    cudaEvent_t ev_in[kStripeBuffers] = {}, ev_comp[kStripeBuffers] = {}, ev_out[kStripeBuffers] = {};
    cudaEvent_t ev_panels = nullptr, ev_pass_out = nullptr;
    void* registered = nullptr;

    ~OocState() {
        if (in) cudaStreamSynchronize(in);
        if (out) cudaStreamSynchronize(out);
        for (int* p : {R, R2, CT, CT2, Cst, Dg, DgK, DgT})
            if (p) cudaFree(p);
        if (faults) cudaFree(faults);
        for (int b = 0; b < kStripeBuffers; ++b) {
            if (buf[b]) cudaFree(buf[b]);
            for (cudaEvent_t e : {ev_in[b], ev_comp[b], ev_out[b]})
                if (e) cudaEventDestroy(e);
        }
        for (cudaEvent_t e : {ev_panels, ev_pass_out})
            if (e) cudaEventDestroy(e);
        if (in) cudaStreamDestroy(in);
        if (out) cudaStreamDestroy(out);
        if (registered) cudaHostUnregister(registered);
    }
};

int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

int fill_inf(int* p, int64_t count, cudaStream_t s) {
    const int64_t blocks = std::min<int64_t>((count + 255) / 256, 4096);
    fw_ooc_fill_kernel<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, s>>>(p, count);
    FW_LAUNCH_CHECK("fw_ooc_fill_kernel");
    return FW_OK;
}

int transpose(const int* src, int64_t lds, int* dst, int64_t ldd, int64_t rows, int64_t cols, cudaStream_t s) {
    const dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
    fw_ooc_transpose_kernel<<<grid, dim3(32, 8), 0, s>>>(src, lds, dst, ldd, rows, cols);
    FW_LAUNCH_CHECK("fw_ooc_transpose_kernel");
    return FW_OK;
}

// A: k-major panel of panel_rows rows, leading dimension lda, of which the
// a_cols columns from A are valid addresses (the same for B).
int update(int* C, int64_t ldc, int64_t M, int64_t N, const int* A, int64_t lda, int64_t a_cols, const int* B,
           int64_t ldb, int64_t b_cols, int64_t panel_rows, int64_t kvalid, int64_t resident, unsigned* faults,
           cudaStream_t s, TileGap rgap = {0, 0}, TileGap cgap = {0, 0}) {
    const int64_t tiles = ((M + kTile - 1) / kTile - (rgap.x1 - rgap.x0)) * ((N + kTile - 1) / kTile - (cgap.x1 - cgap.x0));
    if (tiles <= 0) return FW_OK;
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, resident);
    const int nslab = (int)((kvalid + kSlab - 1) / kSlab);
    // 16-byte accesses need aligned rows and whole vectors inside [0, N).
    const bool vec = (ldc % 4) == 0 && (N % 4) == 0 && (reinterpret_cast<uintptr_t>(C) & 15u) == 0;
    CUtensorMap mapA, mapB;
    if (int rc = panel_map_ld(&mapA, A, (uint64_t)a_cols, (uint64_t)lda, (uint64_t)panel_rows, kTile)) return rc;
    if (int rc = panel_map_ld(&mapB, B, (uint64_t)b_cols, (uint64_t)ldb, (uint64_t)panel_rows, kTile)) return rc;
    prof_begin(KC_OOC_UPDATE, s);
    if (vec)
        fw_ooc_update_kernel<true>
            <<<grid, kThreads, kSmemBytes, s>>>(C, ldc, M, N, mapA, mapB, nslab, rgap, cgap, 1, faults);
    else
        fw_ooc_update_kernel<false>
            <<<grid, kThreads, kSmemBytes, s>>>(C, ldc, M, N, mapA, mapB, nslab, rgap, cgap, 1, faults);
    FW_LAUNCH_CHECK("fw_ooc_update_kernel");
    const double rows = (double)M - std::min<double>((double)M, (double)(rgap.x1 - rgap.x0) * kTile);
    const double cols = (double)N - std::min<double>((double)N, (double)(cgap.x1 - cgap.x0) * kTile);
    prof_end(KC_OOC_UPDATE, s, std::max(rows, 0.0) * std::max(cols, 0.0) * (double)kvalid);
    return FW_OK;
}

}  // namespace

size_t ooc_device_bytes(int64_t n, int64_t W, int64_t H) {
    const int64_t ldp = round_up(n, kTile);
    const int64_t Wp = round_up(W, kTile);
    return sizeof(int) * ((size_t)4 * Wp * ldp + (size_t)n * Wp + (size_t)W * W + (size_t)2 * Wp * Wp +
                          (size_t)kStripeBuffers * H * n);
}

int ooc_solve(int32_t* h_D, int64_t n, int64_t W, int64_t H, cudaStream_t s) {
    static PerDeviceOnce attrs;
    if (int rc = once_per_device(attrs, [] {
            FW_CUDA_TRY(
                cudaFuncSetAttribute(fw_ooc_update_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
            FW_CUDA_TRY(cudaFuncSetAttribute(fw_ooc_update_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kSmemBytes));
            return (int)FW_OK;
        }))
        return rc;
    int dev = 0, sms = 0;
    FW_CUDA_TRY(cudaGetDevice(&dev));
    FW_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t resident = 2 * (int64_t)(sms > 0 ? sms : 152);

    const int64_t ldp = round_up(n, kTile);
    const int64_t Wp = round_up(W, kTile);
    const size_t bytes = sizeof(int) * (size_t)n * (size_t)n;
    OocState st;

    // Page-locked host memory makes the stripe copies asynchronous; pageable
    // memory is registered for the call when the driver allows it, and is
    // otherwise copied through the driver's staging buffers.
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, h_D) != cudaSuccess || pa.type != cudaMemoryTypeHost) {
        cudaGetLastError();
        if (cudaHostRegister(h_D, bytes, cudaHostRegisterDefault) == cudaSuccess)
            st.registered = h_D;
        else
            cudaGetLastError();
    }

    auto alloc = [&](int** p, size_t count) -> int {
        if (cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            return set_error(FW_ERR_NO_MEMORY, "fw_apsp_i32_host: device allocation of " +
                                                   std::to_string(count * sizeof(int)) + " bytes failed");
        }
        return FW_OK;
    };
    for (int** p : {&st.R, &st.R2, &st.CT, &st.CT2})
        if (int rc = alloc(p, (size_t)Wp * ldp)) return rc;
    if (int rc = alloc(&st.Cst, (size_t)n * Wp)) return rc;
    if (int rc = alloc(&st.Dg, (size_t)W * W)) return rc;
    if (int rc = alloc(&st.DgK, (size_t)Wp * Wp)) return rc;
    if (int rc = alloc(&st.DgT, (size_t)Wp * Wp)) return rc;
    for (int b = 0; b < kStripeBuffers; ++b)
        if (int rc = alloc(&st.buf[b], (size_t)H * n)) return rc;
    if (cudaMalloc(reinterpret_cast<void**>(&st.faults), sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        return set_error(FW_ERR_NO_MEMORY, "fw_apsp_i32_host: device allocation of the status word failed");
    }
    FW_CUDA_TRY(cudaMemsetAsync(st.faults, 0, sizeof(unsigned), s));
    FW_CUDA_TRY(cudaStreamCreateWithFlags(&st.in, cudaStreamNonBlocking));
    FW_CUDA_TRY(cudaStreamCreateWithFlags(&st.out, cudaStreamNonBlocking));
    for (int b = 0; b < kStripeBuffers; ++b) {
        FW_CUDA_TRY(cudaEventCreateWithFlags(&st.ev_in[b], cudaEventDisableTiming));
        FW_CUDA_TRY(cudaEventCreateWithFlags(&st.ev_comp[b], cudaEventDisableTiming));
        FW_CUDA_TRY(cudaEventCreateWithFlags(&st.ev_out[b], cudaEventDisableTiming));
    }
    FW_CUDA_TRY(cudaEventCreateWithFlags(&st.ev_panels, cudaEventDisableTiming));
    FW_CUDA_TRY(cudaEventCreateWithFlags(&st.ev_pass_out, cudaEventDisableTiming));

    // Padding: columns >= n of R / CT are never written, rows >= w only in a
    // short last pass, which refills them.
    for (int* p : {st.R, st.CT})
        if (int rc = fill_inf(p, Wp * ldp, s)) return rc;

    int64_t stripe_no = 0;
    for (int64_t p0 = 0; p0 < n; p0 += W) {
        const int64_t w = std::min(W, n - p0);
        // The previous pass's stripes are back in host memory before this
        // pass reads its pivot rows and columns there.
        FW_CUDA_TRY(cudaStreamWaitEvent(s, st.ev_pass_out, 0));
        if (w < Wp && p0 > 0) {
            for (int* p : {st.R, st.CT})
                if (int rc = fill_inf(p, Wp * ldp, s)) return rc;
        }
        FW_CUDA_TRY(cudaMemcpy2DAsync(st.R, ldp * sizeof(int), h_D + p0 * n, n * sizeof(int), n * sizeof(int), w,
                                      cudaMemcpyHostToDevice, s));
        FW_CUDA_TRY(cudaMemcpy2DAsync(st.Cst, Wp * sizeof(int), h_D + p0, n * sizeof(int), w * sizeof(int), n,
                                      cudaMemcpyHostToDevice, s));
        if (int rc = transpose(st.Cst, Wp, st.CT, ldp, n, w, s)) return rc;
        // Close the diagonal block with the in-core sweep.
        FW_CUDA_TRY(cudaMemcpy2DAsync(st.Dg, w * sizeof(int), st.R + p0, ldp * sizeof(int), w * sizeof(int), w,
                                      cudaMemcpyDeviceToDevice, s));
        if (int rc = fw_apsp_i32(st.Dg, w, 32, 8, FW_VARIANT_MULTI_LAYER, reinterpret_cast<fw_stream_t>(s)))
            return rc;
        if (const unsigned* word = last_call_status(s)) {
            fw_ooc_add_status_kernel<<<1, 32, 0, s>>>(word, st.faults);
            FW_LAUNCH_CHECK("fw_ooc_add_status_kernel");
        }
        if (int rc = fill_inf(st.DgK, Wp * Wp, s)) return rc;
        if (int rc = fill_inf(st.DgT, Wp * Wp, s)) return rc;
        FW_CUDA_TRY(cudaMemcpy2DAsync(st.DgK, Wp * sizeof(int), st.Dg, w * sizeof(int), w * sizeof(int), w,
                                      cudaMemcpyDeviceToDevice, s));
        if (int rc = transpose(st.Dg, w, st.DgT, Wp, w, w, s)) return rc;
        // Panels: R2 = min(R, Dg* (x) R), CT2 = min(CT, Dg*^T (x) CT).
        FW_CUDA_TRY(cudaMemcpyAsync(st.R2, st.R, sizeof(int) * Wp * ldp, cudaMemcpyDeviceToDevice, s));
        FW_CUDA_TRY(cudaMemcpyAsync(st.CT2, st.CT, sizeof(int) * Wp * ldp, cudaMemcpyDeviceToDevice, s));
        if (int rc = update(st.R2, ldp, w, n, st.DgT, Wp, Wp, st.R, ldp, ldp, Wp, w, resident, st.faults, s))
            return rc;
        if (int rc = update(st.CT2, ldp, w, n, st.DgK, Wp, Wp, st.CT, ldp, ldp, Wp, w, resident, st.faults, s))
            return rc;
        FW_CUDA_TRY(cudaEventRecord(st.ev_panels, s));
        // Stripes.
        for (int64_t r0 = 0; r0 < n; r0 += H, ++stripe_no) {
            const int64_t h = std::min(H, n - r0);
            const int b = (int)(stripe_no % kStripeBuffers);
            const size_t sb = sizeof(int) * (size_t)h * n;
            FW_CUDA_TRY(cudaStreamWaitEvent(st.in, st.ev_panels, 0));
            FW_CUDA_TRY(cudaStreamWaitEvent(st.in, st.ev_out[b], 0));
            FW_CUDA_TRY(cudaMemcpyAsync(st.buf[b], h_D + r0 * n, sb, cudaMemcpyHostToDevice, st.in));
            FW_CUDA_TRY(cudaEventRecord(st.ev_in[b], st.in));
            FW_CUDA_TRY(cudaStreamWaitEvent(s, st.ev_in[b], 0));
            // tiles outside P's rows and columns: the min-plus update
            const int64_t pr0 = std::max(p0, r0), pr1 = std::min(p0 + w, r0 + h);  // P rows in the stripe
            const TileGap rgap = pr0 < pr1 ? TileGap{(pr0 - r0) / kTile, (pr1 - r0 + kTile - 1) / kTile} : TileGap{0, 0};
            const TileGap cgap{p0 / kTile, (p0 + w + kTile - 1) / kTile};
            if (int rc = update(st.buf[b], n, h, n, st.CT2 + r0, ldp, ldp - r0, st.R2, ldp, ldp, Wp, w, resident,
                                st.faults, s, rgap, cgap))
                return rc;
            // columns of P: the column panel, transposed back
            if (int rc = transpose(st.CT2 + r0, ldp, st.buf[b] + p0, n, w, h, s)) return rc;
            // rows of P: the row panel
            if (pr0 < pr1)
                FW_CUDA_TRY(cudaMemcpy2DAsync(st.buf[b] + (pr0 - r0) * n, n * sizeof(int), st.R2 + (pr0 - p0) * ldp,
                                              ldp * sizeof(int), n * sizeof(int), pr1 - pr0, cudaMemcpyDeviceToDevice,
                                              s));
            FW_CUDA_TRY(cudaEventRecord(st.ev_comp[b], s));
            FW_CUDA_TRY(cudaStreamWaitEvent(st.out, st.ev_comp[b], 0));
            FW_CUDA_TRY(cudaMemcpyAsync(h_D + r0 * n, st.buf[b], sb, cudaMemcpyDeviceToHost, st.out));
            FW_CUDA_TRY(cudaEventRecord(st.ev_out[b], st.out));
        }
        FW_CUDA_TRY(cudaEventRecord(st.ev_pass_out, st.out));
    }
    FW_CUDA_TRY(cudaStreamWaitEvent(s, st.ev_pass_out, 0));
    FW_CUDA_TRY(cudaStreamSynchronize(s));
    unsigned missed = 0;
    FW_CUDA_TRY(cudaMemcpy(&missed, st.faults, sizeof(missed), cudaMemcpyDeviceToHost));
    if (missed)
        return set_error(FW_ERR_TIMEOUT, "fw_apsp_i32_host: " + std::to_string(missed) +
                                             " tile copies did not arrive within their bounded wait; the result is "
                                             "not valid");
    return FW_OK;
}

}  // namespace fw

using namespace fw;

namespace {

constexpr int64_t kDefaultPassWidth = 2048;
constexpr int64_t kMaxHostN = 2000000;  // transpose grid.y = n / 32 < 65536

// Normalised pass width, or -1 when invalid.
int64_t pass_width_of(int64_t n, int64_t w) {
    if (w == 0) w = kDefaultPassWidth;
    if (w < kTile || w % kTile != 0) return -1;
    return std::min(w, round_up(n, kTile));
}

}  // namespace

extern "C" {

size_t fw_host_solve_device_bytes(int64_t n, int64_t pass_width, int64_t stripe_rows) {
    if (n < 1 || n > kMaxHostN || stripe_rows < kTile || stripe_rows % kTile != 0) return 0;
    const int64_t W = pass_width_of(n, pass_width);
    if (W < 0) return 0;
    return ooc_device_bytes(n, W, std::min(stripe_rows, round_up(n, kTile)));
}

int fw_apsp_i32_host(int32_t* h_D, int64_t n, int64_t pass_width, int64_t stripe_rows, fw_stream_t stream) {
    if (h_D == nullptr) return set_error(FW_ERR_INVALID_ARGUMENT, "fw_apsp_i32_host: h_D is NULL");
    if (n < 1 || n > kMaxHostN)
        return set_error(FW_ERR_INVALID_ARGUMENT, "fw_apsp_i32_host: need 1 <= n <= " + std::to_string(kMaxHostN) +
                                                      ", got " + std::to_string(n));
    const int64_t W = pass_width_of(n, pass_width);
    if (W < 0)
        return set_error(FW_ERR_INVALID_ARGUMENT,
                         "fw_apsp_i32_host: pass_width must be 0 or a positive multiple of 128, got " +
                             std::to_string(pass_width));
    int64_t H = stripe_rows;
    if (H == 0) {
        size_t free_b = 0, total_b = 0;
        FW_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
        const double fixed = (double)ooc_device_bytes(n, W, 0);
        double budget = ((double)free_b - fixed - (double)(1ull << 30)) / 2.0;
        budget = std::min(budget, 12.0 * (double)(1ull << 30));
        H = (int64_t)(budget / (3.0 * 4.0 * (double)n)) / kTile * kTile;
        // at least 8 stripes per pass, so the copies of one stripe hide
        // behind the update of the others
        H = std::min(H, round_up((n + 7) / 8, kTile));
        if (H < kTile) H = kTile;
    } else if (H < kTile || H % kTile != 0) {
        return set_error(FW_ERR_INVALID_ARGUMENT,
                         "fw_apsp_i32_host: stripe_rows must be 0 or a positive multiple of 128, got " +
                             std::to_string(stripe_rows));
    }
    H = std::min(H, round_up(n, kTile));
    return ooc_solve(h_D, n, W, H, reinterpret_cast<cudaStream_t>(stream));
}

}  // extern "C"

namespace fw {
unsigned int ooc_copy_faults() {
    unsigned int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_ooc_copy_faults, sizeof(v)) != cudaSuccess) cudaGetLastError();
    return v;
}
}  // namespace fw

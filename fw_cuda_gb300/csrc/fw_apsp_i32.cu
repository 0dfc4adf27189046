// int32 Floyd-Warshall on one GB300: the blocked sweep and the per-pivot sweep.
//
// Blocked sweep (stands in for fwTilingGPU, src/fw_tiling_gpu.cu:253-284, and
// fwMultiLayerTilingGPU, src/fw_multi_layer_tiling_gpu.cu:507-577). For each
// 128-wide pivot block P = [p0, p0 + 128):
//   1. diag      one CTA closes D[P][P] under min-plus (a k-sequential sweep
//                with the pivot row and column double-buffered in shared
//                memory, one barrier per pivot);
//   2. panels    every row-panel tile D[P][J] becomes min(R, Dg* (x) R) and
//                every column-panel tile D[I][P] becomes min(C, C (x) Dg*),
//                where Dg* is the closed diagonal block. Because Dg* is
//                closed these are plain min-plus products with no k-order
//                dependency, so they run as independent 128 x 128 tiles;
//   3. remainder every other tile D[I][J] becomes min(D, C_I (x) R_J).
// The panels are also written to a workspace in the layout the remainder
// reads: the column panel transposed (colT[k][i] = D[i][p0 + k]) and the row
// panel as is (rowP[k][j] = D[p0 + k][j]), both with a leading dimension
// padded to a multiple of 128. Every remainder operand slab is then one
// 32 x 128 box of a 2-D tensor map that the tensor memory accelerator copies
// into shared memory, and the remainder never reads a value another CTA of
// the same launch writes.
//
// With integer weights and no negative cycle every stored value is an exact
// path length below INF or INF itself, so the result does not depend on the
// relaxation order and is bit-identical to the k-i-j sweep of
// src/fw_baseline_cpu.cpp:6-15.
//
// Per-pivot sweep (stands in for fwBaselineGPU, src/fw_baseline_gpu.cu:6-32):
// one launch per pivot k; the pivot row and column are read from a snapshot
// taken by the previous launch, so no launch reads what it writes.
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <utility>

#include "fw_common.cuh"
#include "fw_internal.h"
#include "fw_tile.cuh"
#include "fw_tma.cuh"

namespace fw {

// Tile copies that did not arrive within the bounded wait (a correct build
// never counts one); read by fw_copy_faults.
__device__ unsigned int g_copy_faults = 0;
// Outcome of fw_debug_bounded_wait's kernel: bit 0 the wait gave up, bit 1
// the barrier completed once its transfer count was settled.
__device__ unsigned int g_wait_probe_result = 0;

namespace {

// ------------------------------------------------------------------ kernels
// Phase 1: closure of the pivot block D[P][P] by one CTA of 512 threads, each
// holding a 4 x 8 register block (BlockClosure<128, 32, 16>). Writes the
// closed block back to D and into both workspace panels (transposed into
// colT, as is into rowP).
constexpr int kDiagThreads = 512;
using DiagClosure = BlockClosure<kTile, 32, 16>;

template <bool VEC>
__global__ void __launch_bounds__(kDiagThreads, 1)
    fw_diag_kernel(int* __restrict__ D, int64_t n, int64_t ldp, int64_t p0, int* __restrict__ colT,
                   int* __restrict__ rowP, const unsigned* __restrict__ skip) {
    if (skip && *skip) return;
    __shared__ __align__(16) int prow[2 * kTile];
    __shared__ __align__(16) int pcol[2 * kTile];
    constexpr int RR = DiagClosure::RR, RC = DiagClosure::RC;
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    int c[RR][RC];
    const int* src = D + p0 * n + p0;
    const int64_t rem = n - p0;  // valid rows / columns of the block
#pragma unroll
    for (int r = 0; r < RR; ++r) {
        const int lr = ty * RR + r;
#pragma unroll
        for (int h = 0; h < RC; h += 4) {
            const int lc = tx * RC + h;
            if (VEC) {
                int4 t = make_int4(kInf, kInf, kInf, kInf);
                if (lr < rem && lc < rem) t = *reinterpret_cast<const int4*>(src + lr * n + lc);
                c[r][h] = t.x; c[r][h + 1] = t.y; c[r][h + 2] = t.z; c[r][h + 3] = t.w;
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e) c[r][h + e] = (lr < rem && lc + e < rem) ? src[lr * n + lc + e] : kInf;
            }
        }
    }
    DiagClosure::run(c, prow, pcol, kTile, tx, ty, [] { __syncthreads(); });
    int* dst = D + p0 * n + p0;
#pragma unroll
    for (int r = 0; r < RR; ++r) {
        const int lr = ty * RR + r;
#pragma unroll
        for (int h = 0; h < RC; h += 4) {
            const int lc = tx * RC + h;
            const int4 v = make_int4(c[r][h], c[r][h + 1], c[r][h + 2], c[r][h + 3]);
            if (VEC) {
                if (lr < rem && lc < rem) *reinterpret_cast<int4*>(dst + lr * n + lc) = v;
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (lr < rem && lc + e < rem) dst[lr * n + lc + e] = c[r][h + e];
            }
            *reinterpret_cast<int4*>(rowP + (int64_t)lr * ldp + p0 + lc) = v;
        }
    }
#pragma unroll
    for (int e = 0; e < RC; ++e) {
        int col[RR];
#pragma unroll
        for (int r = 0; r < RR; ++r) col[r] = c[r][e];
        st_vec<RR>(colT + (int64_t)(tx * RC + e) * ldp + p0 + ty * RR, col);
    }
}

// Phase 2: blockIdx.y == 0 -> row-panel tile D[P][J]; == 1 -> column-panel
// tile D[I][P]; blockIdx.x enumerates the tiles other than the pivot tile.
// `one` is the runtime 1 of the FMA-pipe additions (fw_common.cuh).
template <bool VEC>
__global__ void __launch_bounds__(kThreads, 2)
    fw_panel_kernel(int* __restrict__ D, int64_t n, int64_t ldp, int pt, int nslab, int* __restrict__ colT,
                    int* __restrict__ rowP, int one, const unsigned* __restrict__ skip) {
    if (skip && *skip) return;
    extern __shared__ __align__(128) int smem[];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int other = (int)blockIdx.x < pt ? (int)blockIdx.x : (int)blockIdx.x + 1;
    const int64_t p0 = (int64_t)pt * kTile;
    const int64_t q0 = (int64_t)other * kTile;
    int acc[8][8];
    if (blockIdx.y == 0) {
        load_acc<VEC>(acc, D, n, p0, q0, tx, ty);
        mainloop<kColsA>(
            acc, nslab, smem,
            [&](int* dst, int s) { load_kmajor_async(dst, colT, ldp, s * kSlab, p0, tid); },
            [&](int* dst, int s) { load_d_rows<VEC>(dst, D, n, p0 + s * kSlab, q0, tid); }, tx, ty, one);
        store_acc<VEC>(acc, D, n, p0, q0, tx, ty);
        store_acc_ws(acc, rowP, ldp, q0, tx, ty);
    } else {
        load_acc<VEC>(acc, D, n, q0, p0, tx, ty);
        mainloop<kColsA>(
            acc, nslab, smem,
            [&](int* dst, int s) { load_d_transposed<VEC>(dst, D, n, q0, p0 + s * kSlab, tid); },
            [&](int* dst, int s) { load_kmajor_async(dst, rowP, ldp, s * kSlab, p0, tid); }, tx, ty, one);
        store_acc<VEC>(acc, D, n, q0, p0, tx, ty);
        store_acc_ws_transposed(acc, colT, ldp, q0, tx, ty);
    }
}

// Phase 3: tiles (I, J), I from `rows` (nrows of them), J from `cols` (ncols):
// D[I][J] = min(D[I][J], colT[k][I]^T (x) rowP[k][J]) over workspace pivot
// rows k in [slab0 * 32, (slab0 + nslab) * 32). Each CTA walks the tiles
// blockIdx.x, blockIdx.x + gridDim.x, ... in row-major order. The launch
// behind a skip flag is persistent (two CTAs per SM), so when the flag says
// the packed fast path already produced the result it costs only those CTAs;
// otherwise there is one CTA per tile, so that the kernels of a higher
// priority stream can take SMs from it between tiles.
// With cross >= 0 the tiles are instead block `cross`'s update of block
// u = cross + 1's row and column: tiles [0, nrows - 1) are (u, J), J != cross,
// the next nrows - 2 are (I, u), I != cross, u (nrows = T, ncols = 2T - 3).
// A copy that misses its bounded wait is counted in `faults` (the call's
// status word) and in g_copy_faults; the CTA then waits for the copies it
// already issued, leaves that tile and every later tile of its share as they
// were, and returns.
template <bool VEC>
__global__ void __launch_bounds__(kThreads, 2)
    fw_remainder_kernel(int* __restrict__ D, int64_t n, TileSet rows, int nrows, TileSet cols, int ncols, int slab0,
                        int nslab, const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                        int one, const unsigned* __restrict__ skip, int cross, unsigned* __restrict__ faults) {
    if (skip && *skip) return;
    extern __shared__ __align__(128) int smem[];
    __shared__ __align__(8) uint64_t bars[kStages];
    __shared__ int s_ok;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    if (tid == 0) {
        // TMA destinations must be 128-byte aligned; the stage sizes keep every
        // stage and operand aligned when the base is.
        s_ok = (smem_u32(smem) & 127u) == 0;
        for (int i = 0; i < kStages; ++i) mbar_init(&bars[i], 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (!s_ok) {  // no copy can be issued: the CTA's tiles keep their values
        if (tid == 0) count_copy_fault(&g_copy_faults, faults);
        return;
    }
    // Operand slabs, k-major 32 x 128 ints each, by TMA: slab j of the CTA's
    // running count g + j goes to stage (g + j) % kStages, whose barrier
    // completes for the ((g + j) / kStages)-th time.
    int g = 0;
    const int64_t ntiles = cross >= 0 ? (int64_t)ncols : (int64_t)nrows * ncols;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int I, J;
        if (cross < 0) {
            I = tile_of(rows, (int)(t / ncols));
            J = tile_of(cols, (int)(t % ncols));
        } else if (t < nrows - 1) {
            I = cross + 1;
            J = tile_of(all_but(cross), (int)t);
        } else {
            I = tile_of(all_but(cross, cross + 1), (int)t - (nrows - 1));
            J = cross + 1;
        }
        const int r0 = I * kTile, c0 = J * kTile;
        auto issue = [&](int j) {
            if (tid == 0) {
                const int stg = (g + j) % kStages;
                int* dst = smem + stg * kStageInts;
                mbar_expect_tx(&bars[stg], (uint32_t)kStageInts * 4);
                tma_load_2d(dst, &mapA, r0, (slab0 + j) * kSlab, &bars[stg]);
                tma_load_2d(dst + kSlabInts, &mapB, c0, (slab0 + j) * kSlab, &bars[stg]);
            }
        };
        int acc[8][8];
        load_acc<VEC>(acc, D, n, r0, c0, tx, ty);
#pragma unroll
        for (int j = 0; j < kStages - 1; ++j)
            if (j < nslab) issue(j);
        for (int kb = 0; kb < nslab; ++kb) {
            const int stg = (g + kb) % kStages;
            // every thread is past slab kb - 1 (its stage can be refilled), and
            // all agree whether slab kb arrived
            if (!ring_wait_all(&bars[stg], (uint32_t)(((g + kb) / kStages) & 1))) {
                if (tid == 0) count_copy_fault(&g_copy_faults, faults);
                ring_drain(bars, kStages, g + kb, g + min(kb + kStages - 2, nslab - 1));
                return;
            }
            if (kb + kStages - 1 < nslab) issue(kb + kStages - 1);
            const int* st = smem + stg * kStageInts;
            relax_slab<kColsA>(acc, st, st + kSlabInts, tx, ty, one);
        }
        g += nslab;
        store_acc<VEC>(acc, D, n, r0, c0, tx, ty);
        __syncthreads();  // the next tile's prologue refills the ring
    }
}

// Test kernel of fw_debug_bounded_wait: the remainder kernels' bounded wait
// on a barrier whose 16-byte transfer is never issued. Afterwards thread 0
// completes the transfer count itself, so the barrier ends balanced.
__global__ void fw_wait_probe_kernel(int spins, unsigned* __restrict__ result) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_expect_tx(&bar, 16);
    __syncthreads();
    const bool got = mbar_wait(&bar, 0u, spins);
    const bool gave_up = __syncthreads_or(got ? 0 : 1) != 0;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.complete_tx.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bar)), "r"(16u) : "memory");
        const bool after = mbar_wait(&bar, 0u, 1024);
        *result = (gave_up ? 1u : 0u) | (after ? 2u : 0u);
    }
}

// Per-pivot sweep. Prime: snapshot row 0 and column 0.
__global__ void fw_pivot_prime_kernel(const int* __restrict__ D, int64_t n, int* __restrict__ row0,
                                      int* __restrict__ col0) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        row0[j] = D[j];
        col0[j] = D[j * n];
    }
}

// Pivot k over row blockIdx.y: D[i][j] = min(D[i][j], colk[i] + rowk[j]);
// row k + 1 and column k + 1 of the result go to the next snapshot. Stores
// only values that changed. Scalar form, for n % 4 != 0.
__global__ void __launch_bounds__(256)
    fw_pivot_step_kernel(int* __restrict__ D, int64_t n, int64_t k, const int* __restrict__ rowk,
                         const int* __restrict__ colk, int* __restrict__ rown, int* __restrict__ coln) {
    const int64_t i = blockIdx.y;
    const int dik = colk[i];
    int* row = D + i * n;
    const bool next_row = (i == k + 1);
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const int d = row[j];
        const int o = __viaddmin_s32(dik, rowk[j], d);
        if (o != d) row[j] = o;
        if (next_row) rown[j] = o;
        if (j == k + 1) coln[i] = o;
    }
}

// Vector form for n % 4 == 0: a CTA takes kPivRows rows and a chunk of
// 256 * kPivVecs 16-byte vectors of them, so every thread loads its pivot-row
// vectors once for kPivRows rows; 32-bit vector indices, and only the thread
// whose vector holds column k + 1 writes the column snapshot.
constexpr int kPivRows = 4, kPivVecs = 4;
__global__ void __launch_bounds__(256)
    fw_pivot_step_vec_kernel(int* __restrict__ D, int64_t n, int k, const int* __restrict__ rowk,
                             const int* __restrict__ colk, int* __restrict__ rown, int* __restrict__ coln) {
    const int n4 = (int)(n >> 2);
    const int qk1 = (k + 1) >> 2, ek1 = (k + 1) & 3;
    int4 b[kPivVecs];
    int qs[kPivVecs];
#pragma unroll
    for (int v = 0; v < kPivVecs; ++v) {
        qs[v] = (blockIdx.x * kPivVecs + v) * 256 + threadIdx.x;
        if (qs[v] < n4) b[v] = *reinterpret_cast<const int4*>(rowk + 4 * (int64_t)qs[v]);
    }
    // all loads first, so that each thread has kPivRows * kPivVecs 16-byte
    // loads in flight
    int dik[kPivRows];
    int4 d[kPivRows][kPivVecs];
    const int64_t i0 = (int64_t)blockIdx.y * kPivRows;
#pragma unroll
    for (int r = 0; r < kPivRows; ++r) {
        dik[r] = (i0 + r < n) ? colk[i0 + r] : 0;
#pragma unroll
        for (int v = 0; v < kPivVecs; ++v)
            if (i0 + r < n && qs[v] < n4) d[r][v] = *reinterpret_cast<const int4*>(D + (i0 + r) * n + 4 * (int64_t)qs[v]);
    }
#pragma unroll
    for (int r = 0; r < kPivRows; ++r) {
        const int64_t i = i0 + r;
        if (i >= n) break;
        int* row = D + i * n;
        const bool next_row = (i == (int64_t)k + 1);
#pragma unroll
        for (int v = 0; v < kPivVecs; ++v) {
            const int q = qs[v];
            if (q >= n4) continue;
            int4 o;
            o.x = __viaddmin_s32(dik[r], b[v].x, d[r][v].x);
            o.y = __viaddmin_s32(dik[r], b[v].y, d[r][v].y);
            o.z = __viaddmin_s32(dik[r], b[v].z, d[r][v].z);
            o.w = __viaddmin_s32(dik[r], b[v].w, d[r][v].w);
            if (o.x != d[r][v].x || o.y != d[r][v].y || o.z != d[r][v].z || o.w != d[r][v].w)
                *reinterpret_cast<int4*>(row + 4 * (int64_t)q) = o;
            if (next_row) *reinterpret_cast<int4*>(rown + 4 * (int64_t)q) = o;
            if (q == qk1) coln[i] = ek1 == 0 ? o.x : ek1 == 1 ? o.y : ek1 == 2 ? o.z : o.w;
        }
    }
}

template <bool VEC>
struct Blocked {
    int32_t* D;
    int64_t n, ldp;
    int T;
    int* colT;  // [rows_per_pass][ldp]
    int* rowP;
    cudaStream_t s;
    const unsigned* skip;
    unsigned* faults;             // the call's status word (missed copies), may be null
    int64_t resident_ctas = 304;  // CTAs of the persistent remainder: 2 per SM
    AuxStream aux{};
    CUtensorMap mapA{}, mapB{};   // TMA maps over colT and rowP (all panel rows of the workspace)

    int64_t p0(int t) const { return (int64_t)t * kTile; }
    int64_t kv(int t) const { return n - p0(t) < kTile ? n - p0(t) : kTile; }

    // Diagonal closure of block t, its panels written to workspace half h.
    int diag(int t, int h, cudaStream_t q = nullptr) {
        if (q == nullptr) q = s;
        prof_begin(KC_DIAG, q);
        fw_diag_kernel<VEC><<<1, kDiagThreads, 0, q>>>(D, n, ldp, p0(t), colT + h * kTile * ldp, rowP + h * kTile * ldp,
                                                       skip);
        FW_LAUNCH_CHECK("fw_diag_kernel");
        prof_end(KC_DIAG, q, (double)kv(t) * kv(t) * kv(t));
        return FW_OK;
    }
    int panels(int t, int h, cudaStream_t q = nullptr) {
        if (T < 2) return FW_OK;
        if (q == nullptr) q = s;
        const int nslab = (int)((kv(t) + kSlab - 1) / kSlab);
        prof_begin(KC_PANEL, q);
        fw_panel_kernel<VEC><<<dim3(T - 1, 2), kThreads, kSmemBytes, q>>>(D, n, ldp, t, nslab, colT + h * kTile * ldp,
                                                                         rowP + h * kTile * ldp, 1, skip);
        FW_LAUNCH_CHECK("fw_panel_kernel");
        prof_end(KC_PANEL, q, 2.0 * (double)(n - kv(t)) * kv(t) * kv(t));
        return FW_OK;
    }
    // Remainder launch over rows x cols with pivots [k_begin, k_end) of the
    // workspace (k_end - k_begin valid pivots; slabs rounded up).
    int remainder(TileSet rows, int nrows, TileSet cols, int ncols, int k_begin, int k_valid,
                  cudaStream_t q = nullptr, int cross = -1) {
        if (nrows <= 0 || ncols <= 0 || k_valid <= 0) return FW_OK;
        if (q == nullptr) q = s;
        const int slab0 = k_begin / kSlab;
        const int nslab = (k_valid + kSlab - 1) / kSlab;
        const int64_t ntiles = cross >= 0 ? (int64_t)ncols : (int64_t)nrows * ncols;
        const unsigned grid = (unsigned)((skip && ntiles > resident_ctas) ? resident_ctas : ntiles);
        prof_begin(KC_REMAINDER, q);
        fw_remainder_kernel<VEC><<<grid, kThreads, kSmemBytes, q>>>(D, n, rows, nrows, cols, ncols, slab0, nslab, mapA,
                                                                    mapB, 1, skip, cross, faults);
        FW_LAUNCH_CHECK("fw_remainder_kernel");
        const double relax = cross >= 0
                                 ? ((double)kv(cross + 1) * (double)(n - kv(cross)) +
                                    (double)(n - kv(cross) - kv(cross + 1)) * (double)kv(cross + 1)) *
                                       (double)k_valid
                                 : relax_of(rows, nrows) * relax_of(cols, ncols) * (double)k_valid;
        prof_end(KC_REMAINDER, q, relax);
        return FW_OK;
    }
    // Block t's update of block t + 1's row and column, one launch.
    int cross_update(int t, int k_begin, int k_valid, cudaStream_t q) {
        return remainder(TileSet{-1, -1, -1}, T, TileSet{-1, -1, -1}, 2 * T - 3, k_begin, k_valid, q, t);
    }
    // Number of matrix rows (or columns) the tile set covers.
    double relax_of(const TileSet& ts, int count) const {
        (void)count;
        if (ts.single >= 0) return (double)kv(ts.single);
        double r = (double)n;
        if (ts.ex0 >= 0) r -= (double)kv(ts.ex0);
        if (ts.ex1 >= 0) r -= (double)kv(ts.ex1);
        return r;
    }

    // One 128-wide pivot block per remainder pass with a one-block look-ahead
    // (tiling_gpu; kappa <= 4; needs two panel buffers). The high-priority
    // stream carries the chain every later block waits for — block t's update
    // of block t+1's row and column (one launch), then block t+1's closure and
    // panels into the other buffer — while the side stream runs block t's bulk
    // remainder (every tile outside both blocks) concurrently. The chain for
    // block t+1 starts once block t-1's bulk is done (its tiles, and the
    // panel buffer block t+1 reuses).
    int lookahead() {
        if (int rc = aux_stream_get(s, &aux)) return rc;
        FW_CUDA_TRY(cudaEventRecord(aux.fork, s));
        FW_CUDA_TRY(cudaStreamWaitEvent(aux.hi, aux.fork, 0));
        FW_CUDA_TRY(cudaStreamWaitEvent(aux.side, aux.fork, 0));
        if (int rc = diag(0, 0, aux.hi)) return rc;
        if (int rc = panels(0, 0, aux.hi)) return rc;
        FW_CUDA_TRY(cudaEventRecord(aux.panels[0], aux.hi));
        for (int t = 0; t < T; ++t) {
            const int h = t & 1;
            const int k0 = h * kTile, kvt = (int)kv(t);
            if (t + 1 < T) {
                if (t >= 1) FW_CUDA_TRY(cudaStreamWaitEvent(aux.hi, aux.bulk[(t - 1) & 1], 0));
                if (int rc = cross_update(t, k0, kvt, aux.hi)) return rc;
                if (int rc = diag(t + 1, h ^ 1, aux.hi)) return rc;
                if (int rc = panels(t + 1, h ^ 1, aux.hi)) return rc;
                FW_CUDA_TRY(cudaEventRecord(aux.panels[(t + 1) & 1], aux.hi));
            }
            FW_CUDA_TRY(cudaStreamWaitEvent(aux.side, aux.panels[h], 0));
            if (t + 1 < T) {
                if (int rc = remainder(all_but(t, t + 1), T - 2, all_but(t, t + 1), T - 2, k0, kvt, aux.side)) return rc;
            } else {
                if (int rc = remainder(all_but(t), T - 1, all_but(t), T - 1, k0, kvt, aux.side)) return rc;
            }
            FW_CUDA_TRY(cudaEventRecord(aux.bulk[h], aux.side));
        }
        // the side stream's last launch follows every launch of the chain
        FW_CUDA_TRY(cudaStreamWaitEvent(s, aux.bulk[(T - 1) & 1], 0));
        return FW_OK;
    }

    // One 128-wide pivot block per remainder pass (tiling_gpu; kappa <= 4).
    int single(int t) {
        if (int rc = diag(t, 0)) return rc;
        if (int rc = panels(t, 0)) return rc;
        return remainder(all_but(t), T - 1, all_but(t), T - 1, 0, (int)kv(t));
    }

    // Two pivot blocks t1 = t, t2 = t + 1 folded into one remainder pass of
    // 256 pivots (kappa >= 5). With C1/R1 the panels of block 1 after block 1
    // and C2/R2 those of block 2 after both blocks, the final value of a tile
    // outside both blocks' rows and columns is min(D, C1 (x) R1, C2 (x) R2):
    //   1. close block 1, its panels -> workspace half 0 (C1, R1)
    //   2. block 1's update of block 2's row and column (the tiles block 2
    //      needs before it can be closed)
    //   3. close block 2, its panels -> workspace half 1 (C2, R2)
    //   4. the remainder: all other tiles, 256 pivots from both halves
    //   5. block 2's update of block 1's row and column (the panels of
    //      block 1 were final only with respect to block 1).
    int pair(int t) {
        const int t1 = t, t2 = t + 1;
        const int k1 = (int)kv(t1), k2 = (int)kv(t2);
        if (int rc = diag(t1, 0)) return rc;
        if (int rc = panels(t1, 0)) return rc;
        if (int rc = remainder(only(t2), 1, all_but(t1), T - 1, 0, k1)) return rc;
        if (int rc = remainder(all_but(t1, t2), T - 2, only(t2), 1, 0, k1)) return rc;
        if (int rc = diag(t2, 1)) return rc;
        if (int rc = panels(t2, 1)) return rc;
        if (int rc = remainder(all_but(t1, t2), T - 2, all_but(t1, t2), T - 2, 0, kTile + k2)) return rc;
        if (int rc = remainder(only(t1), 1, all_but(t2), T - 1, kTile, k2)) return rc;
        return remainder(all_but(t1, t2), T - 2, only(t1), 1, kTile, k2);
    }
};

template <bool VEC>
int blocked_solve_impl(int32_t* D, int64_t n, int blocks_per_pass, bool lookahead, int* colT, int* rowP, int sets,
                       cudaStream_t s, const unsigned* skip, unsigned* faults) {
    static PerDeviceOnce attrs;
    if (int rc = once_per_device(attrs, [] {
            FW_CUDA_TRY(
                cudaFuncSetAttribute(fw_panel_kernel<VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
            FW_CUDA_TRY(
                cudaFuncSetAttribute(fw_remainder_kernel<VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
            return (int)FW_OK;
        }))
        return rc;
    Blocked<VEC> b{D, n, 0, (int)((n + kTile - 1) / kTile), colT, rowP, s, skip, faults};
    b.ldp = (int64_t)b.T * kTile;
    {
        int dev = 0, sms = 0;
        FW_CUDA_TRY(cudaGetDevice(&dev));
        FW_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        b.resident_ctas = 2 * (int64_t)(sms > 0 ? sms : 152);
    }
    if (int rc = panel_map(&b.mapA, colT, (uint64_t)b.ldp, (uint64_t)sets * kTile, kTile)) return rc;
    if (int rc = panel_map(&b.mapB, rowP, (uint64_t)b.ldp, (uint64_t)sets * kTile, kTile)) return rc;
    if (blocks_per_pass == 1 && lookahead && b.T > 2) return b.lookahead();
    for (int t = 0; t < b.T;) {
        if (blocks_per_pass == 2 && t + 1 < b.T) {
            if (int rc = b.pair(t)) return rc;
            t += 2;
        } else {
            if (int rc = b.single(t)) return rc;
            t += 1;
        }
    }
    return FW_OK;
}

}  // namespace

int blocks_per_pass(int variant, int kappa, int64_t n) {
    // The reference's kappa counts 32-wide tiles per pass; 128-wide blocks
    // cover kappa <= 4, two blocks (256 pivots) cover the larger values. The
    // remainder is compute-bound either way, so below n = 24576 the one-block
    // look-ahead schedule (which hides the closures and panels) is faster and
    // runs instead (measured on GB300 at n = 8192: 30.2 vs 35.7 ms; at
    // n = 32768 the two-block pass is 0.7 % faster).
    return (variant == FW_VARIANT_MULTI_LAYER && normalise_kappa(kappa) > 4 && n >= 24576) ? 2 : 1;
}

size_t blocked_workspace_bytes(int64_t n, int blocks) {
    const int64_t T = (n + kTile - 1) / kTile;
    return (size_t)2 * blocks * kTile * (size_t)(T * kTile) * sizeof(int);
}

int blocked_solve(int32_t* D, int64_t n, int blocks, void* ws, size_t ws_bytes, cudaStream_t s,
                  const unsigned int* skip, unsigned int* faults) {
    const int64_t T = (n + kTile - 1) / kTile;
    // Two panel buffers are needed by the two-block pass and by the look-ahead.
    const bool two = ws_bytes >= blocked_workspace_bytes(n, 2);
    const int sets = two ? 2 : 1;
    int* colT = static_cast<int*>(ws);
    int* rowP = colT + (size_t)sets * kTile * (size_t)(T * kTile);
    const bool vec = (n % 4) == 0;
    return vec ? blocked_solve_impl<true>(D, n, blocks, two, colT, rowP, sets, s, skip, faults)
               : blocked_solve_impl<false>(D, n, blocks, two, colT, rowP, sets, s, skip, faults);
}

size_t pivot_workspace_bytes(int64_t n) { return (size_t)4 * (size_t)((n + 3) & ~int64_t(3)) * sizeof(int); }

namespace {

// The per-pivot sweep's launches, enqueued on `s` (one prime + n steps).
int pivot_enqueue(int32_t* D, int64_t n, void* ws, cudaStream_t s, bool bracket) {
    const int64_t np = (n + 3) & ~int64_t(3);
    int* rowb[2] = {static_cast<int*>(ws), static_cast<int*>(ws) + np};
    int* colb[2] = {static_cast<int*>(ws) + 2 * np, static_cast<int*>(ws) + 3 * np};
    const bool vec = (n % 4) == 0;
    fw_pivot_prime_kernel<<<(unsigned)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024), 256, 0, s>>>(D, n, rowb[0],
                                                                                                    colb[0]);
    FW_LAUNCH_CHECK("fw_pivot_prime_kernel");
    const unsigned gx = (unsigned)((n + 255) / 256 < 64 ? (n + 255) / 256 : 64);
    const dim3 vgrid((unsigned)((n / 4 + 256 * kPivVecs - 1) / (256 * kPivVecs)),
                     (unsigned)((n + kPivRows - 1) / kPivRows));
    for (int64_t k = 0; k < n; ++k) {
        const int cur = (int)(k & 1);
        if (bracket) prof_begin(KC_PIVOT_STEP, s);
        if (vec)
            fw_pivot_step_vec_kernel<<<vgrid, 256, 0, s>>>(D, n, (int)k, rowb[cur], colb[cur], rowb[cur ^ 1],
                                                           colb[cur ^ 1]);
        else
            fw_pivot_step_kernel<<<dim3(gx, (unsigned)n), 256, 0, s>>>(D, n, k, rowb[cur], colb[cur], rowb[cur ^ 1],
                                                                       colb[cur ^ 1]);
        FW_LAUNCH_CHECK("fw_pivot_step_kernel");
        if (bracket) prof_end(KC_PIVOT_STEP, s, (double)n * n);
    }
    return FW_OK;
}

// Small matrices spend the per-pivot sweep in launch overhead (n launches of
// a few microseconds of work each), so for 256 <= n <= 2048 the launches are
// captured once into a CUDA graph on a private stream and replayed on the
// caller's stream. One graph is kept per (device, caller stream), for the last
// (matrix, n, workspace) it was captured with. Under fw_profile_begin the
// replay is timed as one bracket that counts its n step launches.
constexpr int64_t kPivotGraphMinN = 256, kPivotGraphMaxN = 2048;
struct PivotGraph {
    int32_t* D = nullptr;
    int64_t n = 0;
    void* ws = nullptr;
    cudaGraphExec_t exec = nullptr;
};
std::mutex g_pivot_graph_mutex;
std::map<std::pair<int, cudaStream_t>, PivotGraph> g_pivot_graphs;
std::map<int, cudaStream_t> g_pivot_capture;

int pivot_graph_launch(int32_t* D, int64_t n, void* ws, cudaStream_t s) {
    int dev = 0;
    FW_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_pivot_graph_mutex);
    PivotGraph& g = g_pivot_graphs[{dev, s}];
    if (!(g.exec && g.D == D && g.n == n && g.ws == ws)) {
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
        cudaStream_t& cap = g_pivot_capture[dev];
        if (!cap) FW_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaGraph_t graph = nullptr;
        FW_CUDA_TRY(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        const int rc = pivot_enqueue(D, n, ws, cap, false);
        const cudaError_t e = cudaStreamEndCapture(cap, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return cuda_error(e, "cudaStreamEndCapture");
        const cudaError_t ei = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            g.exec = nullptr;
            return cuda_error(ei, "cudaGraphInstantiate");
        }
        g.D = D;
        g.n = n;
        g.ws = ws;
    }
    prof_begin(KC_PIVOT_STEP, s);
    FW_CUDA_TRY(cudaGraphLaunch(g.exec, s));
    prof_end(KC_PIVOT_STEP, s, (double)n * n * n, n);
    return FW_OK;
}

}  // namespace

int pivot_solve(int32_t* D, int64_t n, void* ws, cudaStream_t s, bool may_allocate) {
    if (may_allocate && n >= kPivotGraphMinN && n <= kPivotGraphMaxN) {
        cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
        FW_CUDA_TRY(cudaStreamIsCapturing(s, &st));
        if (st == cudaStreamCaptureStatusNone) return pivot_graph_launch(D, n, ws, s);
    }
    return pivot_enqueue(D, n, ws, s, true);
}

}  // namespace fw

extern "C" int fw_debug_bounded_wait(int spins, fw_stream_t stream) {
    if (spins < 1 || spins > (1 << 20))
        return fw::set_error(FW_ERR_INVALID_ARGUMENT, "fw_debug_bounded_wait: spins must be in [1, 1048576]");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned int* result = nullptr;
    FW_CUDA_TRY(cudaGetSymbolAddress(reinterpret_cast<void**>(&result), fw::g_wait_probe_result));
    FW_CUDA_TRY(cudaMemsetAsync(result, 0, sizeof(unsigned int), s));
    fw::fw_wait_probe_kernel<<<1, 32, 0, s>>>(spins, result);
    FW_LAUNCH_CHECK("fw_wait_probe_kernel");
    FW_CUDA_TRY(cudaStreamSynchronize(s));
    unsigned int v = 0;
    FW_CUDA_TRY(cudaMemcpy(&v, result, sizeof(v), cudaMemcpyDeviceToHost));
    if (!(v & 2u))
        return fw::set_error(FW_ERR_INTERNAL, "fw_debug_bounded_wait: the barrier did not complete after its "
                                              "transfer count was settled");
    if (v & 1u)
        return fw::set_error(FW_ERR_TIMEOUT, "fw_debug_bounded_wait: the bounded wait gave up after " +
                                                 std::to_string(spins) + " tries (no copy was issued)");
    return FW_OK;
}

extern "C" int fw_copy_faults(unsigned int* count) {
    if (count == nullptr) return fw::set_error(FW_ERR_INVALID_ARGUMENT, "fw_copy_faults: count is NULL");
    FW_CUDA_TRY(cudaMemcpyFromSymbol(count, fw::g_copy_faults, sizeof(unsigned int)));
    *count += fw::nh_copy_faults() + fw::ooc_copy_faults();
    return FW_OK;
}

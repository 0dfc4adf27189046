// Differentiable Floyd-Warshall: an fp32 forward that also records next hops,
// and a backward that scatters dL/dD onto the edge weights along the
// recorded shortest paths. No reference counterpart (the reference is int32
// only); the forward's relaxation and next-hop rule are those of the FP64
// oracle sweep: if (D[i][k] + D[k][j] < D[i][j]) { D[i][j] = D[i][k] + D[k][j];
// nh[i][j] = nh[i][k]; }, with missing edges +inf and nh[i][j] = j for an
// edge, i on the diagonal, -1 for no edge.
//
// The forward is the same blocked schedule as the int32 engine — closed
// 128 x 128 diagonal block, row / column panels as min-plus products with
// that closure, then the remainder — on batches of equal-size graphs
// (blockIdx.z = graph). Tiles are 128 x 128 on 512-thread CTAs (an 8 x 4
// value + next-hop register micro-tile per thread); the remainder streams a
// value slab and a next-hop slab of the transposed column panel plus a value
// slab of the row panel per 32 pivots, copied by TMA into a three-stage ring
// (the panels use a two-stage cp.async ring).
//
// Backward, per graph and destination j: the next hops toward j form a tree
// rooted at j, and edge (u, nh[u][j]) lies on the path i -> j exactly when u
// is on it, so dL/dW[u][nh[u][j]] += sum of dL/dD[i][j] over the sources i
// whose path passes through u. One CTA per (destination, graph) walks every
// source's path, accumulating those sums in shared memory, then adds them
// into dL/dW. A walk that does not reach j within n hops is counted in a
// status word instead of looping.
#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "fw_common.cuh"
#include "fw_internal.h"
#include "fw_tma.cuh"

namespace fw {

// Remainder tile copies that missed their bounded wait (see fw_copy_faults).
__device__ unsigned int g_nh_copy_faults = 0;

namespace {

constexpr int kFThreads = 512;  // 16 row groups x 32 column groups

// Value type of the next-hop sweep: fp32 (missing edge +inf) for the
// differentiable form, int32 (missing edge INF = 1e9) for path reconstruction
// of the integer sweep. INF + INF fits int32, so padded pivots never win.
template <typename V>
struct VT;
template <>
struct VT<float> {
    __device__ static float inf() { return INFINITY; }
    __device__ static bool edge(float v) { return isfinite(v); }
};
template <>
struct VT<int> {
    __device__ static int inf() { return kInf; }
    __device__ static bool edge(int v) { return v < kInf; }
};

template <typename V>
struct __align__(16) V4 {
    V x, y, z, w;
};
constexpr int kFStages = 2;
constexpr int kFSlabInts = kSlab * kTile;
constexpr int kFStageInts = 3 * kFSlabInts;  // A values, A next hops, B values
constexpr int kFSmemBytes = kFStages * kFStageInts * 4;  // 96 KB
constexpr int kFTStages = 3;                              // remainder: TMA ring
constexpr int kFTSmemBytes = kFTStages * kFStageInts * 4;  // 144 KB

// Thread (tx = t % 32, ty = t / 32) of a 128 x 128 tile owns rows
// own_row(ty, r), r < 8, and columns tx*4 .. tx*4+3.
template <typename V>
__device__ __forceinline__ void relax_nh(V& c, int& h, V a, int ha, V b) {
    const V s = a + b;
    if (s < c) {
        c = s;
        h = ha;
    }
}

template <typename V>
__device__ __forceinline__ V4<V> ld4v(const V* p) { return *reinterpret_cast<const V4<V>*>(p); }
__device__ __forceinline__ int4 ld4i(const int* p) { return *reinterpret_cast<const int4*>(p); }

// acc/nh for the 128 x 128 tile at (r0, c0) of an n x n matrix (inf / -1 outside).
template <typename V>
__device__ __forceinline__ void f_load_tile(V (&c)[8][4], int (&h)[8][4], const V* D, const int* nh,
                                            int64_t n, int64_t r0, int64_t c0, int tx, int ty) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int64_t i = r0 + own_row(ty, r);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int64_t j = c0 + tx * 4 + e;
            const bool in = i < n && j < n;
            c[r][e] = in ? D[i * n + j] : VT<V>::inf();
            h[r][e] = in ? nh[i * n + j] : -1;
        }
    }
}

template <typename V>
__device__ __forceinline__ void f_store_tile(const V (&c)[8][4], const int (&h)[8][4], V* D, int* nh, int64_t n,
                                             int64_t r0, int64_t c0, int tx, int ty) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int64_t i = r0 + own_row(ty, r);
        if (i >= n) continue;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int64_t j = c0 + tx * 4 + e;
            if (j < n) {
                D[i * n + j] = c[r][e];
                nh[i * n + j] = h[r][e];
            }
        }
    }
}

// Slab of a k-major workspace buffer (32 rows x 128 columns starting at c0).
__device__ __forceinline__ void f_load_kmajor(void* dst, const void* buf, int64_t ldp, int k0, int64_t c0, int tid) {
    for (int q = tid; q < kSlab * 32; q += kFThreads) {
        const int row = q >> 5, ch = q & 31;
        cp_async16(static_cast<int*>(dst) + row * kTile + ch * 4,
                   static_cast<const int*>(buf) + (int64_t)(k0 + row) * ldp + c0 + ch * 4);
    }
}

// Slab of D rows [r0, r0 + 32), columns [c0, c0 + 128) (inf outside).
template <typename V>
__device__ __forceinline__ void f_load_rows(V* dst, const V* D, int64_t n, int64_t r0, int64_t c0, int tid) {
    for (int q = tid; q < kSlab * kTile; q += kFThreads) {
        const int row = q >> 7, col = q & 127;
        const int64_t i = r0 + row, j = c0 + col;
        dst[row * kTile + col] = (i < n && j < n) ? D[i * n + j] : VT<V>::inf();
    }
}

// Transposed slab of D and nh: dst[kk][i] = X[r0 + i][k0 + kk].
template <typename V>
__device__ __forceinline__ void f_load_transposed(V* dv, int* dh, const V* D, const int* nh, int64_t n,
                                                  int64_t r0, int64_t k0, int tid) {
    for (int q = tid; q < kTile * kSlab; q += kFThreads) {
        const int i = q >> 5, kk = q & 31;
        const int64_t gi = r0 + i, gk = k0 + kk;
        const bool in = gi < n && gk < n;
        dv[kk * kTile + i] = in ? D[gi * n + gk] : VT<V>::inf();
        dh[kk * kTile + i] = in ? nh[gi * n + gk] : -1;
    }
}

// One slab: c/h = relax with A (values av, hops ah; k-major) and B (bv; k-major).
template <typename V>
__device__ __forceinline__ void f_relax_slab(V (&c)[8][4], int (&h)[8][4], const V* av, const int* ah,
                                             const V* bv, int nk, int tx, int ty) {
#pragma unroll 2
    for (int kk = 0; kk < nk; ++kk) {
        const V4<V> a0 = ld4v(av + kk * kTile + ty * 4), a1 = ld4v(av + kk * kTile + 64 + ty * 4);
        const int4 h0 = ld4i(ah + kk * kTile + ty * 4), h1 = ld4i(ah + kk * kTile + 64 + ty * 4);
        const V4<V> b = ld4v(bv + kk * kTile + tx * 4);
        const V a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const int ha[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
        const V bb[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int e = 0; e < 4; ++e) relax_nh(c[r][e], h[r][e], a[r], ha[r], bb[e]);
    }
}

// Two-stage pipeline over the pivot slabs: la(av, ah, s) / lb(bv, s) fill slab s.
template <typename V, class LA, class LB>
__device__ __forceinline__ void f_mainloop(V (&c)[8][4], int (&h)[8][4], int kv, int* smem, LA la, LB lb, int tx,
                                           int ty) {
    const int nslab = (kv + kSlab - 1) / kSlab;
    auto stage = [&](int s) { return smem + (s % kFStages) * kFStageInts; };
    {
        int* st = stage(0);
        la(reinterpret_cast<V*>(st), st + kFSlabInts, 0);
        lb(reinterpret_cast<V*>(st + 2 * kFSlabInts), 0);
        cp_async_commit();
    }
    for (int s = 0; s < nslab; ++s) {
        if (s + 1 < nslab) {
            int* st = stage(s + 1);
            la(reinterpret_cast<V*>(st), st + kFSlabInts, s + 1);
            lb(reinterpret_cast<V*>(st + 2 * kFSlabInts), s + 1);
        }
        cp_async_commit();
        cp_async_wait<1>();
        __syncthreads();
        const int* st = stage(s);
        const int nk = min(kSlab, kv - s * kSlab);
        f_relax_slab<V>(c, h, reinterpret_cast<const V*>(st), st + kFSlabInts,
                        reinterpret_cast<const V*>(st + 2 * kFSlabInts), nk, tx, ty);
        __syncthreads();
    }
}

// Next hops of the input: j for an edge, i on the diagonal, -1 otherwise.
template <typename V>
__global__ void fw_nh_init_kernel(const V* __restrict__ D, int* __restrict__ nh, int64_t n, int64_t total) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = q % (n * n);
        const int64_t i = e / n, j = e % n;
        nh[q] = (i == j) ? (int)i : (VT<V>::edge(D[q]) ? (int)j : -1);
    }
}

// Phase 1: closure of the diagonal block of graph blockIdx.z; 512 threads,
// 4 x 8 values + next hops each; also fills the workspace panels.
template <typename V>
__global__ void __launch_bounds__(kFThreads, 1)
    fw_nh_diag_kernel(V* __restrict__ Dall, int* __restrict__ nhall, int64_t n, int64_t ldp, int64_t p0,
                      V* __restrict__ colTall, int* __restrict__ colHall, V* __restrict__ rowPall) {
    __shared__ __align__(16) V prow[2][kTile];
    __shared__ __align__(16) V pcol[2][kTile];
    __shared__ __align__(16) int pcolh[2][kTile];
    const int64_t gph = blockIdx.z;
    V* D = Dall + gph * n * n;
    int* nh = nhall + gph * n * n;
    V* colT = colTall + gph * kTile * ldp;
    int* colH = colHall + gph * kTile * ldp;
    V* rowP = rowPall + gph * kTile * ldp;
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;  // rows ty*4.., columns tx*8..
    V c[4][8];
    int h[4][8];
    const int64_t rem = n - p0;
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int lr = ty * 4 + r, lc = tx * 8 + e;
            const bool in = lr < rem && lc < rem;
            c[r][e] = in ? D[(p0 + lr) * n + p0 + lc] : VT<V>::inf();
            h[r][e] = in ? nh[(p0 + lr) * n + p0 + lc] : -1;
        }
    if (ty == 0)
#pragma unroll
        for (int e = 0; e < 8; ++e) prow[0][tx * 8 + e] = c[0][e];
    if (tx == 0)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            pcol[0][ty * 4 + r] = c[r][0];
            pcolh[0][ty * 4 + r] = h[r][0];
        }
    __syncthreads();
    for (int kb = 0; kb < kTile; kb += 8) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int k = kb + u, buf = u & 1;
            V a[4], b[8];
            int ha[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                a[r] = pcol[buf][ty * 4 + r];
                ha[r] = pcolh[buf][ty * 4 + r];
            }
#pragma unroll
            for (int e = 0; e < 8; ++e) b[e] = prow[buf][tx * 8 + e];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int e = 0; e < 8; ++e) relax_nh(c[r][e], h[r][e], a[r], ha[r], b[e]);
            const int k1 = k + 1;
            if (k1 < kTile) {
                const int sr = (u + 1) & 3, sc = (u + 1) & 7;
                if (ty == (k1 >> 2))
#pragma unroll
                    for (int e = 0; e < 8; ++e) prow[buf ^ 1][tx * 8 + e] = c[sr][e];
                if (tx == (k1 >> 3))
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        pcol[buf ^ 1][ty * 4 + r] = c[r][sc];
                        pcolh[buf ^ 1][ty * 4 + r] = h[r][sc];
                    }
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int lr = ty * 4 + r, lc = tx * 8 + e;
            if (lr < rem && lc < rem) {
                D[(p0 + lr) * n + p0 + lc] = c[r][e];
                nh[(p0 + lr) * n + p0 + lc] = h[r][e];
            }
            colT[(int64_t)lc * ldp + p0 + lr] = c[r][e];
            colH[(int64_t)lc * ldp + p0 + lr] = h[r][e];
            rowP[(int64_t)lr * ldp + p0 + lc] = c[r][e];
        }
}

// Phase 2: blockIdx.y == 0 -> row panel tile (P, J); == 1 -> column panel tile (I, P).
template <typename V>
__global__ void __launch_bounds__(kFThreads, 1)
    fw_nh_panel_kernel(V* __restrict__ Dall, int* __restrict__ nhall, int64_t n, int64_t ldp, int pt,
                       V* __restrict__ colTall, int* __restrict__ colHall, V* __restrict__ rowPall) {
    extern __shared__ __align__(128) int smem[];
    const int64_t gph = blockIdx.z;
    V* D = Dall + gph * n * n;
    int* nh = nhall + gph * n * n;
    V* colT = colTall + gph * kTile * ldp;
    int* colH = colHall + gph * kTile * ldp;
    V* rowP = rowPall + gph * kTile * ldp;
    const int tid = threadIdx.x, tx = tid % 32, ty = tid / 32;
    const int other = (int)blockIdx.x < pt ? (int)blockIdx.x : (int)blockIdx.x + 1;
    const int64_t p0 = (int64_t)pt * kTile, q0 = (int64_t)other * kTile;
    const int kv = (int)(n - p0 < kTile ? n - p0 : kTile);
    V c[8][4];
    int h[8][4];
    if (blockIdx.y == 0) {
        f_load_tile(c, h, D, nh, n, p0, q0, tx, ty);
        f_mainloop(
            c, h, kv, smem,
            [&](V* av, int* ah, int s) {
                f_load_kmajor(av, colT, ldp, s * kSlab, p0, tid);
                f_load_kmajor(ah, colH, ldp, s * kSlab, p0, tid);
            },
            [&](V* bv, int s) { f_load_rows(bv, D, n, p0 + s * kSlab, q0, tid); }, tx, ty);
        f_store_tile(c, h, D, nh, n, p0, q0, tx, ty);
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int e = 0; e < 4; ++e) rowP[(int64_t)own_row(ty, r) * ldp + q0 + tx * 4 + e] = c[r][e];
    } else {
        f_load_tile(c, h, D, nh, n, q0, p0, tx, ty);
        f_mainloop(
            c, h, kv, smem,
            [&](V* av, int* ah, int s) { f_load_transposed(av, ah, D, nh, n, q0, p0 + s * kSlab, tid); },
            [&](V* bv, int s) { f_load_kmajor(bv, rowP, ldp, s * kSlab, p0, tid); }, tx, ty);
        f_store_tile(c, h, D, nh, n, q0, p0, tx, ty);
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                colT[(int64_t)(tx * 4 + e) * ldp + q0 + own_row(ty, r)] = c[r][e];
                colH[(int64_t)(tx * 4 + e) * ldp + q0 + own_row(ty, r)] = h[r][e];
            }
    }
}

// Phase 3: remainder tiles of graph blockIdx.z with the panels of pivot block
// pt: tiles (I, J), I from `rows` (nrows), J from `cols` (ncols), one per
// blockIdx.x; or, with cross >= 0, block pt's update of block u = pt + 1's
// row and column: tiles [0, T - 1) are (u, J), J != pt, the next T - 2 are
// (I, u), I != pt, u. A copy that misses its bounded wait is counted in
// `faults` (the call's status word) and g_nh_copy_faults; the CTA then waits
// for the copies it issued and leaves its tile as it was.
template <typename V>
__global__ void __launch_bounds__(kFThreads, 1)
    fw_nh_remainder_kernel(V* __restrict__ Dall, int* __restrict__ nhall, int64_t n, int pt, int T, TileSet rows,
                           TileSet cols, int ncols, int cross, const __grid_constant__ CUtensorMap mapCT,
                           const __grid_constant__ CUtensorMap mapCH, const __grid_constant__ CUtensorMap mapRP,
                           unsigned* __restrict__ faults) {
    extern __shared__ __align__(128) int smem[];
    __shared__ __align__(8) uint64_t bars[kFTStages];
    __shared__ int s_ok;
    const int tid = threadIdx.x, tx = tid % 32, ty = tid / 32;
    if (tid == 0) {
        s_ok = (smem_u32(smem) & 127u) == 0;
        for (int i = 0; i < kFTStages; ++i) mbar_init(&bars[i], 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (!s_ok) {  // no copy can be issued: the tile keeps its values
        if (tid == 0) count_copy_fault(&g_nh_copy_faults, faults);
        return;
    }
    const int gph = (int)blockIdx.z;
    V* D = Dall + (int64_t)gph * n * n;
    int* nh = nhall + (int64_t)gph * n * n;
    const int x = (int)blockIdx.x;
    int ti, tj;
    if (cross < 0) {
        ti = tile_of(rows, x / ncols);
        tj = tile_of(cols, x % ncols);
    } else if (x < T - 1) {
        ti = pt + 1;
        tj = tile_of(all_but(pt), x);
    } else {
        ti = tile_of(all_but(pt, pt + 1), x - (T - 1));
        tj = pt + 1;
    }
    const int64_t p0 = (int64_t)pt * kTile;
    const int r0 = ti * kTile, c0 = tj * kTile;
    const int kv = (int)(n - p0 < kTile ? n - p0 : kTile);
    const int nslab = (kv + kSlab - 1) / kSlab;
    // Per slab: the column panel's values and next hops at rows r0.., the row
    // panel's values at columns c0.., by TMA into one stage.
    auto issue = [&](int j) {
        if (tid == 0) {
            const int stg = j % kFTStages;
            int* dst = smem + stg * kFStageInts;
            mbar_expect_tx(&bars[stg], (uint32_t)kFStageInts * 4);
            tma_load_3d(dst, &mapCT, r0, j * kSlab, gph, &bars[stg]);
            tma_load_3d(dst + kFSlabInts, &mapCH, r0, j * kSlab, gph, &bars[stg]);
            tma_load_3d(dst + 2 * kFSlabInts, &mapRP, c0, j * kSlab, gph, &bars[stg]);
        }
    };
    V c[8][4];
    int h[8][4];
    f_load_tile(c, h, D, nh, n, r0, c0, tx, ty);
#pragma unroll
    for (int j = 0; j < kFTStages - 1; ++j)
        if (j < nslab) issue(j);
    for (int kb = 0; kb < nslab; ++kb) {
        const int stg = kb % kFTStages;
        // every thread is past slab kb - 1 (its stage can be refilled), and all
        // agree whether slab kb arrived
        if (!ring_wait_all(&bars[stg], (uint32_t)((kb / kFTStages) & 1))) {
            if (tid == 0) count_copy_fault(&g_nh_copy_faults, faults);
            ring_drain(bars, kFTStages, kb, min(kb + kFTStages - 2, nslab - 1));
            return;
        }
        if (kb + kFTStages - 1 < nslab) issue(kb + kFTStages - 1);
        const int* st = smem + stg * kFStageInts;
        f_relax_slab<V>(c, h, reinterpret_cast<const V*>(st), st + kFSlabInts,
                        reinterpret_cast<const V*>(st + 2 * kFSlabInts), min(kSlab, kv - kb * kSlab), tx, ty);
    }
    f_store_tile(c, h, D, nh, n, r0, c0, tx, ty);
}

// Backward: CTA (j, graph). Shared: next hops toward j, dL/dD[:, j], path sums.
__global__ void __launch_bounds__(256)
    fw_backward_kernel(const float* __restrict__ Gall, const int* __restrict__ nhall, float* __restrict__ dWall,
                       int64_t n, int* __restrict__ bad_walks) {
    extern __shared__ __align__(16) int bsm[];
    int* hop = bsm;                                        // n
    float* gcol = reinterpret_cast<float*>(bsm + n);       // n
    float* acc = reinterpret_cast<float*>(bsm + 2 * n);    // n
    const int64_t gph = blockIdx.y;
    const int64_t j = blockIdx.x;
    const float* G = Gall + gph * n * n;
    const int* nh = nhall + gph * n * n;
    float* dW = dWall + gph * n * n;
    for (int64_t u = threadIdx.x; u < n; u += blockDim.x) {
        hop[u] = nh[u * n + j];
        gcol[u] = G[u * n + j];
        acc[u] = 0.f;
    }
    __syncthreads();
    int bad = 0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        if (i == j || hop[i] < 0) continue;
        const float g = gcol[i];
        int64_t u = i, steps = 0;
        while (u != j && steps < n) {
            atomicAdd(&acc[u], g);
            const int v = hop[u];
            if (v < 0 || v >= n) break;
            u = v;
            ++steps;
        }
        if (u != j) ++bad;
    }
    if (bad && bad_walks) atomicAdd(bad_walks, bad);
    __syncthreads();
    for (int64_t u = threadIdx.x; u < n; u += blockDim.x) {
        const int v = hop[u];
        if (u == j || v < 0 || v >= n) continue;
        const float s = acc[u];
        if (s != 0.f) atomicAdd(&dW[u * n + v], s);
    }
}

}  // namespace

// Two panel buffers (colT, colH, rowP each) per graph: the look-ahead closes
// block t + 1 into one while block t's remainder reads the other.
size_t f32_workspace_bytes(int64_t n, int64_t batch) {
    const int64_t ldp = (n + kTile - 1) / kTile * kTile;
    return (size_t)2 * 3 * kTile * ldp * 4 * (size_t)batch;
}

// The blocked sweep with next hops over a batch of graphs, with a one-block
// look-ahead: the high-priority stream carries block t's update of block
// t+1's row and column, block t+1's closure and panels (into the other panel
// buffer), while the side stream runs block t's bulk remainder (tiles outside
// both blocks). The chain for block t+1 starts once block t-1's bulk is done.
template <typename V>
int nh_forward(V* D, int* nh, int64_t n, int64_t batch, void* ws, cudaStream_t s, KernelClass kc, unsigned* faults) {
    static PerDeviceOnce attrs;
    if (int rc = once_per_device(attrs, [] {
            FW_CUDA_TRY(
                cudaFuncSetAttribute(fw_nh_panel_kernel<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFSmemBytes));
            FW_CUDA_TRY(cudaFuncSetAttribute(fw_nh_remainder_kernel<V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kFTSmemBytes));
            return (int)FW_OK;
        }))
        return rc;
    AuxStream aux;
    if (int rc = aux_stream_get(s, &aux)) return rc;
    const int T = (int)((n + kTile - 1) / kTile);
    const int64_t ldp = (int64_t)T * kTile;
    const size_t panel = (size_t)kTile * ldp * batch;
    V* colT[2];
    int* colH[2];
    V* rowP[2];
    for (int b = 0; b < 2; ++b) {
        colT[b] = reinterpret_cast<V*>(static_cast<char*>(ws) + (size_t)b * 3 * panel * 4);
        colH[b] = reinterpret_cast<int*>(colT[b] + panel);
        rowP[b] = reinterpret_cast<V*>(colH[b] + panel);
    }
    const unsigned nb = (unsigned)batch;
    // TMA maps over the panel buffers: batch panels of 128 rows x ldp each.
    CUtensorMap mapCT[2], mapCH[2], mapRP[2];
    for (int b = 0; b < 2; ++b) {
        if (int rc = panel_map_3d(&mapCT[b], colT[b], (uint64_t)ldp, kTile, (uint64_t)batch, kTile)) return rc;
        if (int rc = panel_map_3d(&mapCH[b], colH[b], (uint64_t)ldp, kTile, (uint64_t)batch, kTile)) return rc;
        if (int rc = panel_map_3d(&mapRP[b], rowP[b], (uint64_t)ldp, kTile, (uint64_t)batch, kTile)) return rc;
    }
    auto close = [&](int t, cudaStream_t q) -> int {
        const int b = t & 1;
        fw_nh_diag_kernel<V><<<dim3(1, 1, nb), kFThreads, 0, q>>>(D, nh, n, ldp, (int64_t)t * kTile, colT[b], colH[b],
                                                                  rowP[b]);
        FW_LAUNCH_CHECK("fw_nh_diag_kernel");
        if (T > 1) {
            fw_nh_panel_kernel<V><<<dim3(T - 1, 2, nb), kFThreads, kFSmemBytes, q>>>(D, nh, n, ldp, t, colT[b],
                                                                                     colH[b], rowP[b]);
            FW_LAUNCH_CHECK("fw_nh_panel_kernel");
        }
        return FW_OK;
    };
    auto remainder = [&](int t, TileSet rows, int nrows, TileSet cols, int ncols, int cross, cudaStream_t q) -> int {
        const int tiles = cross >= 0 ? 2 * T - 3 : nrows * ncols;
        if (tiles <= 0) return FW_OK;
        const int b = t & 1;
        fw_nh_remainder_kernel<V><<<dim3((unsigned)tiles, 1, nb), kFThreads, kFTSmemBytes, q>>>(
            D, nh, n, t, T, rows, cols, ncols, cross, mapCT[b], mapCH[b], mapRP[b], faults);
        FW_LAUNCH_CHECK("fw_nh_remainder_kernel");
        return FW_OK;
    };

    const int64_t total = n * n * batch;
    prof_begin(kc, s);
    fw_nh_init_kernel<V><<<(unsigned)std::min<int64_t>((total + 255) / 256, 4096), 256, 0, s>>>(D, nh, n, total);
    FW_LAUNCH_CHECK("fw_nh_init_kernel");
    FW_CUDA_TRY(cudaEventRecord(aux.fork, s));
    FW_CUDA_TRY(cudaStreamWaitEvent(aux.hi, aux.fork, 0));
    FW_CUDA_TRY(cudaStreamWaitEvent(aux.side, aux.fork, 0));
    if (int rc = close(0, aux.hi)) return rc;
    FW_CUDA_TRY(cudaEventRecord(aux.panels[0], aux.hi));
    const TileSet none{-1, -1, -1};
    for (int t = 0; t < T; ++t) {
        if (t + 1 < T) {
            if (t >= 1) FW_CUDA_TRY(cudaStreamWaitEvent(aux.hi, aux.bulk[(t - 1) & 1], 0));
            if (int rc = remainder(t, none, 0, none, 0, t, aux.hi)) return rc;
            if (int rc = close(t + 1, aux.hi)) return rc;
            FW_CUDA_TRY(cudaEventRecord(aux.panels[(t + 1) & 1], aux.hi));
        }
        FW_CUDA_TRY(cudaStreamWaitEvent(aux.side, aux.panels[t & 1], 0));
        if (t + 1 < T) {
            if (int rc = remainder(t, all_but(t, t + 1), T - 2, all_but(t, t + 1), T - 2, -1, aux.side)) return rc;
        } else {
            if (int rc = remainder(t, all_but(t), T - 1, all_but(t), T - 1, -1, aux.side)) return rc;
        }
        FW_CUDA_TRY(cudaEventRecord(aux.bulk[t & 1], aux.side));
    }
    // the side stream's last launch follows every launch of the chain
    FW_CUDA_TRY(cudaStreamWaitEvent(s, aux.bulk[(T - 1) & 1], 0));
    prof_end(kc, s, (double)n * n * n * batch);
    return FW_OK;
}

int f32_forward(float* D, int* nh, int64_t n, int64_t batch, void* ws, cudaStream_t s, unsigned* faults) {
    return nh_forward<float>(D, nh, n, batch, ws, s, KC_FWD_F32, faults);
}

int i32_paths(int* D, int* nh, int64_t n, int64_t batch, void* ws, cudaStream_t s, unsigned* faults) {
    return nh_forward<int>(D, nh, n, batch, ws, s, KC_PATHS_I32, faults);
}

int f32_backward(const float* G, const int* nh, float* dW, int64_t n, int64_t batch, int* d_bad, cudaStream_t s) {
    FW_CUDA_TRY(cudaMemsetAsync(dW, 0, sizeof(float) * (size_t)(n * n * batch), s));
    const size_t smem = (size_t)3 * n * 4;
    if (smem > 48 * 1024) {
        FW_CUDA_TRY(cudaFuncSetAttribute(fw_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    prof_begin(KC_BWD_F32, s);
    fw_backward_kernel<<<dim3((unsigned)n, (unsigned)batch), 256, smem, s>>>(G, nh, dW, n, d_bad);
    FW_LAUNCH_CHECK("fw_backward_kernel");
    prof_end(KC_BWD_F32, s, (double)n * n * batch);
    return FW_OK;
}

}  // namespace fw

namespace fw {
unsigned int nh_copy_faults() {
    unsigned int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_nh_copy_faults, sizeof(v)) != cudaSuccess) cudaGetLastError();
    return v;
}
}  // namespace fw

// Shared device-side building blocks of the fw103 kernels (sm_103a).
//
// The relaxation is the reference's D[i][j] = min(D[i][j], D[i][k] + D[k][j])
// in plain int32 arithmetic (src/fw_baseline_cpu.cpp:9-12,
// src/fw_tiling_gpu.cu:235-245). Padding outside the matrix is INF, as in the
// reference's tile loads (src/fw_tiling_gpu.cu:30-33), so a padded pivot
// never wins: INF + INF = 2e9 still fits in int32.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "fw103.h"

namespace fw {

constexpr int kInf = FW_INF;

// Blocked sweep geometry. A pivot block is 128 vertices wide; the matrix is
// processed in 128 x 128 tiles by 256-thread CTAs, each thread holding an
// 8 x 8 register micro-tile; operands stream through shared memory in slabs
// of 32 pivots.
constexpr int kTile = 128;
constexpr int kSlab = 32;
constexpr int kThreads = 256;
constexpr int kStages = 3;
constexpr int kSlabInts = kSlab * kTile;                 // one operand slab
constexpr int kStageInts = 2 * kSlabInts;                // A slab + B slab
constexpr int kSmemBytes = kStages * kStageInts * 4;     // 96 KB

// The micro-tile columns (bit c = column c of the 8) that fold a pivot pair
// with two DPX add-min instructions (form A); the other columns use form B
// (see relax2). Measured on GB300 with the TMA-fed remainder kernel, whole
// multi-layer solves (kappa 8, n = 32768): the first k columns in form A,
// 8 of 8 (DPX only) 1975 ms, 7 of 8 1918, 6 of 8 1797, 5 of 8 1806, 4 of 8
// 1807, 3 of 8 1715, 2 of 8 1846, 1 of 8 2045 ms. Then every set of two,
// three and four columns (154 builds of the library timed in one process,
// same matrix, bit-identical results): the fastest eight at n = 16384 re-timed
// at n = 32768 gave {0, 2, 5, 6} 1662.5 ms, {1, 2, 4, 6} 1668.7, {1, 3, 4, 5}
// 1673.7, {3, 4, 5, 6} 1674.6 ... {1, 4, 6} 1683.4 ms (at n = 16384 the best
// pair of columns, {1, 4}, was 12 % slower than {0, 2, 5, 6}). Which columns
// take form A changes how the compiler interleaves the two pipes.
constexpr unsigned cols_below(int k) { return (1u << k) - 1u; }
constexpr unsigned kColsA = (1u << 0) | (1u << 2) | (1u << 5) | (1u << 6);

// Register micro-tile ownership inside a 128 x 128 tile (thread t, tx = t % 16,
// ty = t / 16): rows ty*4 + {0..3} and 64 + ty*4 + {0..3}; columns
// tx*4 + {0..3} and 64 + tx*4 + {0..3}. Each group of 4 is one 16-byte
// vector in shared memory and in global memory.
__device__ __forceinline__ int own_row(int ty, int r) { return (r < 4) ? ty * 4 + r : 64 + ty * 4 + (r - 4); }
__device__ __forceinline__ int own_col(int tx, int c) { return (c < 4) ? tx * 4 + c : 64 + tx * 4 + (c - 4); }

// a * one + b with `one` a runtime 1: an integer multiply-add, which issues on
// the FMA pipe, instead of an add, which would issue on the ALU pipe that the
// DPX instructions already saturate. Exact: the low 32 bits of a*1 + b.
__device__ __forceinline__ int add_on_fma(int a, int b, int one) {
    int s;
    asm("mad.lo.s32 %0, %1, %3, %2;" : "=r"(s) : "r"(a), "r"(b), "r"(one));
    return s;
}

// Two pivots folded into one accumulator: min(acc, a0 + b0, a1 + b1).
// Form A: two DPX add-min instructions (ALU pipe). Form B: two multiply-adds
// (FMA pipe) and one three-way DPX min (ALU pipe). `form_a` is a compile-time
// constant at every call site once the micro-tile loops are unrolled.
__device__ __forceinline__ int relax2(bool form_a, int acc, int a0, int b0, int a1, int b1, int one) {
    if (form_a) {
        return __viaddmin_s32(a1, b1, __viaddmin_s32(a0, b0, acc));
    } else {
        return __vimin3_s32(acc, add_on_fma(a0, b0, one), add_on_fma(a1, b1, one));
    }
}

// One pivot pair of the 8 x 8 micro-tile update; the columns in COLS use form A.
template <unsigned COLS>
__device__ __forceinline__ void relax_tile_pair(int (&acc)[8][8], const int (&a0)[8], const int (&b0)[8],
                                                const int (&a1)[8], const int (&b1)[8], int one) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            acc[r][c] = relax2(((COLS >> c) & 1u) != 0, acc[r][c], a0[r], b0[c], a1[r], b1[c], one);
        }
    }
}

// Reads the thread's 8 A values (pivot row kk of a k-major A slab) and 8 B
// values into registers with four 16-byte shared loads.
__device__ __forceinline__ void load_frag(const int* As, const int* Bs, int kk, int tx, int ty, int (&a)[8],
                                          int (&b)[8]) {
    const int4 a_lo = *reinterpret_cast<const int4*>(As + kk * kTile + ty * 4);
    const int4 a_hi = *reinterpret_cast<const int4*>(As + kk * kTile + 64 + ty * 4);
    const int4 b_lo = *reinterpret_cast<const int4*>(Bs + kk * kTile + tx * 4);
    const int4 b_hi = *reinterpret_cast<const int4*>(Bs + kk * kTile + 64 + tx * 4);
    a[0] = a_lo.x; a[1] = a_lo.y; a[2] = a_lo.z; a[3] = a_lo.w;
    a[4] = a_hi.x; a[5] = a_hi.y; a[6] = a_hi.z; a[7] = a_hi.w;
    b[0] = b_lo.x; b[1] = b_lo.y; b[2] = b_lo.z; b[3] = b_lo.w;
    b[4] = b_hi.x; b[5] = b_hi.y; b[6] = b_hi.z; b[7] = b_hi.w;
}

// acc = min(acc, A (x) B) over one slab of kSlab pivots held in shared memory
// (A k-major [kSlab][128], B k-major [kSlab][128]).
template <unsigned COLS>
__device__ __forceinline__ void relax_slab(int (&acc)[8][8], const int* As, const int* Bs, int tx, int ty, int one) {
#pragma unroll 1
    for (int kk = 0; kk < kSlab; kk += 2) {
        int a0[8], b0[8], a1[8], b1[8];
        load_frag(As, Bs, kk, tx, ty, a0, b0);
        load_frag(As, Bs, kk + 1, tx, ty, a1, b1);
        relax_tile_pair<COLS>(acc, a0, b0, a1, b1, one);
    }
}

// ------------------------------------------------------------ async copies
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(smem_dst)), "l"(gmem_src)
                 : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// ------------------------------------------------------------ small vectors
template <int R>
__device__ __forceinline__ void ld_vec(const int* p, int (&v)[R]) {
    if constexpr (R % 4 == 0) {
#pragma unroll
        for (int q = 0; q < R; q += 4) {
            const int4 t = *reinterpret_cast<const int4*>(p + q);
            v[q] = t.x; v[q + 1] = t.y; v[q + 2] = t.z; v[q + 3] = t.w;
        }
    } else if constexpr (R == 2) {
        const int2 t = *reinterpret_cast<const int2*>(p);
        v[0] = t.x; v[1] = t.y;
    } else {
#pragma unroll
        for (int q = 0; q < R; ++q) v[q] = p[q];
    }
}

template <int R>
__device__ __forceinline__ void st_vec(int* p, const int (&v)[R]) {
    if constexpr (R % 4 == 0) {
#pragma unroll
        for (int q = 0; q < R; q += 4) *reinterpret_cast<int4*>(p + q) = make_int4(v[q], v[q + 1], v[q + 2], v[q + 3]);
    } else if constexpr (R == 2) {
        *reinterpret_cast<int2*>(p) = make_int2(v[0], v[1]);
    } else {
#pragma unroll
        for (int q = 0; q < R; ++q) p[q] = v[q];
    }
}

// Tile index sets of the remainder launches: either every tile index except
// up to two excluded ones (ex0 < ex1, -1 = none), or one single index.
struct TileSet {
    int single;  // >= 0: the only index; -1: all but the excluded ones
    int ex0, ex1;
};

__device__ __forceinline__ int tile_of(const TileSet& s, int idx) {
    if (s.single >= 0) return s.single;
    if (s.ex0 >= 0 && idx >= s.ex0) ++idx;
    if (s.ex1 >= 0 && idx >= s.ex1) ++idx;
    return idx;
}

__host__ __device__ inline TileSet all_but(int a, int b = -1) {
    if (b >= 0 && b < a) {
        const int t = a;
        a = b;
        b = t;
    }
    if (a < 0) {
        a = b;
        b = -1;
    }
    return TileSet{-1, a, b};
}
__host__ __device__ inline TileSet only(int t) { return TileSet{t, -1, -1}; }

// ------------------------------------------------------------ block closure
// Min-plus closure (the k-sequential Floyd-Warshall sweep) of an NB x NB block
// held in registers by a TY x TX grid of threads, each owning rows
// ty*RR .. ty*RR+RR-1 and columns tx*RC .. tx*RC+RC-1. Pivot k reads row k
// and column k from a shared-memory snapshot; after relaxing, the owners of
// row k+1 and column k+1 publish them into the other buffer, so each pivot
// costs one barrier and no thread reads a value another thread writes in the
// same pivot step. prow / pcol: 2 * NB ints each, 16-byte aligned. `kcount`
// pivots are applied, rounded up to the unroll width (padded pivots are INF
// rows and columns and change nothing). `sync` is the barrier of the
// participating threads.
template <int NB, int TY, int TX>
struct BlockClosure {
    static constexpr int RR = NB / TY;
    static constexpr int RC = NB / TX;
    static constexpr int U = RR > RC ? RR : RC;

    template <class Sync>
    __device__ __forceinline__ static void run(int (&c)[RR][RC], int* prow, int* pcol, int kcount, int tx, int ty,
                                               Sync sync) {
        if (ty == 0) st_vec<RC>(prow + tx * RC, c[0]);
        if (tx == 0) {
            int col[RR];
#pragma unroll
            for (int r = 0; r < RR; ++r) col[r] = c[r][0];
            st_vec<RR>(pcol + ty * RR, col);
        }
        sync();
        for (int kb = 0; kb < kcount; kb += U) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int k = kb + u;
                const int buf = k & 1;
                int a[RR], b[RC];
                ld_vec<RR>(pcol + buf * NB + ty * RR, a);
                ld_vec<RC>(prow + buf * NB + tx * RC, b);
#pragma unroll
                for (int r = 0; r < RR; ++r)
#pragma unroll
                    for (int e = 0; e < RC; ++e) c[r][e] = __viaddmin_s32(a[r], b[e], c[r][e]);
                const int k1 = k + 1;
                if (k1 < NB) {
                    // k1 % RR and k1 % RC, static because kb is a multiple of U
                    const int sr = (u + 1) % RR, sc = (u + 1) % RC;
                    if (ty == k1 / RR) st_vec<RC>(prow + (buf ^ 1) * NB + tx * RC, c[sr]);
                    if (tx == k1 / RC) {
                        int col[RR];
#pragma unroll
                        for (int r = 0; r < RR; ++r) col[r] = c[r][sc];
                        st_vec<RR>(pcol + (buf ^ 1) * NB + ty * RR, col);
                    }
                }
                sync();
            }
        }
    }
};

}  // namespace fw

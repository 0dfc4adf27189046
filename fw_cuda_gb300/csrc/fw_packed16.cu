// Exact packed 16-bit fast path for the int32 sweep (FW_VARIANT_AUTO).
//
// Every relaxation of the int32 sweep runs here as one half of a packed
// `__viaddmin_u16x2`, two relaxations per DPX instruction, on a 16-bit copy of
// the matrix, and the result is written back to the int32 matrix only when it
// is provably identical to what the int32 sweep (and so the reference's
// baseline_cpu, src/fw_baseline_cpu.cpp:6-15) returns; otherwise the int32
// blocked sweep runs instead. The decision is taken on the device, so the
// call stays asynchronous.
//
// Why it is exact. Let CAP = 32767. The input qualifies when every entry is
// either INF or an integer in [0, CAP). Entries are encoded as themselves,
// INF as CAP. Sums of two encoded values stay below 65535, so the packed
// add never wraps, and min(c, a + b) never exceeds CAP: the sweep computes the
// min-plus closure over [0, CAP] with every value = min(CAP, d), d the true
// shortest-path length over the real edges (weights are non-negative, so a
// path shorter than CAP has only prefixes shorter than CAP, all computed
// exactly). The int32 sweep returns d for reachable pairs and INF for the
// others. So entries below CAP are exact, and an entry equal to CAP is INF
// unless some finite d >= CAP exists. If one did, its shortest path would
// pass a vertex u whose prefix length lies in [CAP - w_max, CAP) (prefixes
// grow by at most the largest edge weight w_max), and d(i, u) is that prefix
// length. Hence: if the largest result below CAP is below CAP - w_max, every
// CAP entry is INF and decoding is exact; if not, the int32 sweep runs.
//
// Layout: D16 is the matrix as uint16, leading dimension ld16 = n rounded up
// to 256, padded with CAP (padded vertices have no edges). Tiles are
// 256 x 256 values on 512-thread CTAs; each thread holds 8 rows x 8 words
// (16 columns) in registers. The pivot block is 256 wide. The column panel is
// kept transposed in a workspace as 32-bit words with the 16-bit value in both
// halves (colD[k][i] = v | v << 16, the A operand of the packed add), the row
// panel as plain packed rows (rowP[k][*], the B operand).
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "fw_common.cuh"
#include "fw_internal.h"
#include "fw_tma.cuh"

namespace fw {
namespace {

constexpr uint32_t kCap = 0x7FFF;
constexpr int kPT = 256;           // tile / pivot block (values)
constexpr int kPW = kPT / 2;       // tile width in 32-bit words
constexpr int kPThreads = 512;     // 32 row groups x 16 word groups
constexpr int kPStages = 3;
constexpr int kPSlabA = kSlab * kPT;   // words: 32 pivots x 256 rows (duplicated values)
constexpr int kPSlabB = kSlab * kPW;   // words: 32 pivots x 128 words
constexpr int kPStageWords = kPSlabA + kPSlabB;
constexpr int kPSmemBytes = kPStages * kPStageWords * 4;  // 144 KB

struct P16Status {
    unsigned int ineligible;  // nonzero: some entry is neither INF nor in [0, CAP)
    unsigned int wmax;        // largest finite input entry
    unsigned int rmax;        // largest result entry below CAP
    unsigned int done;        // 1: D holds the decoded packed result
    unsigned int copy_fault;  // nonzero: a tile copy did not arrive in time (the int32 sweep runs)
};

__device__ __forceinline__ uint32_t dup16(uint32_t v) { return v | (v << 16); }

// Rows and words of a thread (tx = t % 16, ty = t / 16) in a 256 x 256 tile.
__device__ __forceinline__ int prow_of(int ty, int r) { return (r < 4) ? ty * 4 + r : 128 + ty * 4 + (r - 4); }
__device__ __forceinline__ int pword_of(int tx, int w) { return (w < 4) ? tx * 4 + w : 64 + tx * 4 + (w - 4); }

// ------------------------------------------------------------ encode / decode
// Row-parallel passes over the matrix, eight values per thread: one 16-byte
// D16 vector, two 16-byte int32 vectors when n % 4 == 0 and the eight values
// lie inside the row, single values otherwise. blockIdx.y strides over rows.
constexpr int kCodeThreads = 256;
__device__ __forceinline__ uint32_t encode1(int v, unsigned& bad, unsigned& wmax) {
    if (v == kInf) return kCap;
    if (v >= 0 && (uint32_t)v < kCap) {
        wmax = max(wmax, (unsigned)v);
        return (uint32_t)v;
    }
    bad = 1;
    return kCap;
}

__device__ __forceinline__ void reduce_status(unsigned bad, unsigned wmax, P16Status* st) {
    for (int o = 16; o > 0; o >>= 1) {
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
        wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (bad) atomicOr(&st->ineligible, 1u);
        if (wmax) atomicMax(&st->wmax, wmax);
    }
}

template <bool VEC>
__global__ void __launch_bounds__(kCodeThreads)
    fw_p16_encode_kernel(const int* __restrict__ D, int64_t n, uint16_t* __restrict__ D16, int64_t ld16,
                         P16Status* st) {
    unsigned bad = 0, wmax = 0;
    for (int64_t i = blockIdx.y; i < ld16; i += gridDim.y) {
        for (int64_t j0 = ((int64_t)blockIdx.x * kCodeThreads + threadIdx.x) * 8; j0 < ld16;
             j0 += (int64_t)gridDim.x * kCodeThreads * 8) {
            uint32_t e[8];
            if (VEC && i < n && j0 + 8 <= n) {
                const int4 a = *reinterpret_cast<const int4*>(D + i * n + j0);
                const int4 b = *reinterpret_cast<const int4*>(D + i * n + j0 + 4);
                e[0] = encode1(a.x, bad, wmax); e[1] = encode1(a.y, bad, wmax);
                e[2] = encode1(a.z, bad, wmax); e[3] = encode1(a.w, bad, wmax);
                e[4] = encode1(b.x, bad, wmax); e[5] = encode1(b.y, bad, wmax);
                e[6] = encode1(b.z, bad, wmax); e[7] = encode1(b.w, bad, wmax);
            } else {
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    e[u] = (i < n && j0 + u < n) ? encode1(D[i * n + j0 + u], bad, wmax) : kCap;
            }
            *reinterpret_cast<uint4*>(D16 + i * ld16 + j0) =
                make_uint4(e[0] | (e[1] << 16), e[2] | (e[3] << 16), e[4] | (e[5] << 16), e[6] | (e[7] << 16));
        }
    }
    reduce_status(bad, wmax, st);
}

__global__ void __launch_bounds__(kCodeThreads)
    fw_p16_rmax_kernel(const uint16_t* __restrict__ D16, int64_t n, int64_t ld16, P16Status* st) {
    if (st->ineligible || st->copy_fault) return;
    unsigned m = 0;
    for (int64_t i = blockIdx.y; i < n; i += gridDim.y) {
        for (int64_t j0 = ((int64_t)blockIdx.x * kCodeThreads + threadIdx.x) * 8; j0 < n;
             j0 += (int64_t)gridDim.x * kCodeThreads * 8) {
            const uint4 w = *reinterpret_cast<const uint4*>(D16 + i * ld16 + j0);
            const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint32_t v = (ws[u >> 1] >> ((u & 1) * 16)) & 0xFFFFu;
                if (j0 + u < n && v < kCap) m = max(m, v);
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(&st->rmax, m);
}

template <bool VEC>
__global__ void __launch_bounds__(kCodeThreads)
    fw_p16_decode_kernel(const uint16_t* __restrict__ D16, int* __restrict__ D, int64_t n, int64_t ld16,
                         P16Status* st) {
    if (st->ineligible || st->copy_fault || st->rmax + st->wmax >= kCap) return;  // the int32 sweep runs instead
    for (int64_t i = blockIdx.y; i < n; i += gridDim.y) {
        for (int64_t j0 = ((int64_t)blockIdx.x * kCodeThreads + threadIdx.x) * 8; j0 < n;
             j0 += (int64_t)gridDim.x * kCodeThreads * 8) {
            const uint4 w = *reinterpret_cast<const uint4*>(D16 + i * ld16 + j0);
            const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
            int o[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint32_t v = (ws[u >> 1] >> ((u & 1) * 16)) & 0xFFFFu;
                o[u] = (v == kCap) ? kInf : (int)v;
            }
            if (VEC && j0 + 8 <= n) {
                *reinterpret_cast<int4*>(D + i * n + j0) = make_int4(o[0], o[1], o[2], o[3]);
                *reinterpret_cast<int4*>(D + i * n + j0 + 4) = make_int4(o[4], o[5], o[6], o[7]);
            } else {
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (j0 + u < n) D[i * n + j0 + u] = o[u];
            }
        }
    }
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) st->done = 1;
}

// ------------------------------------------------------------ tile helpers
__device__ __forceinline__ const uint32_t* words(const uint16_t* p) { return reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ void p_load_tile(uint32_t (&c)[8][8], const uint16_t* D16, int64_t ldw, int64_t r0,
                                            int64_t w0, int tx, int ty) {
    const uint32_t* Dw = words(D16);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const uint32_t* row = Dw + (r0 + prow_of(ty, r)) * ldw + w0;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint4 t = *reinterpret_cast<const uint4*>(row + h * 64 + tx * 4);
            c[r][h * 4 + 0] = t.x; c[r][h * 4 + 1] = t.y; c[r][h * 4 + 2] = t.z; c[r][h * 4 + 3] = t.w;
        }
    }
}

__device__ __forceinline__ void p_store_tile(const uint32_t (&c)[8][8], uint16_t* D16, int64_t ldw, int64_t r0,
                                             int64_t w0, int tx, int ty) {
    uint32_t* Dw = reinterpret_cast<uint32_t*>(D16);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        uint32_t* row = Dw + (r0 + prow_of(ty, r)) * ldw + w0;
#pragma unroll
        for (int h = 0; h < 2; ++h)
            *reinterpret_cast<uint4*>(row + h * 64 + tx * 4) =
                make_uint4(c[r][h * 4 + 0], c[r][h * 4 + 1], c[r][h * 4 + 2], c[r][h * 4 + 3]);
    }
}

// Transposed, duplicated store of the tile: colD[k][r0 + i] = dup(tile[i][k]).
__device__ __forceinline__ void p_store_coldup(const uint32_t (&c)[8][8], uint32_t* colD, int64_t ldc, int64_t r0,
                                               int tx, int ty) {
#pragma unroll
    for (int w = 0; w < 8; ++w) {
        const int k0 = 2 * pword_of(tx, w);
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            uint32_t v[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) v[r] = dup16(half ? (c[r][w] >> 16) : (c[r][w] & 0xFFFFu));
            uint32_t* dst = colD + (int64_t)(k0 + half) * ldc + r0 + ty * 4;
            *reinterpret_cast<uint4*>(dst) = make_uint4(v[0], v[1], v[2], v[3]);
            *reinterpret_cast<uint4*>(dst + 128) = make_uint4(v[4], v[5], v[6], v[7]);
        }
    }
}

// Slab of a k-major word buffer: rows [k0, k0 + 32), `width` words from c0.
template <int WIDTH>
__device__ __forceinline__ void p_load_kmajor(uint32_t* dst, const uint32_t* buf, int64_t ld, int k0, int64_t c0,
                                              int tid) {
    constexpr int CH = WIDTH / 4;  // 16-byte chunks per row
    for (int q = tid; q < kSlab * CH; q += kPThreads) {
        const int row = q / CH, ch = q % CH;
        cp_async16(dst + row * WIDTH + ch * 4, buf + (int64_t)(k0 + row) * ld + c0 + ch * 4);
    }
}

// Transposed, duplicated slab of D16: dst[kk][i] = dup(D16[r0 + i][p0 + k0 + kk]).
__device__ __forceinline__ void p_load_transposed_dup(uint32_t* dst, const uint16_t* D16, int64_t ld16, int64_t r0,
                                                      int64_t kcol0, int tid) {
    for (int q = tid; q < kPT * (kSlab / 2); q += kPThreads) {
        const int i = q / (kSlab / 2), wp = q % (kSlab / 2);
        const uint32_t w = words(D16)[((r0 + i) * ld16 + kcol0) / 2 + wp];
        dst[(2 * wp) * kPT + i] = dup16(w & 0xFFFFu);
        dst[(2 * wp + 1) * kPT + i] = dup16(w >> 16);
    }
}

// The word columns (bit w = column w of the thread's 8) that fold a pivot
// pair with two packed DPX add-mins; the others add with two 32-bit
// multiply-adds (exact as packed adds: each half stays below 65535, so no
// carry crosses the halves) on the FMA pipe and take one packed three-way DPX
// min. Measured on GB300 with the TMA-fed remainder kernel (whole packed
// solve, n = 32768): the first k columns in form A, 7 of 8 964 ms, 6 of 8
// 942, 5 of 8 922, 4 of 8 884, 3 of 8 930, 2 of 8 978 ms; of the sets of
// four, the even columns 875 ms, columns 0-3 884, 2-5 894, {0,1,4,5} 895,
// {0,3,4,7} 919, odd 933, 4-7 947 ms. Every set of two to six columns
// (238 builds of the library timed in one process on the same matrix, all
// results bit-identical) kept the even columns first: at n = 16384 113.1 ms
// against 114.9 ms for the next ({1, 2, 3, 5}), and at n = 32768, for the
// eight fastest, 868.9 ms against 884.4-894.7 ms. The choice changes how the
// compiler schedules the two pipes.
constexpr unsigned kP16ColsA = 0x55u;

template <unsigned COLS>
__device__ __forceinline__ void p_relax_slab(uint32_t (&c)[8][8], const uint32_t* As, const uint32_t* Bs, int tx,
                                             int ty, int one) {
#pragma unroll 1
    for (int kk = 0; kk < kSlab; kk += 2) {
        uint32_t a0[8], b0[8], a1[8], b1[8];
        {
            const uint4 x0 = *reinterpret_cast<const uint4*>(As + kk * kPT + ty * 4);
            const uint4 x1 = *reinterpret_cast<const uint4*>(As + kk * kPT + 128 + ty * 4);
            const uint4 y0 = *reinterpret_cast<const uint4*>(Bs + kk * kPW + tx * 4);
            const uint4 y1 = *reinterpret_cast<const uint4*>(Bs + kk * kPW + 64 + tx * 4);
            a0[0] = x0.x; a0[1] = x0.y; a0[2] = x0.z; a0[3] = x0.w; a0[4] = x1.x; a0[5] = x1.y; a0[6] = x1.z; a0[7] = x1.w;
            b0[0] = y0.x; b0[1] = y0.y; b0[2] = y0.z; b0[3] = y0.w; b0[4] = y1.x; b0[5] = y1.y; b0[6] = y1.z; b0[7] = y1.w;
        }
        {
            const uint4 x0 = *reinterpret_cast<const uint4*>(As + (kk + 1) * kPT + ty * 4);
            const uint4 x1 = *reinterpret_cast<const uint4*>(As + (kk + 1) * kPT + 128 + ty * 4);
            const uint4 y0 = *reinterpret_cast<const uint4*>(Bs + (kk + 1) * kPW + tx * 4);
            const uint4 y1 = *reinterpret_cast<const uint4*>(Bs + (kk + 1) * kPW + 64 + tx * 4);
            a1[0] = x0.x; a1[1] = x0.y; a1[2] = x0.z; a1[3] = x0.w; a1[4] = x1.x; a1[5] = x1.y; a1[6] = x1.z; a1[7] = x1.w;
            b1[0] = y0.x; b1[1] = y0.y; b1[2] = y0.z; b1[3] = y0.w; b1[4] = y1.x; b1[5] = y1.y; b1[6] = y1.z; b1[7] = y1.w;
        }
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int w = 0; w < 8; ++w) {
                if ((COLS >> w) & 1u) {
                    c[r][w] = __viaddmin_u16x2(a1[r], b1[w], __viaddmin_u16x2(a0[r], b0[w], c[r][w]));
                } else {
                    const uint32_t s0 = (uint32_t)add_on_fma((int)a0[r], (int)b0[w], one);
                    const uint32_t s1 = (uint32_t)add_on_fma((int)a1[r], (int)b1[w], one);
                    c[r][w] = __vimin3_u16x2(c[r][w], s0, s1);
                }
            }
    }
}

template <unsigned COLS = kP16ColsA, class LA, class LB>
__device__ __forceinline__ void p_mainloop(uint32_t (&c)[8][8], int nslab, uint32_t* smem, LA la, LB lb, int tx,
                                           int ty, int one) {
#pragma unroll
    for (int s = 0; s < kPStages - 1; ++s) {
        if (s < nslab) {
            la(smem + s * kPStageWords, s);
            lb(smem + s * kPStageWords + kPSlabA, s);
        }
        cp_async_commit();
    }
    for (int kb = 0; kb < nslab; ++kb) {
        cp_async_wait<kPStages - 2>();
        __syncthreads();
        const int nxt = kb + kPStages - 1;
        if (nxt < nslab) {
            uint32_t* st = smem + (nxt % kPStages) * kPStageWords;
            la(st, nxt);
            lb(st + kPSlabA, nxt);
        }
        cp_async_commit();
        const uint32_t* st = smem + (kb % kPStages) * kPStageWords;
        p_relax_slab<COLS>(c, st, st + kPSlabA, tx, ty, one);
    }
}

// ------------------------------------------------------------ diagonal closure
// Thread (tx, ty) holds rows ty*4 + {0..3} and 128 + ty*4 + {0..3}, words
// tx*4 + {0..3} and 64 + tx*4 + {0..3} of the 256 x 256 block. Pivot k's row
// is row r = (k >= 128 ? 4 : 0) + k % 4 of ty = (k % 128) / 4; its column is
// half k % 2 of word w = (k >= 128 ? 4 : 0) + (k / 2) % 4 of tx = (k % 128) / 8.
// The owners publish pivot k + 1 into the other buffer after relaxing pivot k.
template <int RS, int WS, int HALF>
__device__ __forceinline__ void p_publish(const uint32_t (&c)[8][8], uint32_t* prw_next, uint32_t* pcl_next,
                                          bool row_owner, bool col_owner, int tx, int ty) {
    if (row_owner) {
        *reinterpret_cast<uint4*>(prw_next + tx * 4) = make_uint4(c[RS][0], c[RS][1], c[RS][2], c[RS][3]);
        *reinterpret_cast<uint4*>(prw_next + 64 + tx * 4) = make_uint4(c[RS][4], c[RS][5], c[RS][6], c[RS][7]);
    }
    if (col_owner) {
        uint32_t v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) v[r] = dup16(HALF ? (c[r][WS] >> 16) : (c[r][WS] & 0xFFFFu));
        *reinterpret_cast<uint4*>(pcl_next + ty * 4) = make_uint4(v[0], v[1], v[2], v[3]);
        *reinterpret_cast<uint4*>(pcl_next + 128 + ty * 4) = make_uint4(v[4], v[5], v[6], v[7]);
    }
}

// Pivot UPPER * 128 + kb + U (kb a multiple of 8); U is a template argument so
// that the owners' register indices are compile-time constants.
template <int UPPER, int U>
__device__ __forceinline__ void p_diag_step(uint32_t (&c)[8][8], uint32_t (*prw)[kPW], uint32_t (*pcl)[kPT], int tx,
                                            int ty, int kb) {
    constexpr int buf = U & 1;  // k & 1
    uint32_t a[8], b[8];
    {
        const uint4 x0 = *reinterpret_cast<const uint4*>(&pcl[buf][ty * 4]);
        const uint4 x1 = *reinterpret_cast<const uint4*>(&pcl[buf][128 + ty * 4]);
        const uint4 y0 = *reinterpret_cast<const uint4*>(&prw[buf][tx * 4]);
        const uint4 y1 = *reinterpret_cast<const uint4*>(&prw[buf][64 + tx * 4]);
        a[0] = x0.x; a[1] = x0.y; a[2] = x0.z; a[3] = x0.w; a[4] = x1.x; a[5] = x1.y; a[6] = x1.z; a[7] = x1.w;
        b[0] = y0.x; b[1] = y0.y; b[2] = y0.z; b[3] = y0.w; b[4] = y1.x; b[5] = y1.y; b[6] = y1.z; b[7] = y1.w;
    }
#pragma unroll
    for (int r = 0; r < 8; ++r)
#pragma unroll
        for (int w = 0; w < 8; ++w) c[r][w] = __viaddmin_u16x2(a[r], b[w], c[r][w]);
    uint32_t* prw_next = prw[buf ^ 1];
    uint32_t* pcl_next = pcl[buf ^ 1];
    if (U < 7) {
        // pivot k + 1 = UPPER * 128 + kb + U + 1, same group
        p_publish<UPPER * 4 + ((U + 1) & 3), UPPER * 4 + ((U + 1) >> 1), (U + 1) & 1>(
            c, prw_next, pcl_next, ty == ((kb + U + 1) >> 2), tx == (kb >> 3), tx, ty);
    } else if (!UPPER && kb == 120) {
        // pivot 128: row 4 of ty 0, low half of word 4 of tx 0
        p_publish<4, 4, 0>(c, prw_next, pcl_next, ty == 0, tx == 0, tx, ty);
    } else if (!(UPPER && kb == 120)) {
        // pivot k + 1 = UPPER * 128 + kb + 8, next group
        p_publish<UPPER * 4, UPPER * 4, 0>(c, prw_next, pcl_next, ty == ((kb + 8) >> 2), tx == ((kb + 8) >> 3), tx,
                                           ty);
    }
    __syncthreads();
}

// Pivots UPPER * 128 + [0, 128), eight per group.
template <int UPPER>
__device__ __forceinline__ void p_diag_phase(uint32_t (&c)[8][8], uint32_t (*prw)[kPW], uint32_t (*pcl)[kPT], int tx,
                                             int ty) {
    for (int kb = 0; kb < 128; kb += 8) {
        p_diag_step<UPPER, 0>(c, prw, pcl, tx, ty, kb);
        p_diag_step<UPPER, 1>(c, prw, pcl, tx, ty, kb);
        p_diag_step<UPPER, 2>(c, prw, pcl, tx, ty, kb);
        p_diag_step<UPPER, 3>(c, prw, pcl, tx, ty, kb);
        p_diag_step<UPPER, 4>(c, prw, pcl, tx, ty, kb);
        p_diag_step<UPPER, 5>(c, prw, pcl, tx, ty, kb);
        p_diag_step<UPPER, 6>(c, prw, pcl, tx, ty, kb);
        p_diag_step<UPPER, 7>(c, prw, pcl, tx, ty, kb);
    }
}

// ------------------------------------------------------------ kernels
// Closure of the 256 x 256 pivot block, one CTA; writes D16, colD (transposed,
// duplicated) and rowP (packed rows) for the block.
__global__ void __launch_bounds__(kPThreads, 1)
    fw_p16_diag_kernel(uint16_t* __restrict__ D16, int64_t ld16, int64_t p0, uint32_t* __restrict__ colD,
                       uint32_t* __restrict__ rowP, const P16Status* st) {
    if (st->ineligible) return;
    __shared__ __align__(16) uint32_t prw[2][kPW];  // pivot row, packed
    __shared__ __align__(16) uint32_t pcl[2][kPT];  // pivot column, duplicated
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    const int64_t ldw = ld16 / 2;
    uint32_t c[8][8];
    p_load_tile(c, D16, ldw, p0, p0 / 2, tx, ty);
    // pivot 0: row 0 is rows r = 0 of ty = 0; column 0 is the low half of word 0 (tx = 0, w = 0)
    if (ty == 0) {
#pragma unroll
        for (int w = 0; w < 8; ++w) prw[0][pword_of(tx, w)] = c[0][w];
    }
    if (tx == 0) {
#pragma unroll
        for (int r = 0; r < 8; ++r) pcl[0][prow_of(ty, r)] = dup16(c[r][0] & 0xFFFFu);
    }
    __syncthreads();
    p_diag_phase<0>(c, prw, pcl, tx, ty);
    p_diag_phase<1>(c, prw, pcl, tx, ty);
    p_store_tile(c, D16, ldw, p0, p0 / 2, tx, ty);
    p_store_coldup(c, colD, ld16, p0, tx, ty);
    // rowP rows are the pivot rows k = p0.. as packed words, ld = ld16 / 2
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        uint32_t* row = rowP + (int64_t)prow_of(ty, r) * ldw + p0 / 2;
#pragma unroll
        for (int h = 0; h < 2; ++h)
            *reinterpret_cast<uint4*>(row + h * 64 + tx * 4) =
                make_uint4(c[r][h * 4 + 0], c[r][h * 4 + 1], c[r][h * 4 + 2], c[r][h * 4 + 3]);
    }
}

// blockIdx.y == 0: row panel tile (P, J); == 1: column panel tile (I, P).
__global__ void __launch_bounds__(kPThreads, 1)
    fw_p16_panel_kernel(uint16_t* __restrict__ D16, int64_t ld16, int pt, uint32_t* __restrict__ colD,
                        uint32_t* __restrict__ rowP, const P16Status* st, int one) {
    if (st->ineligible) return;
    extern __shared__ __align__(128) uint32_t psm[];
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    const int other = (int)blockIdx.x < pt ? (int)blockIdx.x : (int)blockIdx.x + 1;
    const int64_t p0 = (int64_t)pt * kPT, q0 = (int64_t)other * kPT, ldw = ld16 / 2;
    uint32_t c[8][8];
    if (blockIdx.y == 0) {
        p_load_tile(c, D16, ldw, p0, q0 / 2, tx, ty);
        p_mainloop(
            c, kPT / kSlab, psm, [&](uint32_t* dst, int s) { p_load_kmajor<kPT>(dst, colD, ld16, s * kSlab, p0, tid); },
            [&](uint32_t* dst, int s) {
                p_load_kmajor<kPW>(dst, words(D16), ldw, (int)(p0 + s * kSlab), q0 / 2, tid);
            },
            tx, ty, one);
        p_store_tile(c, D16, ldw, p0, q0 / 2, tx, ty);
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            uint32_t* row = rowP + (int64_t)prow_of(ty, r) * ldw + q0 / 2;
#pragma unroll
            for (int h = 0; h < 2; ++h)
                *reinterpret_cast<uint4*>(row + h * 64 + tx * 4) =
                    make_uint4(c[r][h * 4 + 0], c[r][h * 4 + 1], c[r][h * 4 + 2], c[r][h * 4 + 3]);
        }
    } else {
        p_load_tile(c, D16, ldw, q0, p0 / 2, tx, ty);
        p_mainloop(
            c, kPT / kSlab, psm,
            [&](uint32_t* dst, int s) { p_load_transposed_dup(dst, D16, ld16, q0, p0 + s * kSlab, tid); },
            [&](uint32_t* dst, int s) { p_load_kmajor<kPW>(dst, rowP, ldw, s * kSlab, p0 / 2, tid); }, tx, ty, one);
        p_store_tile(c, D16, ldw, q0, p0 / 2, tx, ty);
        p_store_coldup(c, colD, ld16, q0, tx, ty);
    }
}

// ------------------------------------------------------------ TMA tile pipeline
// The remainder and cross tiles stream their operand slabs with the tensor
// memory accelerator: per 32-pivot slab one 2-D box of the column panel
// (32 x 256 words) and one of the row panel (32 x 128 words) land in a
// shared-memory stage and complete a per-stage mbarrier. Every wait is
// bounded; a copy that does not arrive sets copy_fault, the packed result is
// then not taken and the int32 sweep runs. After a miss the CTA issues no
// further copy, waits (bounded) for the ones it issued and leaves its tile.
constexpr uint32_t kPStageTx = (uint32_t)kPStageWords * 4;  // bytes per stage

// One tile (r0, w0) of D16 (row r0, word column w0) updated with the 256
// pivots of the panels behind mapA (colD) and mapB (rowP).
__device__ __forceinline__ void p_update_tile(uint16_t* __restrict__ D16, int64_t ld16, int64_t r0, int64_t w0,
                                              const CUtensorMap* mapA, const CUtensorMap* mapB, P16Status* st,
                                              int one) {
    extern __shared__ __align__(128) uint32_t psm[];
    __shared__ __align__(8) uint64_t bars[kPStages];
    __shared__ int s_ok;
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    const int64_t ldw = ld16 / 2;
    constexpr int nslab = kPT / kSlab;
    if (tid == 0) {
        // TMA destinations must be 128-byte aligned; the stage sizes keep every
        // stage and operand aligned when the base is.
        s_ok = (smem_u32(psm) & 127u) == 0;
        if (!s_ok) atomicOr(&st->copy_fault, 2u);
        for (int i = 0; i < kPStages; ++i) mbar_init(&bars[i], 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (!s_ok) return;
    auto issue = [&](int j) {  // slab j into stage j % kPStages, thread 0 only
        if (tid == 0) {
            const int stg = j % kPStages;
            uint32_t* dst = psm + stg * kPStageWords;
            mbar_expect_tx(&bars[stg], kPStageTx);
            tma_load_2d(dst, mapA, (int)r0, j * kSlab, &bars[stg]);
            tma_load_2d(dst + kPSlabA, mapB, (int)w0, j * kSlab, &bars[stg]);
        }
    };
    uint32_t c[8][8];
    p_load_tile(c, D16, ldw, r0, w0, tx, ty);
#pragma unroll
    for (int j = 0; j < kPStages - 1; ++j) issue(j);
    for (int kb = 0; kb < nslab; ++kb) {
        const int stg = kb % kPStages;
        // every thread is past slab kb - 1 (its stage can be refilled), and all
        // agree whether slab kb arrived
        if (!ring_wait_all(&bars[stg], (uint32_t)((kb / kPStages) & 1))) {
            if (tid == 0) atomicOr(&st->copy_fault, 1u);
            ring_drain(bars, kPStages, kb, min(kb + kPStages - 2, nslab - 1));
            return;
        }
        if (kb + kPStages - 1 < nslab) issue(kb + kPStages - 1);
        const uint32_t* stage = psm + stg * kPStageWords;
        p_relax_slab<kP16ColsA>(c, stage, stage + kPSlabA, tx, ty, one);
    }
    p_store_tile(c, D16, ldw, r0, w0, tx, ty);
}

// Remainder tiles (I, J), I from `rows`, J from `cols`, with the 256 pivots of
// the panels in colD / rowP.
__global__ void __launch_bounds__(kPThreads, 1)
    fw_p16_remainder_kernel(uint16_t* __restrict__ D16, int64_t ld16, TileSet rows, TileSet cols,
                            const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                            P16Status* st, int one) {
    if (st->ineligible) return;
    p_update_tile(D16, ld16, (int64_t)tile_of(rows, blockIdx.y) * kPT, (int64_t)tile_of(cols, blockIdx.x) * kPW,
                  &mapA, &mapB, st, one);
}

// Block t's update of block u = t + 1's row and column in one launch: CTAs
// [0, T - 1) take the row tiles (u, J), J != t; CTAs [T - 1, 2T - 3) the
// column tiles (I, u), I != t, u.
__global__ void __launch_bounds__(kPThreads, 1)
    fw_p16_cross_kernel(uint16_t* __restrict__ D16, int64_t ld16, int t, int T,
                        const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                        P16Status* st, int one) {
    if (st->ineligible) return;
    const int u = t + 1;
    int I, J;
    if ((int)blockIdx.x < T - 1) {
        I = u;
        J = tile_of(all_but(t), blockIdx.x);
    } else {
        I = tile_of(all_but(t, u), blockIdx.x - (T - 1));
        J = u;
    }
    p_update_tile(D16, ld16, (int64_t)I * kPT, (int64_t)J * kPW, &mapA, &mapB, st, one);
}

}  // namespace

int64_t p16_ld(int64_t n) { return (n + kPT - 1) / kPT * kPT; }

size_t p16_workspace_bytes(int64_t n) {
    const int64_t ld = p16_ld(n);
    return 256                                   // status
           + (size_t)ld * ld * 2                 // D16
           + 2 * ((size_t)kPT * ld * 4           // colD (duplicated words), two stage buffers
                  + (size_t)kPT * (ld / 2) * 4); // rowP (packed words), two stage buffers
}

// Enqueues encode, the packed sweep and the guarded decode on `s`; *done_flag
// receives the device address of the word that tells the int32 kernels to
// skip. The sweep looks one pivot block ahead (two panel buffers): see the
// schedule below.
int p16_solve(int32_t* D, int64_t n, void* ws, cudaStream_t s, const unsigned int** done_flag,
              bool inject_copy_fault) {
    static PerDeviceOnce attrs;
    if (int rc = once_per_device(attrs, [] {
            FW_CUDA_TRY(
                cudaFuncSetAttribute(fw_p16_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kPSmemBytes));
            FW_CUDA_TRY(
                cudaFuncSetAttribute(fw_p16_remainder_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kPSmemBytes));
            FW_CUDA_TRY(
                cudaFuncSetAttribute(fw_p16_cross_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kPSmemBytes));
            return (int)FW_OK;
        }))
        return rc;
    AuxStream aux;
    if (int rc = aux_stream_get(s, &aux)) return rc;
    const int64_t ld = p16_ld(n);
    const int T = (int)(ld / kPT);
    char* base = static_cast<char*>(ws);
    P16Status* st = reinterpret_cast<P16Status*>(base);
    uint16_t* D16 = reinterpret_cast<uint16_t*>(base + 256);
    uint32_t* colD[2];
    uint32_t* rowP[2];
    colD[0] = reinterpret_cast<uint32_t*>(base + 256 + (size_t)ld * ld * 2);
    rowP[0] = colD[0] + (size_t)kPT * ld;
    colD[1] = rowP[0] + (size_t)kPT * (ld / 2);
    rowP[1] = colD[1] + (size_t)kPT * ld;
    // TMA maps of the two panel buffers: colD rows of ld words (boxes of 256),
    // rowP rows of ld / 2 words (boxes of 128).
    CUtensorMap mapA[2], mapB[2];
    for (int b = 0; b < 2; ++b) {
        if (int rc = panel_map(&mapA[b], colD[b], (uint64_t)ld, kPT, kPT)) return rc;
        if (int rc = panel_map(&mapB[b], rowP[b], (uint64_t)(ld / 2), kPT, kPW)) return rc;
    }
    FW_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(P16Status), s));
    // Encode / check / decode: column chunks of 2048 values across blockIdx.x,
    // rows strided over blockIdx.y.
    const bool vec = (n % 4) == 0;
    const dim3 cgrid((unsigned)((ld + 8 * kCodeThreads - 1) / (8 * kCodeThreads)),
                     (unsigned)(ld < 2048 ? ld : 2048));
    if (vec)
        fw_p16_encode_kernel<true><<<cgrid, kCodeThreads, 0, s>>>(D, n, D16, ld, st);
    else
        fw_p16_encode_kernel<false><<<cgrid, kCodeThreads, 0, s>>>(D, n, D16, ld, st);
    FW_LAUNCH_CHECK("fw_p16_encode_kernel");

    auto kv = [&](int t) { return (double)((n - (int64_t)t * kPT) < kPT ? n - (int64_t)t * kPT : kPT); };
    auto close = [&](int t, cudaStream_t q) -> int {
        const int b = t & 1;
        prof_begin(KC_P16_DIAG, q);
        fw_p16_diag_kernel<<<1, kPThreads, 0, q>>>(D16, ld, (int64_t)t * kPT, colD[b], rowP[b], st);
        FW_LAUNCH_CHECK("fw_p16_diag_kernel");
        prof_end(KC_P16_DIAG, q, kv(t) * kv(t) * kv(t));
        if (T > 1) {
            prof_begin(KC_P16_PANEL, q);
            fw_p16_panel_kernel<<<dim3(T - 1, 2), kPThreads, kPSmemBytes, q>>>(D16, ld, t, colD[b], rowP[b], st, 1);
            FW_LAUNCH_CHECK("fw_p16_panel_kernel");
            prof_end(KC_P16_PANEL, q, 2.0 * ((double)n - kv(t)) * kv(t) * kv(t));
        }
        return FW_OK;
    };
    auto rows_of = [&](const TileSet& ts) {
        if (ts.single >= 0) return kv(ts.single);
        double r = (double)n;
        if (ts.ex0 >= 0) r -= kv(ts.ex0);
        if (ts.ex1 >= 0) r -= kv(ts.ex1);
        return r;
    };
    auto remainder = [&](int t, TileSet rows, int nrows, TileSet cols, int ncols, cudaStream_t q) -> int {
        if (nrows <= 0 || ncols <= 0) return FW_OK;
        const int b = t & 1;
        prof_begin(KC_P16_REMAINDER, q);
        fw_p16_remainder_kernel<<<dim3(ncols, nrows), kPThreads, kPSmemBytes, q>>>(D16, ld, rows, cols, mapA[b],
                                                                                  mapB[b], st, 1);
        FW_LAUNCH_CHECK("fw_p16_remainder_kernel");
        prof_end(KC_P16_REMAINDER, q, rows_of(rows) * rows_of(cols) * kv(t));
        return FW_OK;
    };

    // Block t's row and column update of block t + 1 (one launch).
    auto cross = [&](int t, cudaStream_t q) -> int {
        const int b = t & 1, u = t + 1;
        prof_begin(KC_P16_REMAINDER, q);
        fw_p16_cross_kernel<<<(unsigned)(2 * T - 3), kPThreads, kPSmemBytes, q>>>(D16, ld, t, T, mapA[b], mapB[b], st,
                                                                                 1);
        FW_LAUNCH_CHECK("fw_p16_cross_kernel");
        prof_end(KC_P16_REMAINDER, q, (kv(u) * ((double)n - kv(t)) + ((double)n - kv(t) - kv(u)) * kv(u)) * kv(t));
        return FW_OK;
    };

    // Schedule: the high-priority stream carries the chain that every later
    // block waits for — block t's update of block t+1's row and column, then
    // block t+1's closure and panels — while the side stream runs block t's
    // bulk remainder (every tile outside both blocks) concurrently. The chain
    // for block t+1 starts once the bulk of block t-1 is done (its tiles, and
    // the panel buffer block t+1 reuses).
    FW_CUDA_TRY(cudaEventRecord(aux.fork, s));
    FW_CUDA_TRY(cudaStreamWaitEvent(aux.hi, aux.fork, 0));
    FW_CUDA_TRY(cudaStreamWaitEvent(aux.side, aux.fork, 0));
    if (int rc = close(0, aux.hi)) return rc;
    FW_CUDA_TRY(cudaEventRecord(aux.panels[0], aux.hi));
    for (int t = 0; t < T; ++t) {
        if (t + 1 < T) {
            if (t >= 1) FW_CUDA_TRY(cudaStreamWaitEvent(aux.hi, aux.bulk[(t - 1) & 1], 0));
            if (int rc = cross(t, aux.hi)) return rc;
            if (int rc = close(t + 1, aux.hi)) return rc;
            FW_CUDA_TRY(cudaEventRecord(aux.panels[(t + 1) & 1], aux.hi));
        }
        FW_CUDA_TRY(cudaStreamWaitEvent(aux.side, aux.panels[t & 1], 0));
        if (t + 1 < T) {
            if (int rc = remainder(t, all_but(t, t + 1), T - 2, all_but(t, t + 1), T - 2, aux.side)) return rc;
        } else {
            if (int rc = remainder(t, all_but(t), T - 1, all_but(t), T - 1, aux.side)) return rc;
        }
        FW_CUDA_TRY(cudaEventRecord(aux.bulk[t & 1], aux.side));
    }
    // The side stream's last launch follows every launch of the chain.
    FW_CUDA_TRY(cudaStreamWaitEvent(s, aux.bulk[(T - 1) & 1], 0));
    if (inject_copy_fault) FW_CUDA_TRY(cudaMemsetAsync(&st->copy_fault, 0x01, 1, s));
    fw_p16_rmax_kernel<<<cgrid, kCodeThreads, 0, s>>>(D16, n, ld, st);
    FW_LAUNCH_CHECK("fw_p16_rmax_kernel");
    if (vec)
        fw_p16_decode_kernel<true><<<cgrid, kCodeThreads, 0, s>>>(D16, D, n, ld, st);
    else
        fw_p16_decode_kernel<false><<<cgrid, kCodeThreads, 0, s>>>(D16, D, n, ld, st);
    FW_LAUNCH_CHECK("fw_p16_decode_kernel");
    *done_flag = &st->done;
    return FW_OK;
}

}  // namespace fw

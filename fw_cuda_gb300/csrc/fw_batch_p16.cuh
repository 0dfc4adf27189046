// Exact packed 16-bit blocked sweep of one graph by one CTA, for the batched
// path (fw_batched.cu). The single-graph form is fw_packed16.cu; the argument
// for exactness is the same, taken per graph:
//
//   CAP = 32767. A graph qualifies when every entry is INF or an integer in
//   [0, CAP). Entries are encoded as themselves, INF as CAP, two per 32-bit
//   word; packed sums of two encoded values stay below 65535, so every value
//   the sweep computes is min(CAP, d) with d the true shortest-path length
//   (non-negative weights: a path shorter than CAP has only shorter
//   prefixes). Below CAP the results are exact; a CAP entry is INF unless a
//   finite d >= CAP exists, and then some vertex u on that path has
//   d(i, u) in [CAP - w_max, CAP). So when the largest result below CAP is
//   below CAP - w_max (w_max the largest finite entry), decoding CAP -> INF
//   gives the int32 sweep's result (src/fw_baseline_cpu.cpp:6-15) bit for
//   bit; otherwise the graph is left untouched and handed to the int32 path.
//
// The CTA (256 threads) keeps two 16-bit copies of the graph (leading
// dimension ld = n rounded up to 128 values, padded with CAP) in its
// workspace slice: E, the encoded input, and S, the matrix being swept. The
// first pivot block reads its tiles from E and writes them to S; later
// blocks work in S; the last block writes every tile, final, decoded
// (CAP -> INF) straight into the int32 graph and takes the largest result
// below CAP from registers. E stays as the input was, so a graph that fails
// the proof is restored from it before it is handed to the int32 path.
// Per 128-wide pivot block
// P: the closure of the diagonal block in registers; then the row panel
// min(R, Dg* x R) and, tile row after tile row, the column panel
// min(C, C x Dg*) and the remainder min(D, C x R) (plain min-plus products,
// Dg* being closed). The A operand of a product (128 rows x 128 pivots, each
// value duplicated into both halves of a word for the packed add-min) stays
// resident in shared memory for every tile that uses it: Dg* for the row
// panel, the tile row's pre-update column panel for its own product, then
// its updated column panel for the tile row's remainder tiles. The B operand
// (the pivot rows, packed words) streams from W's rows of P in 32-pivot
// slabs through a three-stage cp.async ring. A tile is 128 rows x 128 values
// = 64 words; each thread holds 8 rows x 4 words (16 bytes per row) and folds
// pivot pairs as the single-graph kernels do: two packed DPX add-mins
// (form A) or two 32-bit multiply-adds by a runtime 1 on the FMA pipe plus
// one packed three-way DPX min (form B; exact because every half is at most
// CAP, so no carry crosses into the other half).
#pragma once

#include <cstdint>

#include "fw_common.cuh"
#include "fw_tile.cuh"

namespace fw {

constexpr uint32_t kQCap = 0x7FFF;
constexpr int kQMaxN = 1024;                          // largest graph the packed batched path takes
constexpr int kQTileW = kTile / 2;                    // tile width in words
constexpr int kQPanelWords = kTile * kTile;           // resident A: 128 pivots x 128 rows (duplicated values)
constexpr int kQSlabB = kSlab * kQTileW;              // words: 32 pivots x 64 words
constexpr int kQSmemBytes = (kQPanelWords + kStages * kQSlabB) * 4;  // 64 KB + 24 KB
// Words (bit w of the thread's 4) that take form A: {1, 2} (the batched
// workload in 3.67 ms; {0, 2} 3.72, {0, 1} 3.71, {1, 3} 3.70, {0, 3} 3.74,
// {0} 3.78, {1, 2, 3} 3.72 ms).
constexpr unsigned kQWordsA = 0x6u;

// Words of one 16-bit copy of a graph `ld` values wide (ld a multiple of
// 128); a CTA's workspace slice holds two (E and S) for the largest graph.
__host__ __device__ inline int64_t q_copy_words(int64_t ld) { return ld * (ld / 2); }
__host__ __device__ inline int64_t q_ws_words(int64_t ld) { return 2 * q_copy_words(ld); }

// The resident A panel holds A[k][i] (pivot k, tile row i) at
// k * 128 + (i ^ q_swz(k)): rows of eight pivots are XOR-swizzled in 16-byte
// chunks, so that the transposed stores from registers (threads of a warp
// writing pivots 8 apart) spread over the banks, while every thread's
// 16-byte reads of four consecutive rows stay aligned.
__device__ __forceinline__ int q_swz(int k) { return ((k >> 3) & 7) << 2; }

__device__ __forceinline__ uint32_t q_dup(uint32_t v) { return v | (v << 16); }

// Two pivots folded into one packed accumulator word.
__device__ __forceinline__ uint32_t q_relax2(bool form_a, uint32_t acc, uint32_t a0, uint32_t b0, uint32_t a1,
                                             uint32_t b1, int one) {
    if (form_a) return __viaddmin_u16x2(a1, b1, __viaddmin_u16x2(a0, b0, acc));
    const uint32_t s0 = (uint32_t)add_on_fma((int)a0, (int)b0, one);
    const uint32_t s1 = (uint32_t)add_on_fma((int)a1, (int)b1, one);
    return __vimin3_u16x2(acc, s0, s1);
}

// acc = min(acc, A (x) B) over the 32 pivots [k0, k0 + 32): A the resident
// panel, B a k-major [32][64] slab of packed words. NR = 8: all of the
// thread's rows; NR = 4: its first four (rows 64.. of the tile lie outside
// the graph). The swizzle is constant over groups of eight pivots.
template <int NR>
__device__ __forceinline__ void q_relax_slab(uint32_t (&c)[8][4], const uint32_t* Ap, int k0, const uint32_t* Bs,
                                             int tx, int ty, int one) {
#pragma unroll 1
    for (int g = 0; g < kSlab; g += 8) {
        const int swz = q_swz(k0 + g);
        const uint32_t* A8 = Ap + (k0 + g) * kTile;
        const int lo = (ty * 4) ^ swz, hi = (64 + ty * 4) ^ swz;
#pragma unroll
        for (int kk = 0; kk < 8; kk += 2) {
            uint32_t a0[8], a1[8], b0[4], b1[4];
            const uint4 l0 = *reinterpret_cast<const uint4*>(A8 + kk * kTile + lo);
            const uint4 l1 = *reinterpret_cast<const uint4*>(A8 + (kk + 1) * kTile + lo);
            const uint4 q0 = *reinterpret_cast<const uint4*>(Bs + (g + kk) * kQTileW + tx * 4);
            const uint4 q1 = *reinterpret_cast<const uint4*>(Bs + (g + kk + 1) * kQTileW + tx * 4);
            a0[0] = l0.x; a0[1] = l0.y; a0[2] = l0.z; a0[3] = l0.w;
            a1[0] = l1.x; a1[1] = l1.y; a1[2] = l1.z; a1[3] = l1.w;
            if (NR == 8) {
                const uint4 h0 = *reinterpret_cast<const uint4*>(A8 + kk * kTile + hi);
                const uint4 h1 = *reinterpret_cast<const uint4*>(A8 + (kk + 1) * kTile + hi);
                a0[4] = h0.x; a0[5] = h0.y; a0[6] = h0.z; a0[7] = h0.w;
                a1[4] = h1.x; a1[5] = h1.y; a1[6] = h1.z; a1[7] = h1.w;
            }
            b0[0] = q0.x; b0[1] = q0.y; b0[2] = q0.z; b0[3] = q0.w;
            b1[0] = q1.x; b1[1] = q1.y; b1[2] = q1.z; b1[3] = q1.w;
#pragma unroll
            for (int r = 0; r < NR; ++r)
#pragma unroll
                for (int w = 0; w < 4; ++w)
                    c[r][w] = q_relax2(((kQWordsA >> w) & 1u) != 0, c[r][w], a0[r], b0[w], a1[r], b1[w], one);
        }
    }
}

// The thread's part of the tile held as c, transposed and duplicated into
// the resident A panel: A[k][i] = dup(value (i, k)) for the tile's rows i and
// columns k (column k = value 2 * word + half).
__device__ __forceinline__ void q_store_panel(const uint32_t (&c)[8][4], uint32_t* Ap, int tx, int ty) {
    const int swz = (tx & 7) << 2;  // q_swz(k) for every k = 8 tx + 0..7
#pragma unroll
    for (int w = 0; w < 4; ++w) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = 2 * (tx * 4 + w) + h;
            uint32_t v[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) v[r] = q_dup((c[r][w] >> (16 * h)) & 0xFFFFu);
            *reinterpret_cast<uint4*>(Ap + k * kTile + ((ty * 4) ^ swz)) = make_uint4(v[0], v[1], v[2], v[3]);
            *reinterpret_cast<uint4*>(Ap + k * kTile + ((64 + ty * 4) ^ swz)) = make_uint4(v[4], v[5], v[6], v[7]);
        }
    }
}

// Which of its rows a warp updates in a tile with `rows` rows inside the
// graph: warp w holds rows 8w .. 8w + 7 and 64 + 8w .. 64 + 8w + 7; rows
// outside the graph stay CAP whatever the pivots, so a warp skips them
// (2: all eight, 1: the first four, 0: none).
__device__ __forceinline__ int q_row_mode(int rows) {
    const int w = threadIdx.x >> 5;
    return (64 + 8 * w < rows) ? 2 : (8 * w < rows ? 1 : 0);
}

// The thread's 8 rows x 4 words of the tile at (r0, word w0) of a packed
// matrix with `ldw` words per row.
__device__ __forceinline__ void q_load_tile(uint32_t (&c)[8][4], const uint32_t* Wm, int64_t ldw, int64_t r0,
                                            int64_t w0, int tx, int ty) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const uint4 t = *reinterpret_cast<const uint4*>(Wm + (r0 + own_row(ty, r)) * ldw + w0 + tx * 4);
        c[r][0] = t.x; c[r][1] = t.y; c[r][2] = t.z; c[r][3] = t.w;
    }
}

__device__ __forceinline__ void q_store_tile(const uint32_t (&c)[8][4], uint32_t* Wm, int64_t ldw, int64_t r0,
                                             int64_t w0, int tx, int ty) {
#pragma unroll
    for (int r = 0; r < 8; ++r)
        *reinterpret_cast<uint4*>(Wm + (r0 + own_row(ty, r)) * ldw + w0 + tx * 4) =
            make_uint4(c[r][0], c[r][1], c[r][2], c[r][3]);
}

// The thread's 8 rows x 8 values of the tile at (r0, word w0), final:
// decoded (CAP -> INF) into the n x n int32 graph G (rows of n values, any
// alignment; rows and columns past n are padding and skipped), and
// m = max(m, every value below CAP). Padding is CAP throughout the sweep, so
// it never counts.
__device__ __forceinline__ void q_store_tile_i32(const uint32_t (&c)[8][4], int* __restrict__ G, int n, int r0,
                                                 int w0, int tx, int ty, unsigned& m) {
    const int col0 = 2 * (w0 + tx * 4);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        int v[8];
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            const uint32_t lo = c[r][w] & 0xFFFFu, hi = c[r][w] >> 16;
            if (lo < kQCap) m = max(m, lo);
            if (hi < kQCap) m = max(m, hi);
            v[2 * w] = lo == kQCap ? kInf : (int)lo;
            v[2 * w + 1] = hi == kQCap ? kInf : (int)hi;
        }
        const int row = r0 + own_row(ty, r);
        if (row >= n) continue;
        int* p = G + (int64_t)row * n + col0;
        if (col0 + 8 <= n) {
            const uintptr_t a = reinterpret_cast<uintptr_t>(p);
            if ((a & 15) == 0) {
                reinterpret_cast<int4*>(p)[0] = make_int4(v[0], v[1], v[2], v[3]);
                reinterpret_cast<int4*>(p)[1] = make_int4(v[4], v[5], v[6], v[7]);
            } else if ((a & 7) == 0) {
#pragma unroll
                for (int e = 0; e < 4; ++e) reinterpret_cast<int2*>(p)[e] = make_int2(v[2 * e], v[2 * e + 1]);
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e) p[e] = v[e];
            }
        } else {
#pragma unroll
            for (int e = 0; e < 8; ++e)
                if (col0 + e < n) p[e] = v[e];
        }
    }
}

// k-major slab [32][width] words from rows k0.. of a buffer with `ld` words
// per row, columns c0.. (16-byte aligned), by cp.async.
template <int WIDTH>
__device__ __forceinline__ void q_load_kmajor_async(uint32_t* dst, const uint32_t* buf, int64_t ld, int k0, int64_t c0,
                                                    int tid) {
    constexpr int kVecs = kSlab * WIDTH / 4;
#pragma unroll
    for (int q = tid; q < kVecs; q += kThreads) {
        const int row = q / (WIDTH / 4), ch = q % (WIDTH / 4);
        cp_async16(dst + row * WIDTH + ch * 4, buf + (int64_t)(k0 + row) * ld + c0 + ch * 4);
    }
}

// acc = min(acc, A (x) B) over `nslab` slabs: A the resident panel, B
// streamed through a three-stage cp.async ring (the int32 mainloop's
// schedule); lb fills slab s of B. `rows`: the tile's rows inside the graph
// (see q_row_mode).
template <class LB>
__device__ __forceinline__ void q_mainloop(uint32_t (&c)[8][4], int nslab, int rows, const uint32_t* Ap,
                                           uint32_t* Bst, LB lb, int tx, int ty, int one) {
    const int mode = q_row_mode(rows);
#pragma unroll
    for (int s = 0; s < kStages - 1; ++s) {
        if (s < nslab) lb(Bst + s * kQSlabB, s);
        cp_async_commit();
    }
    for (int kb = 0; kb < nslab; ++kb) {
        cp_async_wait<kStages - 2>();
        __syncthreads();
        const int nxt = kb + kStages - 1;
        if (nxt < nslab) lb(Bst + (nxt % kStages) * kQSlabB, nxt);
        cp_async_commit();
        const uint32_t* Bs = Bst + (kb % kStages) * kQSlabB;
        if (mode == 2)
            q_relax_slab<8>(c, Ap, kb * kSlab, Bs, tx, ty, one);
        else if (mode == 1)
            q_relax_slab<4>(c, Ap, kb * kSlab, Bs, tx, ty, one);
    }
    cp_async_wait<0>();
}

// Publishes pivot k (k & 7 == U, so the thread's register row and word are
// compile-time) of the block held as c: row k into prow (64 words), column k
// duplicated into pcol (128 words).
template <int U>
__device__ __forceinline__ void q_publish(const uint32_t (&c)[8][4], int k, uint32_t* prow, uint32_t* pcol, int tx,
                                          int ty) {
    constexpr int lo = U & 3;          // row k within its group of four rows
    constexpr int w = (U >> 1) & 3;    // the word of column k among the thread's four
    constexpr int sh = (U & 1) * 16;   // the half of that word
    if (ty == ((k & 63) >> 2)) {       // row k = own_row(ty, lo + 4 * (k >> 6))
        const bool hi = (k >> 6) != 0;
        *reinterpret_cast<uint4*>(prow + tx * 4) =
            make_uint4(hi ? c[4 + lo][0] : c[lo][0], hi ? c[4 + lo][1] : c[lo][1], hi ? c[4 + lo][2] : c[lo][2],
                       hi ? c[4 + lo][3] : c[lo][3]);
    }
    if (tx == (k >> 3)) {  // column k = value 2 * (tx * 4 + w) + U % 2
        uint32_t v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) v[r] = q_dup((c[r][w] >> sh) & 0xFFFFu);
        *reinterpret_cast<uint4*>(pcol + ty * 4) = make_uint4(v[0], v[1], v[2], v[3]);
        *reinterpret_cast<uint4*>(pcol + 64 + ty * 4) = make_uint4(v[4], v[5], v[6], v[7]);
    }
}

// Pivot k = kb + U of the closure: relax with the snapshot in buffer U & 1,
// publish pivot k + 1 into the other buffer, one barrier.
template <int U>
__device__ __forceinline__ void q_close_step(uint32_t (&c)[8][4], uint32_t* prow, uint32_t* pcol, int k, int kr,
                                             int tx, int ty) {
    constexpr int buf = U & 1;
    const uint4 al = *reinterpret_cast<const uint4*>(pcol + buf * kTile + ty * 4);
    const uint4 ah = *reinterpret_cast<const uint4*>(pcol + buf * kTile + 64 + ty * 4);
    const uint4 bq = *reinterpret_cast<const uint4*>(prow + buf * kQTileW + tx * 4);
    const uint32_t a[8] = {al.x, al.y, al.z, al.w, ah.x, ah.y, ah.z, ah.w};
    const uint32_t b[4] = {bq.x, bq.y, bq.z, bq.w};
#pragma unroll
    for (int r = 0; r < 8; ++r)
#pragma unroll
        for (int w = 0; w < 4; ++w) c[r][w] = __viaddmin_u16x2(a[r], b[w], c[r][w]);
    if (k + 1 < kr) q_publish<(U + 1) & 7>(c, k + 1, prow + (buf ^ 1) * kQTileW, pcol + (buf ^ 1) * kTile, tx, ty);
    __syncthreads();
}

// Closure of the diagonal block held as c (rows own_row(ty, r), words
// tx*4..) over its first `kv` pivots, rounded up to a multiple of 8 (the
// pivots past kv lie outside the graph: CAP rows and columns, which change
// nothing). prow: 2 x 64 words, pcol: 2 x 128 duplicated words, snapshots of
// the pivot row and column double-buffered so that each pivot costs one
// barrier and no thread reads what another writes in the same step.
__device__ __forceinline__ void q_close(uint32_t (&c)[8][4], uint32_t* prow, uint32_t* pcol, int kv, int tx, int ty) {
    const int kr = (kv + 7) & ~7;
    q_publish<0>(c, 0, prow, pcol, tx, ty);
    __syncthreads();
    for (int kb = 0; kb < kr; kb += 8) {
        q_close_step<0>(c, prow, pcol, kb + 0, kr, tx, ty);
        q_close_step<1>(c, prow, pcol, kb + 1, kr, tx, ty);
        q_close_step<2>(c, prow, pcol, kb + 2, kr, tx, ty);
        q_close_step<3>(c, prow, pcol, kb + 3, kr, tx, ty);
        q_close_step<4>(c, prow, pcol, kb + 4, kr, tx, ty);
        q_close_step<5>(c, prow, pcol, kb + 5, kr, tx, ty);
        q_close_step<6>(c, prow, pcol, kb + 6, kr, tx, ty);
        q_close_step<7>(c, prow, pcol, kb + 7, kr, tx, ty);
    }
}

// Per-graph proof state, in shared memory.
struct QProof {
    unsigned bad;   // some entry is neither INF nor in [0, CAP)
    unsigned wmax;  // largest finite entry
    unsigned rmax;  // largest result below CAP
};

// The per-graph passes below give each warp whole rows and each lane
// consecutive columns (coalesced accesses to the graph's unaligned int32
// rows), with kQPassU independent loads per lane in flight.
constexpr int kQPassU = 4;

__device__ __forceinline__ uint32_t q_encode1(int v, unsigned& bad, unsigned& wmax) {
    if (v == kInf) return kQCap;
    if (v >= 0 && (uint32_t)v < kQCap) {
        wmax = max(wmax, (uint32_t)v);
        return (uint32_t)v;
    }
    bad = 1;
    return kQCap;
}

// W = encode(G) for an n x n int32 graph at G (row-major, rows need not be
// aligned); W has `ld` values (ld / 2 words) per row and ld rows, padding CAP.
__device__ __forceinline__ void q_encode(const int* __restrict__ G, int n, uint32_t* __restrict__ Wm, int ld,
                                         QProof* pf) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ldw = ld / 2;
    unsigned bad = 0, wmax = 0;
    for (int i = warp; i < ld; i += kThreads / 32) {
        const int* row = G + (int64_t)i * n;
        for (int jw0 = 0; jw0 < ldw; jw0 += 32 * kQPassU) {
            int v[kQPassU][2];
#pragma unroll
            for (int u = 0; u < kQPassU; ++u) {
                const int j = 2 * (jw0 + u * 32 + lane);
                v[u][0] = (i < n && j < n) ? __ldg(row + j) : kInf;
                v[u][1] = (i < n && j + 1 < n) ? __ldg(row + j + 1) : kInf;
            }
#pragma unroll
            for (int u = 0; u < kQPassU; ++u) {
                const int jw = jw0 + u * 32 + lane;
                if (jw < ldw)
                    Wm[(int64_t)i * ldw + jw] = q_encode1(v[u][0], bad, wmax) | (q_encode1(v[u][1], bad, wmax) << 16);
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
        wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
    }
    if (lane == 0) {
        if (bad) atomicOr(&pf->bad, 1u);
        if (wmax) atomicMax(&pf->wmax, wmax);
    }
}

// G = decode(W) (CAP -> INF) for the graph's n x n entries: restores the
// input from E when a graph fails the proof.
__device__ __forceinline__ void q_decode(const uint32_t* __restrict__ Wm, int* __restrict__ G, int n, int ld) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ldw = ld / 2;
    for (int i = warp; i < n; i += kThreads / 32) {
        const uint32_t* wrow = Wm + (int64_t)i * ldw;
        int* row = G + (int64_t)i * n;
        for (int j0 = 0; j0 < n; j0 += 32 * kQPassU) {
            uint32_t x[kQPassU];
#pragma unroll
            for (int u = 0; u < kQPassU; ++u) {
                const int j = j0 + u * 32 + lane;
                x[u] = (j < n) ? wrow[j >> 1] : 0u;
            }
#pragma unroll
            for (int u = 0; u < kQPassU; ++u) {
                const int j = j0 + u * 32 + lane;
                if (j < n) {
                    const uint32_t v = (x[u] >> ((j & 1) * 16)) & 0xFFFFu;
                    row[j] = (v == kQCap) ? kInf : (int)v;
                }
            }
        }
    }
}

// The blocked sweep of the graph (ld x ld values, T = ld / 128 blocks, n
// valid): the first block reads E and writes S, later blocks read and write
// S, and the last block writes its tiles into G (int32) instead, except the
// diagonal block and the row panel, which its later steps read as B and so
// also go to S. Returns the thread's largest result below CAP.
// smem: the resident A panel (kQPanelWords), then the B ring (kStages x
// kQSlabB words; its start also holds the closure's pivot buffers).
__device__ __forceinline__ unsigned q_sweep(const uint32_t* E, uint32_t* S, int* G, int n, int ld, uint32_t* smem,
                                            int one) {
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int T = ld / kTile;
    const int64_t ldw = ld / 2;
    uint32_t* Ap = smem;
    uint32_t* Bst = smem + kQPanelWords;
    unsigned m = 0;
    for (int pt = 0; pt < T; ++pt) {
        const int p0 = pt * kTile, pw0 = p0 / 2;
        const int kv = min(kTile, n - p0);
        const int nslab = (kv + kSlab - 1) / kSlab;
        const uint32_t* src = pt == 0 ? E : S;  // tiles before this block's update
        const bool last = pt == T - 1;
        // B slabs: rows p0 + 32 s .. (the pivot rows), words w0 .., of `from`
        auto pivot_rows = [&](const uint32_t* from, int64_t w0) {
            return [=](uint32_t* dst, int sl) { q_load_kmajor_async<kQTileW>(dst, from, ldw, p0 + sl * kSlab, w0, tid); };
        };
        uint32_t c[8][4];
        // 1. diagonal block: closure in registers; S and the resident A = Dg*
        q_load_tile(c, src, ldw, p0, pw0, tx, ty);
        q_close(c, Bst, Bst + 2 * kQTileW, kv, tx, ty);
        q_store_tile(c, S, ldw, p0, pw0, tx, ty);
        if (last) q_store_tile_i32(c, G, n, p0, pw0, tx, ty, m);
        q_store_panel(c, Ap, tx, ty);
        __syncthreads();
        // 2. row panel: S[P][J] = min(X[P][J], Dg* (x) X[P][J]), X = src: B the
        //    tile's own rows before the update (in S from the second block on,
        //    where every thread has read them before the last slab's barrier,
        //    so the stores after the loop are safe)
        for (int tj = 0; tj < T; ++tj) {
            if (tj == pt) continue;
            const int64_t w0 = (int64_t)tj * kQTileW;
            q_load_tile(c, src, ldw, p0, w0, tx, ty);
            q_mainloop(c, nslab, kv, Ap, Bst, pivot_rows(src, w0), tx, ty, one);
            q_store_tile(c, S, ldw, p0, w0, tx, ty);
            if (last) q_store_tile_i32(c, G, n, p0, (int)w0, tx, ty, m);
            __syncthreads();  // the next tile's prologue refills the ring
        }
        // 3. tile row after tile row
        for (int ti = 0; ti < T; ++ti) {
            if (ti == pt) continue;
            const int r0 = ti * kTile;
            const int rows = min(kTile, n - r0);
            // column panel min(C, C (x) Dg*): A = C (before the update), B = Dg* rows (S)
            q_load_tile(c, src, ldw, r0, pw0, tx, ty);
            q_store_panel(c, Ap, tx, ty);
            __syncthreads();
            q_mainloop(c, nslab, rows, Ap, Bst, pivot_rows(S, pw0), tx, ty, one);
            __syncthreads();  // every thread is done with A = C before it becomes C'
            if (last)
                q_store_tile_i32(c, G, n, r0, pw0, tx, ty, m);
            else
                q_store_tile(c, S, ldw, r0, pw0, tx, ty);
            q_store_panel(c, Ap, tx, ty);
            __syncthreads();
            // remainder min(X[I][J], C' (x) S[P][J]), J != P
            for (int tj = 0; tj < T; ++tj) {
                if (tj == pt) continue;
                const int64_t w0 = (int64_t)tj * kQTileW;
                q_load_tile(c, src, ldw, r0, w0, tx, ty);
                q_mainloop(c, nslab, rows, Ap, Bst, pivot_rows(S, w0), tx, ty, one);
                if (last)
                    q_store_tile_i32(c, G, n, r0, (int)w0, tx, ty, m);
                else
                    q_store_tile(c, S, ldw, r0, w0, tx, ty);
                __syncthreads();  // the next tile's prologue refills the ring; the A panel is rewritten next
            }
        }
    }
    return m;
}

}  // namespace fw

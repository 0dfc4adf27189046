// Batched APSP: thousands of independent graphs of uneven size in one
// persistent launch. No reference counterpart; each graph's result is the
// reference's k-i-j sweep (src/fw_baseline_cpu.cpp:6-15) of that graph.
//
// Layout: every graph g is an n_g x n_g int32 row-major matrix at element
// offset offsets[g] of one packed device buffer, solved in place.
//
// Plan (host, once per batch shape): the graphs are sorted by size, largest
// first, and split into buckets:
//   bucket 0  n > 128        a whole CTA runs the blocked sweep on the graph
//                            (128-wide pivot blocks, the same diag / panel /
//                            remainder tiles and pipelined main loop as the
//                            single-graph engine, the column panel kept in a
//                            per-CTA workspace slice), tile after tile;
//   bucket 1  64 < n <= 128  the graph lives in the registers of one CTA and
//                            is closed by BlockClosure<128>;
//   bucket 2  32 < n <= 64   likewise, padded to 64, by 1 or 4 graphs per CTA;
//   bucket 3  16 < n <= 32   padded to 32, 1, 4 or 8 graphs per CTA;
//   bucket 4        n <= 16  padded to 16, 1, 4 or 8 graphs per CTA.
// The kernel is persistent: each CTA (or each group of threads inside it)
// takes the next graph of the current bucket from an atomic counter, so
// large graphs start first and small ones fill in behind them. The launch
// (counter reset + kernel) is captured once into a CUDA graph per packed
// buffer and replayed. The autotuner picks, per bucket, how many graphs share
// a CTA, and the number of resident CTAs per SM, by timing the candidates on
// a scratch copy of the batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "fw_batch_p16.cuh"
#include "fw_common.cuh"
#include "fw_internal.h"
#include "fw_tile.cuh"

namespace fw {
namespace {

constexpr int kBuckets = 5;
constexpr int kBatchMaxN = 4096;
// Device counters of one launch: one per bucket of the int32 kernel, the
// packed kernel's graph counter, the length of its hand-back list.
constexpr int kCounters = kBuckets + 2;
constexpr int kQCounter = kBuckets, kFallbackCount = kBuckets + 1;
// Form-A columns of the per-CTA sweep (see kColsA), chosen apart from the
// TMA-fed remainder's because its slabs arrive by cp.async.
constexpr unsigned kBatchedColsA = cols_below(5);

struct BatchItem {
    int64_t offset;
    int32_t n;
    int32_t index;
};

struct BatchSched {
    int start[kBuckets];
    int count[kBuckets];
    int groups[kBuckets];  // graphs per CTA (small buckets): 1, 4 or 8
};

__device__ __forceinline__ void named_sync(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// ------------------------------------------------------------ small graphs
// One graph of n <= NB held in the registers of a group of 256/G threads.
// The graph (n*n contiguous ints) is staged through shared memory with
// coalesced copies in and out; the pivot buffers of all groups come first.
constexpr int kPivotInts = 8 * 4 * 32;  // >= G * 4 * NB for every (NB, G) used

template <int NB, int G>
__device__ __forceinline__ void small_bucket(int* __restrict__ packed, const BatchItem* __restrict__ items, int start,
                                             int count, int* counter, int* smem, int* s_item) {
    constexpr int GS = kThreads / G;
    constexpr int TY = (GS == 256) ? 16 : 8;
    constexpr int TX = GS / TY;
    using Closure = BlockClosure<NB, TY, TX>;
    constexpr int RR = Closure::RR, RC = Closure::RC;
    static_assert(G * 4 * NB <= kPivotInts, "pivot buffers exceed their area");
    static_assert(kPivotInts + G * NB * NB <= kSmemBytes / 4, "staging exceeds shared memory");
    const int g = threadIdx.x / GS, gt = threadIdx.x % GS;
    const int tx = gt % TX, ty = gt / TX;
    int* prow = smem + g * 4 * NB;
    int* pcol = prow + 2 * NB;
    int* stage = smem + kPivotInts + g * NB * NB;
    auto gsync = [g] {
        if constexpr (GS == 256) {
            __syncthreads();
        } else if constexpr (GS == 32) {
            __syncwarp();
        } else {
            named_sync(1 + g, GS);
        }
    };
    for (;;) {
        if (gt == 0) s_item[g] = atomicAdd(counter, 1);
        gsync();
        const int it = s_item[g];
        gsync();
        if (it >= count) break;
        const BatchItem item = items[start + it];
        int* Gm = packed + item.offset;
        const int n = item.n;
        const int nn = n * n;
        for (int q = gt; q < nn; q += GS) stage[q] = Gm[q];
        gsync();
        int c[RR][RC];
#pragma unroll
        for (int r = 0; r < RR; ++r) {
            const int i = ty * RR + r;
            const int* row = stage + i * n + tx * RC;
#pragma unroll
            for (int e = 0; e < RC; ++e) c[r][e] = (i < n && tx * RC + e < n) ? row[e] : kInf;
        }
        Closure::run(c, prow, pcol, n, tx, ty, gsync);
#pragma unroll
        for (int r = 0; r < RR; ++r) {
            const int i = ty * RR + r;
            int* row = stage + i * n + tx * RC;
#pragma unroll
            for (int e = 0; e < RC; ++e)
                if (i < n && tx * RC + e < n) row[e] = c[r][e];
        }
        gsync();
        for (int q = gt; q < nn; q += GS) Gm[q] = stage[q];
    }
}

template <int NB>
__device__ __forceinline__ void small_bucket_any(int groups, int* packed, const BatchItem* items, int start, int count,
                                                 int* counter, int* smem, int* s_item) {
    if constexpr (NB <= 32) {
        if (groups == 8) return small_bucket<NB, 8>(packed, items, start, count, counter, smem, s_item);
    }
    if constexpr (NB <= 64) {
        if (groups == 4) return small_bucket<NB, 4>(packed, items, start, count, counter, smem, s_item);
    }
    small_bucket<NB, 1>(packed, items, start, count, counter, smem, s_item);
}

// ------------------------------------------------------------ one large graph
// The blocked sweep of one n x n graph by one CTA: per 128-wide pivot block,
// the diagonal closure, the row and column panels, then the remainder tiles,
// one tile at a time. This CTA's workspace slice holds the current panels in
// the single-graph engine's layout: colT (128 x ldw ints) the column panel
// transposed, rowP (128 x ldw) the row panel, so the remainder streams both
// operands with 16-byte cp.async whatever the graph's row alignment.
// The graph's n x n values sit in G with leading dimension ldg (ldg = n in
// place; ldg = the padded staging width, a multiple of 128 with INF padding,
// when VEC), so the tile helpers take ldg as the matrix extent.
template <bool VEC>
__device__ __forceinline__ void blocked_in_cta(int* __restrict__ Gm, int n, int64_t ldg, int* __restrict__ colT,
                                               int* __restrict__ rowP, int64_t ldw, int* smem, int one) {
    using Closure = BlockClosure<kTile, 16, 16>;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int T = (n + kTile - 1) / kTile;
    for (int pt = 0; pt < T; ++pt) {
        const int p0 = pt * kTile;
        const int kv = min(kTile, n - p0);
        const int nslab = (kv + kSlab - 1) / kSlab;
        {  // 1. diagonal block
            int c[8][8];
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int i = ty * 8 + r;
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int j = tx * 8 + e;
                    c[r][e] = (i < kv && j < kv) ? Gm[(int64_t)(p0 + i) * ldg + p0 + j] : kInf;
                }
            }
            Closure::run(c, smem, smem + 2 * kTile, kv, tx, ty, [] { __syncthreads(); });
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int i = ty * 8 + r;
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int j = tx * 8 + e;
                    if (i < kv && j < kv) Gm[(int64_t)(p0 + i) * ldg + p0 + j] = c[r][e];
                }
            }
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                int col[8];
#pragma unroll
                for (int r = 0; r < 8; ++r) col[r] = c[r][e];
                st_vec<8>(colT + (int64_t)(tx * 8 + e) * ldw + p0 + ty * 8, col);
            }
#pragma unroll
            for (int r = 0; r < 8; ++r) st_vec<8>(rowP + (int64_t)(ty * 8 + r) * ldw + p0 + tx * 8, c[r]);
            __syncthreads();
        }
        int acc[8][8];
        // 2. row panel: D[P][J] = min(D[P][J], Dg* (x) D[P][J])
        for (int tj = 0; tj < T; ++tj) {
            if (tj == pt) continue;
            const int64_t q0 = (int64_t)tj * kTile;
            load_acc<VEC>(acc, Gm, ldg, p0, q0, tx, ty);
            mainloop<kBatchedColsA>(
                acc, nslab, smem, [&](int* dst, int s) { load_kmajor_async(dst, colT, ldw, s * kSlab, p0, tid); },
                [&](int* dst, int s) { load_d_rows<VEC>(dst, Gm, ldg, p0 + s * kSlab, q0, tid); }, tx, ty, one);
            store_acc<VEC>(acc, Gm, ldg, p0, q0, tx, ty);
            store_acc_ws(acc, rowP, ldw, q0, tx, ty);
            __syncthreads();
        }
        // 3. column panel: D[I][P] = min(D[I][P], D[I][P] (x) Dg*), also into colT
        for (int ti = 0; ti < T; ++ti) {
            if (ti == pt) continue;
            const int64_t r0 = (int64_t)ti * kTile;
            load_acc<VEC>(acc, Gm, ldg, r0, p0, tx, ty);
            mainloop<kBatchedColsA>(
                acc, nslab, smem,
                [&](int* dst, int s) { load_d_transposed<VEC>(dst, Gm, ldg, r0, p0 + s * kSlab, tid); },
                [&](int* dst, int s) { load_kmajor_async(dst, rowP, ldw, s * kSlab, p0, tid); }, tx, ty, one);
            store_acc<VEC>(acc, Gm, ldg, r0, p0, tx, ty);
            store_acc_ws_transposed(acc, colT, ldw, r0, tx, ty);
            __syncthreads();
        }
        // 4. remainder
        for (int ti = 0; ti < T; ++ti) {
            if (ti == pt) continue;
            const int64_t r0 = (int64_t)ti * kTile;
            for (int tj = 0; tj < T; ++tj) {
                if (tj == pt) continue;
                const int64_t q0 = (int64_t)tj * kTile;
                load_acc<VEC>(acc, Gm, ldg, r0, q0, tx, ty);
                mainloop<kBatchedColsA>(
                    acc, nslab, smem, [&](int* dst, int s) { load_kmajor_async(dst, colT, ldw, s * kSlab, r0, tid); },
                    [&](int* dst, int s) { load_kmajor_async(dst, rowP, ldw, s * kSlab, q0, tid); }, tx, ty, one);
                store_acc<VEC>(acc, Gm, ldg, r0, q0, tx, ty);
                __syncthreads();
            }
        }
    }
}

// Large graphs in the exact packed 16-bit form (fw_batch_p16.cuh): one CTA
// per graph, persistent over items [start, start + count) (all with
// 128 < n <= kQMaxN). A graph that does not qualify is left untouched; one
// whose result the proof cannot take is restored to its input from the
// encoded copy E. Either way its item index is appended to `fallback` for
// the int32 kernel, which runs after this one.
__global__ void __launch_bounds__(kThreads, 2)
    fw_batched_p16_kernel(int* __restrict__ packed, const BatchItem* __restrict__ items, int start, int count,
                          int* __restrict__ counters, int* __restrict__ fallback, uint32_t* __restrict__ ws,
                          int64_t ws_words, int one) {
    extern __shared__ __align__(128) uint32_t qsm[];
    __shared__ int s_item;
    __shared__ QProof pf;
    uint32_t* E = ws + (int64_t)blockIdx.x * ws_words;
    const int tid = threadIdx.x;
    for (;;) {
        __syncthreads();  // the previous graph's readers of s_item and pf are done
        if (tid == 0) {
            s_item = atomicAdd(&counters[kQCounter], 1);
            pf.bad = 0;
            pf.wmax = 0;
            pf.rmax = 0;
        }
        __syncthreads();
        const int it = s_item;
        if (it >= count) break;
        const BatchItem item = items[start + it];
        const int n = item.n;
        const int ld = (n + kTile - 1) / kTile * kTile;
        int* G = packed + item.offset;
        uint32_t* S = E + q_copy_words(ld);
        q_encode(G, n, E, ld, &pf);
        __syncthreads();
        bool take = pf.bad == 0;  // G untouched otherwise
        if (take) {
            unsigned m = q_sweep(E, S, G, n, ld, qsm, one);  // writes the results into G
            for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
            if ((tid & 31) == 0 && m) atomicMax(&pf.rmax, m);
            __syncthreads();
            take = pf.rmax + pf.wmax < kQCap;
            if (!take) q_decode(E, G, n, ld);  // the proof failed: G back to the input
        }
        if (!take && tid == 0) fallback[atomicAdd(&counters[kFallbackCount], 1)] = start + it;
    }
}

__global__ void __launch_bounds__(kThreads, 2)
    fw_batched_kernel(int* __restrict__ packed, const BatchItem* __restrict__ items, BatchSched sched,
                      int* __restrict__ counters, const int* __restrict__ fallback, int* __restrict__ ws, int64_t ldw,
                      int one) {
    extern __shared__ __align__(128) int smem[];
    __shared__ int s_item[8];
    // bucket 0: whole CTA per graph, solved in place: first the graphs the
    // packed kernel (which ran before this one) handed back, then the large
    // graphs it does not take
    int* colT = ws + (int64_t)blockIdx.x * 2 * kTile * ldw;
    int* rowP = colT + (int64_t)kTile * ldw;
    const int handed_back = counters[kFallbackCount];
    for (;;) {
        if (threadIdx.x == 0) s_item[0] = atomicAdd(&counters[0], 1);
        __syncthreads();
        const int it = s_item[0];
        __syncthreads();
        if (it >= handed_back + sched.count[0]) break;
        const BatchItem item = it < handed_back ? items[fallback[it]] : items[sched.start[0] + it - handed_back];
        blocked_in_cta<false>(packed + item.offset, item.n, item.n, colT, rowP, ldw, smem, one);
    }
    small_bucket<128, 1>(packed, items, sched.start[1], sched.count[1], &counters[1], smem, s_item);
    __syncthreads();
    small_bucket_any<64>(sched.groups[2], packed, items, sched.start[2], sched.count[2], &counters[2], smem, s_item);
    __syncthreads();
    small_bucket_any<32>(sched.groups[3], packed, items, sched.start[3], sched.count[3], &counters[3], smem, s_item);
    __syncthreads();
    small_bucket_any<16>(sched.groups[4], packed, items, sched.start[4], sched.count[4], &counters[4], smem, s_item);
}

int bucket_of(int n) {
    if (n > 128) return 0;
    if (n > 64) return 1;
    if (n > 32) return 2;
    if (n > 16) return 3;
    return 4;
}

}  // namespace
}  // namespace fw

using namespace fw;

struct fw_batch_plan {
    int device = 0;
    int64_t count = 0;
    int32_t maxn = 0;
    int64_t total_elems = 0;  // one past the last element any graph uses
    double relaxations = 0;
    BatchSched sched{};
    int blocks_per_sm = 2;
    int sms = 0;
    int64_t ldw = 0;
    BatchItem* d_items = nullptr;
    int* d_counters = nullptr;
    int* d_ws = nullptr;
    int ws_ctas = 0;
    // Graphs with n > 128: items [big_start, big_start + big_count), the
    // first big_int32 of them (n > kQMaxN) always on the int32 path.
    int big_start = 0, big_count = 0, big_int32 = 0;
    bool use_p16 = false;      // the rest by the packed kernel (else all on the int32 path)
    int q_blocks_per_sm = 2;
    int64_t q_ws_words = 0;    // packed workspace words per CTA
    uint32_t* d_qws = nullptr;
    int* d_fallback = nullptr;
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    const int32_t* exec_packed = nullptr;
    std::string schedule;
};

namespace {

// Splits the n > 128 graphs between the packed and the int32 kernels.
void apply_form(fw_batch_plan* p) {
    const int q = p->big_count - p->big_int32;
    p->sched.start[0] = p->big_start;
    p->sched.count[0] = (p->use_p16 && q > 0) ? p->big_int32 : p->big_count;
}

int packed_count(const fw_batch_plan* p) { return p->use_p16 ? p->big_count - p->big_int32 : 0; }

void plan_describe(fw_batch_plan* p) {
    char buf[320];
    std::snprintf(buf, sizeof(buf),
                  "graphs=%lld maxn=%d buckets[n>128:%d (packed %d, int32 %d) n<=128:%d n<=64:%d/g%d n<=32:%d/g%d "
                  "n<=16:%d/g%d] ctas/sm=%d packed ctas/sm=%d",
                  (long long)p->count, p->maxn, p->big_count, packed_count(p), p->sched.count[0], p->sched.count[1],
                  p->sched.count[2], p->sched.groups[2], p->sched.count[3], p->sched.groups[3], p->sched.count[4],
                  p->sched.groups[4], p->blocks_per_sm, p->q_blocks_per_sm);
    p->schedule = buf;
}

void drop_graph(fw_batch_plan* p) {
    if (p->exec) cudaGraphExecDestroy(p->exec);
    p->exec = nullptr;
    p->exec_packed = nullptr;
}

int launch_direct(fw_batch_plan* p, int32_t* d_packed, cudaStream_t s) {
    FW_CUDA_TRY(cudaMemsetAsync(p->d_counters, 0, kCounters * sizeof(int), s));
    const int q = packed_count(p);
    if (q > 0) {
        fw_batched_p16_kernel<<<p->sms * p->q_blocks_per_sm, kThreads, kQSmemBytes, s>>>(
            d_packed, p->d_items, p->big_start + p->big_int32, q, p->d_counters, p->d_fallback, p->d_qws,
            p->q_ws_words, 1);
        FW_LAUNCH_CHECK("fw_batched_p16_kernel");
    }
    const int grid = p->sms * p->blocks_per_sm;
    fw_batched_kernel<<<grid, kThreads, kSmemBytes, s>>>(d_packed, p->d_items, p->sched, p->d_counters,
                                                         p->d_fallback, p->d_ws, p->ldw, 1);
    FW_LAUNCH_CHECK("fw_batched_kernel");
    return FW_OK;
}

}  // namespace

extern "C" {

int fw_batch_pack_offsets(const int32_t* h_sizes, int64_t count, int64_t* h_offsets, int64_t* total_elems) {
    if (!h_sizes || !h_offsets || count < 1) return set_error(FW_ERR_INVALID_ARGUMENT, "bad arguments");
    int64_t off = 0;
    for (int64_t g = 0; g < count; ++g) {
        if (h_sizes[g] < 1) return set_error(FW_ERR_INVALID_ARGUMENT, "graph sizes must be >= 1");
        h_offsets[g] = off;
        off += ((int64_t)h_sizes[g] * h_sizes[g] + 3) & ~int64_t(3);  // 16-byte aligned starts
    }
    if (total_elems) *total_elems = off;
    return FW_OK;
}

int fw_batch_plan_create(fw_batch_plan** out, const int32_t* h_sizes, const int64_t* h_offsets, int64_t count) {
    if (!out || !h_sizes || !h_offsets || count < 1)
        return set_error(FW_ERR_INVALID_ARGUMENT, "fw_batch_plan_create: NULL argument or count < 1");
    if (count > (int64_t)1 << 30) return set_error(FW_ERR_INVALID_ARGUMENT, "too many graphs");
    *out = nullptr;
    std::vector<BatchItem> items(count);
    int32_t maxn = 0;
    int64_t end = 0;
    double relax = 0;
    for (int64_t g = 0; g < count; ++g) {
        const int32_t n = h_sizes[g];
        if (n < 1 || n > kBatchMaxN)
            return set_error(FW_ERR_INVALID_ARGUMENT, "graph " + std::to_string(g) + ": n = " + std::to_string(n) +
                                                          " outside [1, " + std::to_string(kBatchMaxN) + "]");
        if (h_offsets[g] < 0) return set_error(FW_ERR_INVALID_ARGUMENT, "negative offset");
        items[g] = {h_offsets[g], n, (int32_t)g};
        maxn = std::max(maxn, n);
        end = std::max(end, h_offsets[g] + (int64_t)n * n);
        relax += (double)n * n * n;
    }
    // Graphs must not overlap (they are solved concurrently).
    std::vector<int64_t> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return items[a].offset < items[b].offset; });
    for (int64_t q = 1; q < count; ++q) {
        const BatchItem& a = items[order[q - 1]];
        if (a.offset + (int64_t)a.n * a.n > items[order[q]].offset)
            return set_error(FW_ERR_INVALID_ARGUMENT, "graphs " + std::to_string(a.index) + " and " +
                                                          std::to_string(items[order[q]].index) + " overlap");
    }
    std::stable_sort(items.begin(), items.end(), [](const BatchItem& a, const BatchItem& b) { return a.n > b.n; });
    auto* p = new fw_batch_plan();
    p->count = count;
    p->maxn = maxn;
    p->total_elems = end;
    p->relaxations = relax;
    for (int b = 0; b < kBuckets; ++b) {
        p->sched.start[b] = 0;
        p->sched.count[b] = 0;
        p->sched.groups[b] = 1;
    }
    int32_t maxq = 0;  // largest graph the packed path takes
    for (int64_t q = 0; q < count; ++q) {
        const int b = bucket_of(items[q].n);
        if (p->sched.count[b] == 0) p->sched.start[b] = (int)q;
        p->sched.count[b]++;
        if (b == 0 && items[q].n > kQMaxN) p->big_int32++;
        if (b == 0 && items[q].n <= kQMaxN) maxq = std::max(maxq, items[q].n);
    }
    p->big_start = p->sched.start[0];
    p->big_count = p->sched.count[0];
    p->use_p16 = p->big_count > p->big_int32;
    apply_form(p);
    // Defaults before tuning: pack small graphs 4 (n <= 64) or 8 (n <= 32) per CTA.
    p->sched.groups[2] = 4;
    p->sched.groups[3] = 8;
    p->sched.groups[4] = 8;
    int rc = FW_OK;
    do {
        if (cudaGetDevice(&p->device) != cudaSuccess) { rc = cuda_error(cudaGetLastError(), "cudaGetDevice"); break; }
        if (cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess) {
            rc = cuda_error(cudaGetLastError(), "cudaDeviceGetAttribute");
            break;
        }
        p->ldw = ((int64_t)maxn + kTile - 1) / kTile * kTile;
        p->ws_ctas = p->sms * 2;
        if (cudaFuncSetAttribute(fw_batched_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes) !=
            cudaSuccess) {
            rc = cuda_error(cudaGetLastError(), "cudaFuncSetAttribute");
            break;
        }
        if (p->big_count > p->big_int32) {
            if (cudaFuncSetAttribute(fw_batched_p16_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     kQSmemBytes) != cudaSuccess) {
                rc = cuda_error(cudaGetLastError(), "cudaFuncSetAttribute");
                break;
            }
            p->q_ws_words = q_ws_words(((int64_t)maxq + kTile - 1) / kTile * kTile);
            if (cudaMalloc(&p->d_qws, sizeof(uint32_t) * (size_t)p->q_ws_words * p->sms * 2) != cudaSuccess ||
                cudaMalloc(&p->d_fallback, sizeof(int) * (size_t)p->big_count) != cudaSuccess) {
                cudaGetLastError();
                rc = set_error(FW_ERR_NO_MEMORY, "fw_batch_plan_create: device allocation failed");
                break;
            }
        }
        if (cudaMalloc(&p->d_items, sizeof(BatchItem) * count) != cudaSuccess ||
            cudaMalloc(&p->d_counters, sizeof(int) * kCounters) != cudaSuccess ||
            cudaMalloc(&p->d_ws, sizeof(int) * (size_t)2 * kTile * p->ldw * p->ws_ctas) != cudaSuccess) {
            cudaGetLastError();
            rc = set_error(FW_ERR_NO_MEMORY, "fw_batch_plan_create: device allocation failed");
            break;
        }

        if (cudaMemcpy(p->d_items, items.data(), sizeof(BatchItem) * count, cudaMemcpyHostToDevice) != cudaSuccess) {
            rc = cuda_error(cudaGetLastError(), "cudaMemcpy(items)");
            break;
        }
        if (cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
            rc = cuda_error(cudaGetLastError(), "cudaStreamCreate");
            break;
        }
    } while (false);
    if (rc != FW_OK) {
        fw_batch_plan_destroy(p);
        return rc;
    }
    plan_describe(p);
    *out = p;
    return FW_OK;
}

void fw_batch_plan_destroy(fw_batch_plan* p) {
    if (!p) return;
    drop_graph(p);
    if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
    cudaFree(p->d_items);
    cudaFree(p->d_counters);
    cudaFree(p->d_ws);
    cudaFree(p->d_qws);
    cudaFree(p->d_fallback);
    delete p;
}

int fw_batch_plan_describe(const fw_batch_plan* p, char* buf, size_t cap, double* relaxations) {
    if (!p) return set_error(FW_ERR_INVALID_ARGUMENT, "NULL plan");
    if (buf && cap) std::snprintf(buf, cap, "%s", p->schedule.c_str());
    if (relaxations) *relaxations = p->relaxations;
    return FW_OK;
}

int fw_apsp_batched_i32(fw_batch_plan* p, int32_t* d_packed, fw_stream_t stream) {
    if (!p || !d_packed) return set_error(FW_ERR_INVALID_ARGUMENT, "fw_apsp_batched_i32: NULL plan or buffer");
    int dev = 0;
    FW_CUDA_TRY(cudaGetDevice(&dev));
    if (dev != p->device)
        return set_error(FW_ERR_INVALID_ARGUMENT, "fw_apsp_batched_i32: the plan was created on device " +
                                                      std::to_string(p->device) + ", the current device is " +
                                                      std::to_string(dev));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (p->exec == nullptr || p->exec_packed != d_packed) {
        drop_graph(p);
        cudaGraph_t graph = nullptr;
        FW_CUDA_TRY(cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal));
        int rc = launch_direct(p, d_packed, p->cap_stream);
        cudaError_t e = cudaStreamEndCapture(p->cap_stream, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return cuda_error(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&p->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            p->exec = nullptr;
            return cuda_error(e, "cudaGraphInstantiate");
        }
        p->exec_packed = d_packed;
    }
    prof_begin(KC_BATCHED, s);
    FW_CUDA_TRY(cudaGraphLaunch(p->exec, s));
    prof_end(KC_BATCHED, s, p->relaxations);
    return FW_OK;
}

// Times the candidate schedules on a scratch copy of the batch and keeps the
// fastest: the arithmetic form of the graphs with n > 128 (exact packed
// 16-bit with its CTAs per SM, or int32), per small bucket the number of
// graphs per CTA, then the number of resident CTAs per SM of the int32 kernel
// for the whole batch. Synchronises the stream.
int fw_batch_plan_autotune(fw_batch_plan* p, const int32_t* d_packed, fw_stream_t stream) {
    if (!p || !d_packed) return set_error(FW_ERR_INVALID_ARGUMENT, "fw_batch_plan_autotune: NULL argument");
    int dev = 0;
    FW_CUDA_TRY(cudaGetDevice(&dev));
    if (dev != p->device)
        return set_error(FW_ERR_INVALID_ARGUMENT, "fw_batch_plan_autotune: the plan was created on device " +
                                                      std::to_string(p->device) + ", the current device is " +
                                                      std::to_string(dev));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int32_t* scratch = nullptr;
    const size_t bytes = sizeof(int32_t) * (size_t)p->total_elems;
    if (cudaMalloc(&scratch, bytes) != cudaSuccess) {
        cudaGetLastError();
        return set_error(FW_ERR_NO_MEMORY, "fw_batch_plan_autotune: scratch copy allocation failed");
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const BatchSched full = p->sched;  // groups of the small buckets and their counts
    auto time_once = [&](float* ms) -> int {
        FW_CUDA_TRY(cudaMemcpyAsync(scratch, d_packed, bytes, cudaMemcpyDeviceToDevice, s));
        FW_CUDA_TRY(cudaEventRecord(e0, s));
        if (int rc = launch_direct(p, scratch, s)) return rc;
        FW_CUDA_TRY(cudaEventRecord(e1, s));
        FW_CUDA_TRY(cudaEventSynchronize(e1));
        FW_CUDA_TRY(cudaEventElapsedTime(ms, e0, e1));
        return FW_OK;
    };
    auto best_of = [&](float* out) -> int {  // one warm-up run, best of two timed runs
        float best = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
            float ms = 0;
            if (int rc = time_once(&ms)) return rc;
            if (rep > 0) best = std::min(best, ms);
        }
        *out = best;
        return FW_OK;
    };
    int rc = FW_OK;
    auto set_counts = [&](bool big, bool small) {
        for (int q = 1; q < kBuckets; ++q) p->sched.count[q] = small ? full.count[q] : 0;
        apply_form(p);
        if (!big) {
            p->sched.count[0] = 0;
            p->use_p16 = false;
        }
    };
    // 1. Graphs with n > 128 alone: the packed kernel (1 or 2 CTAs per SM,
    //    int32 for the graphs it hands back or cannot take) against the int32
    //    kernel for all of them.
    if (p->big_count > p->big_int32) {
        float best = 1e30f;
        bool form = true;
        int qbps = p->q_blocks_per_sm;
        for (int trial = 0; trial < 3 && rc == FW_OK; ++trial) {
            p->use_p16 = trial < 2;
            p->q_blocks_per_sm = trial == 1 ? 1 : 2;
            set_counts(true, false);
            float ms = 0;
            rc = best_of(&ms);
            if (rc == FW_OK && ms < best) {
                best = ms;
                form = p->use_p16;
                qbps = p->q_blocks_per_sm;
            }
        }
        p->use_p16 = form;
        p->q_blocks_per_sm = qbps;
    }
    const bool form = p->use_p16;
    // 2. Each small bucket alone: graphs per CTA.
    const int options[kBuckets][3] = {{1, 1, 1}, {1, 1, 1}, {1, 4, 4}, {1, 4, 8}, {1, 4, 8}};
    for (int b = 2; b < kBuckets && rc == FW_OK; ++b) {
        if (full.count[b] == 0) continue;
        set_counts(false, false);
        p->sched.count[b] = full.count[b];
        float best = 1e30f;
        int choice = full.groups[b];
        for (int o = 0; o < 3 && rc == FW_OK; ++o) {
            if (o > 0 && options[b][o] == options[b][o - 1]) continue;
            p->sched.groups[b] = options[b][o];
            float ms = 0;
            rc = best_of(&ms);
            if (rc == FW_OK && ms < best) {
                best = ms;
                choice = options[b][o];
            }
        }
        p->sched.groups[b] = choice;
    }
    p->use_p16 = form;
    set_counts(true, true);
    // 3. The whole batch: resident CTAs per SM of the int32 kernel.
    if (rc == FW_OK) {
        float best = 1e30f;
        int choice = p->blocks_per_sm;
        for (int bps = 1; bps <= 2 && rc == FW_OK; ++bps) {
            p->blocks_per_sm = bps;
            float ms = 0;
            rc = best_of(&ms);
            if (rc == FW_OK && ms < best) {
                best = ms;
                choice = bps;
            }
        }
        p->blocks_per_sm = choice;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(scratch);
    drop_graph(p);  // the captured launch used the old schedule
    plan_describe(p);
    return rc;
}

}  // extern "C"

// Tile loaders, stores and the pipelined min-plus main loop shared by the
// blocked kernels (one graph: fw_apsp_i32.cu; many graphs: fw_batched.cu).
#pragma once

#include "fw_common.cuh"

namespace fw {

// Slab [k0, k0 + 32) x [c0, c0 + 128) of a k-major workspace buffer.
__device__ __forceinline__ void load_kmajor_async(int* dst, const int* __restrict__ buf, int64_t ldp, int k0,
                                                  int64_t c0, int tid) {
#pragma unroll
    for (int q = tid; q < kSlab * 32; q += kThreads) {
        const int row = q >> 5, ch = q & 31;
        cp_async16(dst + row * kTile + ch * 4, buf + (int64_t)(k0 + row) * ldp + c0 + ch * 4);
    }
}

// Slab of D, rows [r0, r0 + 32), columns [c0, c0 + 128), INF outside the
// matrix; row-major, which is k-major when the rows are pivots.
template <bool VEC>
__device__ __forceinline__ void load_d_rows(int* dst, const int* __restrict__ D, int64_t n, int64_t r0, int64_t c0,
                                            int tid) {
#pragma unroll
    for (int q = tid; q < kSlab * 32; q += kThreads) {
        const int row = q >> 5, ch = q & 31;
        const int64_t gr = r0 + row, gc = c0 + ch * 4;
        int* d = dst + row * kTile + ch * 4;
        if (VEC) {
            if (gr < n && gc < n) {
                cp_async16(d, D + gr * n + gc);
            } else {
                *reinterpret_cast<int4*>(d) = make_int4(kInf, kInf, kInf, kInf);
            }
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) d[e] = (gr < n && gc + e < n) ? D[gr * n + gc + e] : kInf;
        }
    }
}

// Transposed slab of D: dst[kk][i] = D[r0 + i][k0 + kk], INF outside.
template <bool VEC>
__device__ __forceinline__ void load_d_transposed(int* dst, const int* __restrict__ D, int64_t n, int64_t r0,
                                                  int64_t k0, int tid) {
#pragma unroll
    for (int q = tid; q < kTile * 8; q += kThreads) {
        const int i = q >> 3, ch = q & 7;
        const int64_t gr = r0 + i, gc = k0 + ch * 4;
        int v[4];
        if (VEC && gr < n && gc < n) {
            const int4 t = *reinterpret_cast<const int4*>(D + gr * n + gc);
            v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) v[e] = (gr < n && gc + e < n) ? D[gr * n + gc + e] : kInf;
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) dst[(ch * 4 + e) * kTile + i] = v[e];
    }
}

// The thread's 8 x 8 micro-tile of the 128 x 128 tile at (r0, c0) of D.
template <bool VEC>
__device__ __forceinline__ void load_acc(int (&acc)[8][8], const int* __restrict__ D, int64_t n, int64_t r0,
                                         int64_t c0, int tx, int ty) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int64_t gr = r0 + own_row(ty, r);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int64_t gc = c0 + h * 64 + tx * 4;
            if (VEC) {
                int4 t = make_int4(kInf, kInf, kInf, kInf);
                if (gr < n && gc < n) t = *reinterpret_cast<const int4*>(D + gr * n + gc);
                acc[r][h * 4 + 0] = t.x; acc[r][h * 4 + 1] = t.y;
                acc[r][h * 4 + 2] = t.z; acc[r][h * 4 + 3] = t.w;
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    acc[r][h * 4 + e] = (gr < n && gc + e < n) ? D[gr * n + gc + e] : kInf;
            }
        }
    }
}

template <bool VEC>
__device__ __forceinline__ void store_acc(const int (&acc)[8][8], int* __restrict__ D, int64_t n, int64_t r0,
                                          int64_t c0, int tx, int ty) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int64_t gr = r0 + own_row(ty, r);
        if (gr >= n) continue;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int64_t gc = c0 + h * 64 + tx * 4;
            if (VEC) {
                if (gc < n)
                    *reinterpret_cast<int4*>(D + gr * n + gc) =
                        make_int4(acc[r][h * 4 + 0], acc[r][h * 4 + 1], acc[r][h * 4 + 2], acc[r][h * 4 + 3]);
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (gc + e < n) D[gr * n + gc + e] = acc[r][h * 4 + e];
            }
        }
    }
}

// Row-major store of the micro-tile into a k-major workspace (no masking:
// the workspace covers the padded extent).
__device__ __forceinline__ void store_acc_ws(const int (&acc)[8][8], int* __restrict__ buf, int64_t ldp, int64_t c0,
                                             int tx, int ty) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int64_t row = own_row(ty, r);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            *reinterpret_cast<int4*>(buf + row * ldp + c0 + h * 64 + tx * 4) =
                make_int4(acc[r][h * 4 + 0], acc[r][h * 4 + 1], acc[r][h * 4 + 2], acc[r][h * 4 + 3]);
        }
    }
}

// Transposed store: buf[c][r0 + r] = acc[r][c].
__device__ __forceinline__ void store_acc_ws_transposed(const int (&acc)[8][8], int* __restrict__ buf, int64_t ldp,
                                                        int64_t r0, int tx, int ty) {
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int64_t col = own_col(tx, c);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            *reinterpret_cast<int4*>(buf + col * ldp + r0 + h * 64 + ty * 4) =
                make_int4(acc[h * 4 + 0][c], acc[h * 4 + 1][c], acc[h * 4 + 2][c], acc[h * 4 + 3][c]);
        }
    }
}

// Multi-stage cp.async pipeline over `nslab` operand slabs: acc = min(acc, A (x) B).
// (The panel kernels and the batched kernel use it; the remainder kernels
// stream their slabs by TMA instead.)
// la(dst, s) / lb(dst, s) fill slab s of A / B (asynchronously or not).
template <unsigned COLS, class LA, class LB>
__device__ __forceinline__ void mainloop(int (&acc)[8][8], int nslab, int* smem, LA la, LB lb, int tx, int ty,
                                         int one) {
#pragma unroll
    for (int s = 0; s < kStages - 1; ++s) {
        if (s < nslab) {
            la(smem + s * kStageInts, s);
            lb(smem + s * kStageInts + kSlabInts, s);
        }
        cp_async_commit();
    }
    for (int kb = 0; kb < nslab; ++kb) {
        cp_async_wait<kStages - 2>();
        __syncthreads();
        const int nxt = kb + kStages - 1;
        if (nxt < nslab) {
            int* st = smem + (nxt % kStages) * kStageInts;
            la(st, nxt);
            lb(st + kSlabInts, nxt);
        }
        cp_async_commit();
        const int* st = smem + (kb % kStages) * kStageInts;
        relax_slab<COLS>(acc, st, st + kSlabInts, tx, ty, one);
    }
}

}  // namespace fw

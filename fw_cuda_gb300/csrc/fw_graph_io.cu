// Graph input front-end and result checks on the device. No counterpart in
// the reference, which generates dense matrices on the host
// (src/graph_generator.cpp:7-46) and checks negative cycles on the host
// (src/utils.cpp:5-12).
//
//   fw_dense_from_csr_i32   CSR adjacency (row pointers, column indices,
//                           int32 weights) -> dense n x n int32 matrix in the
//                           reference's convention: INF for a missing edge, 0
//                           on the diagonal, the smallest weight of duplicate
//                           edges (a negative self-loop makes the diagonal
//                           negative, as in the sweep).
//   fw_negative_cycle_i32   per graph of a batch, 1 if some D[i][i] < 0 after
//                           the sweep (the reference's hasNegativeCycle).
#include <cuda_runtime.h>

#include <string>

#include "fw_common.cuh"
#include "fw_internal.h"

namespace fw {
namespace {

// Rows strided over blockIdx.y, columns over the x dimension.
__global__ void fw_fill_dense_kernel(int* __restrict__ D, int64_t n) {
    for (int64_t i = blockIdx.y; i < n; i += gridDim.y) {
        int* row = D + i * n;
        for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
            row[j] = (i == j) ? 0 : kInf;
    }
}

// One warp per row: scatter the row's edges with atomicMin (duplicates keep
// the smallest weight). Column indices outside [0, n) and weights >= INF are
// skipped and counted in *bad.
__global__ void fw_scatter_csr_kernel(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                      const int32_t* __restrict__ w, int64_t n, int* __restrict__ D,
                                      unsigned* __restrict__ bad) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    unsigned nbad = 0;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        const int64_t b = rowptr[i], e = rowptr[i + 1];
        for (int64_t q = b + lane; q < e; q += 32) {
            const int64_t j = col[q];
            const int v = w[q];
            if (j < 0 || j >= n || v >= kInf) {
                ++nbad;
                continue;
            }
            atomicMin(&D[i * n + j], v);
        }
    }
    if (bad && nbad) atomicAdd(bad, nbad);
}

__global__ void fw_negative_cycle_kernel(const int* __restrict__ D, int64_t n, int* __restrict__ flags) {
    const int* G = D + (int64_t)blockIdx.x * n * n;
    int neg = 0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) neg |= (G[i * n + i] < 0);
    neg = __syncthreads_or(neg);
    if (threadIdx.x == 0) flags[blockIdx.x] = neg ? 1 : 0;
}

}  // namespace
}  // namespace fw

using namespace fw;

extern "C" {

int fw_dense_from_csr_i32(const int64_t* d_rowptr, const int32_t* d_col, const int32_t* d_w, int64_t n,
                          int32_t* d_D, uint32_t* d_bad, fw_stream_t stream) {
    if (!d_rowptr || !d_D || n < 1) return set_error(FW_ERR_INVALID_ARGUMENT, "fw_dense_from_csr_i32: bad arguments");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const unsigned gx = (unsigned)((n + 255) / 256 < 64 ? (n + 255) / 256 : 64);
    const unsigned gy = (unsigned)(n < 65535 ? n : 65535);
    fw_fill_dense_kernel<<<dim3(gx, gy), 256, 0, s>>>(d_D, n);
    FW_LAUNCH_CHECK("fw_fill_dense_kernel");
    if (d_col && d_w) {
        const int64_t warps = n < 65536 ? n : 65536;
        fw_scatter_csr_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(d_rowptr, d_col, d_w, n, d_D, d_bad);
        FW_LAUNCH_CHECK("fw_scatter_csr_kernel");
    }
    return FW_OK;
}

int fw_negative_cycle_i32(const int32_t* d_D, int64_t n, int64_t batch, int32_t* d_flags, fw_stream_t stream) {
    if (!d_D || !d_flags || n < 1 || batch < 1 || batch > 2147483647)
        return set_error(FW_ERR_INVALID_ARGUMENT, "fw_negative_cycle_i32: bad arguments");
    fw_negative_cycle_kernel<<<(unsigned)batch, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(d_D, n, d_flags);
    FW_LAUNCH_CHECK("fw_negative_cycle_kernel");
    return FW_OK;
}

}  // extern "C"

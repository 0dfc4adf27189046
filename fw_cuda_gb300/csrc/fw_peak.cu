// Register-only relaxation-rate kernels: the integer issue ceiling that the
// blocked sweep's roofline fraction is quoted against.
//
// Each thread keeps 16 accumulators and folds pivot pairs into them exactly
// as the remainder kernel does (fw_common.cuh relax2), with operands taken
// from other accumulators so that nothing can be hoisted out of the loop. No
// memory is touched inside the timed loop.
#include <cuda_runtime.h>

#include "fw_common.cuh"
#include "fw_internal.h"

namespace fw {
namespace {

constexpr int kPeakIters = 4096;

template <int MIXA>
__global__ void __launch_bounds__(256) fw_peak_kernel(const int* __restrict__ in, int* __restrict__ out, int iters,
                                                      int one) {
    // Two rows of the 8-column micro-tile: 16 accumulators, columns below
    // MIXA in form A exactly as in the remainder kernel.
    int acc[2][8];
    int a0[2], a1[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        a0[r] = in[(threadIdx.x + r) & 255];
        a1[r] = in[256 + ((threadIdx.x + r) & 255)];
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[r][c] = in[512 + ((threadIdx.x + 8 * r + c) & 255)];
    }
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int r = 0; r < 2; ++r) {
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const int b0 = acc[r ^ 1][c];
                const int b1 = acc[r][(c + 1) & 7];
                acc[r][c] = relax2(c < MIXA, acc[r][c], a0[r], b0, a1[r], b1, one);
            }
        }
    }
    int s = 0;
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 8; ++c) s ^= acc[r][c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Packed 16-bit relaxations: 16 accumulator words of two 15-bit lanes each
// fold pivot pairs exactly as the packed remainder kernel does (word columns
// below MIXW: two packed DPX add-mins; the others: two adds on the FMA pipe and
// one packed three-way DPX min), operands from other accumulators.
template <int MIXW>
__global__ void __launch_bounds__(256) fw_peak_packed_kernel(const unsigned* __restrict__ in,
                                                             unsigned* __restrict__ out, int iters, int one) {
    unsigned acc[2][8], a0[2], a1[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        a0[r] = in[(threadIdx.x + r) & 255] & 0x3FFF3FFFu;
        a1[r] = in[256 + ((threadIdx.x + r) & 255)] & 0x3FFF3FFFu;
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[r][c] = in[512 + ((threadIdx.x + 8 * r + c) & 255)] & 0x3FFF3FFFu;
    }
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int r = 0; r < 2; ++r) {
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const unsigned b0 = acc[r ^ 1][c];
                const unsigned b1 = acc[r][(c + 1) & 7];
                if (c < MIXW) {
                    acc[r][c] = __viaddmin_u16x2(a1[r], b1, __viaddmin_u16x2(a0[r], b0, acc[r][c]));
                } else {
                    // lanes stay below 2^15, so the 32-bit sums carry nothing across lanes
                    const unsigned s0 = (unsigned)add_on_fma((int)a0[r], (int)b0, one);
                    const unsigned s1 = (unsigned)add_on_fma((int)a1[r], (int)b1, one);
                    acc[r][c] = __vimin3_u16x2(acc[r][c], s0, s1);
                }
            }
        }
    }
    unsigned s = 0;
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 8; ++c) s ^= acc[r][c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Instruction-class probes of the int32 relaxation ceiling: each thread keeps
// 16 independent accumulators and updates every one of them per iteration
// with operands taken from other accumulators (nothing can be hoisted). OP:
//   0 DPX add-min            acc = min(x + o, acc)            (1 relaxation)
//   1 integer multiply-add   acc = o * one + acc
//   2 DPX three-way min      acc = min(acc, o, p)
//   3 add                    acc = acc + o
//   4 min                    acc = min(acc, o)
//   5 add-min and multiply-add alternating over the accumulators
//   6 form B (two multiply-adds + one three-way min: 2 relaxations)
//   7 form A (two DPX add-mins: 2 relaxations)
//   8 three relaxations: form B, then one DPX add-min
template <int OP>
__global__ void __launch_bounds__(256) fw_rate_kernel(const int* __restrict__ in, int* __restrict__ out, int iters,
                                                      int one) {
    int acc[16], x[4];
#pragma unroll
    for (int i = 0; i < 16; ++i) acc[i] = in[(threadIdx.x + i) & 255];
#pragma unroll
    for (int i = 0; i < 4; ++i) x[i] = in[256 + ((threadIdx.x + i) & 255)];
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int o = acc[(i + 5) & 15];
            const int p = acc[(i + 11) & 15];
            if (OP == 0) acc[i] = __viaddmin_s32(x[i & 3], o, acc[i]);
            if (OP == 1) acc[i] = add_on_fma(o, acc[i], one);
            if (OP == 2) acc[i] = __vimin3_s32(acc[i], o, p);
            if (OP == 3) acc[i] = acc[i] + o;
            if (OP == 4) acc[i] = min(acc[i], o);
            if (OP == 5) acc[i] = (i & 1) ? add_on_fma(o, acc[i], one) : __viaddmin_s32(x[i & 3], o, acc[i]);
            if (OP == 6) acc[i] = relax2(false, acc[i], x[i & 3], o, x[(i + 1) & 3], p, one);
            if (OP == 7) acc[i] = relax2(true, acc[i], x[i & 3], o, x[(i + 1) & 3], p, one);
            if (OP == 8) acc[i] = __viaddmin_s32(x[(i + 2) & 3], acc[(i + 3) & 15],
                                                 relax2(false, acc[i], x[i & 3], o, x[(i + 1) & 3], p, one));
        }
    }
    int s = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) s ^= acc[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Best of five timed launches (after one warm-up) of fw_rate_kernel<OP>;
// *rate = `per_thread_iter` units per thread-iteration / second.
template <int OP>
int time_rate(int blocks, const int* in, int* out, cudaStream_t s, double per_thread_iter, double* rate) {
    constexpr int kIters = 2048;
    cudaEvent_t e0, e1;
    FW_CUDA_TRY(cudaEventCreate(&e0));
    FW_CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 6; ++rep) {
        cudaEventRecord(e0, s);
        fw_rate_kernel<OP><<<blocks, 256, 0, s>>>(in, out, kIters, 1);
        cudaEventRecord(e1, s);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return cuda_error(e, "fw_rate_kernel");
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *rate = (double)blocks * 256.0 * kIters * per_thread_iter / (best * 1e-3);
    return FW_OK;
}

template <int MIXA>
int time_peak(int blocks, const int* in, int* out, cudaStream_t s, double* rate) {
    cudaEvent_t e0, e1;
    FW_CUDA_TRY(cudaEventCreate(&e0));
    FW_CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(e0, s);
        fw_peak_kernel<MIXA><<<blocks, 256, 0, s>>>(in, out, kPeakIters, 1);
        cudaEventRecord(e1, s);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return cuda_error(e, "fw_peak_kernel");
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;  // rep 0 warms up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // 16 accumulators x 2 relaxations per iteration.
    *rate = (double)blocks * 256.0 * kPeakIters * 32.0 / (best * 1e-3);
    return FW_OK;
}

template <int MIXW>
int time_peak_packed(int blocks, const unsigned* in, unsigned* out, cudaStream_t s, double* rate) {
    cudaEvent_t e0, e1;
    FW_CUDA_TRY(cudaEventCreate(&e0));
    FW_CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(e0, s);
        fw_peak_packed_kernel<MIXW><<<blocks, 256, 0, s>>>(in, out, kPeakIters, 1);
        cudaEventRecord(e1, s);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return cuda_error(e, "fw_peak_packed_kernel");
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;  // rep 0 warms up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // 16 accumulator words x 2 pivots x 2 lanes per iteration.
    *rate = (double)blocks * 256.0 * kPeakIters * 64.0 / (best * 1e-3);
    return FW_OK;
}

}  // namespace

int measure_relax_peak_packed(double* dpx_only, double* mixed, cudaStream_t s) {
    int dev = 0, sms = 0;
    FW_CUDA_TRY(cudaGetDevice(&dev));
    FW_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8;
    unsigned *in = nullptr, *out = nullptr;
    FW_CUDA_TRY(cudaMallocAsync(&in, 768 * sizeof(unsigned), s));
    FW_CUDA_TRY(cudaMallocAsync(&out, (size_t)blocks * 256 * sizeof(unsigned), s));
    FW_CUDA_TRY(cudaMemsetAsync(in, 0, 768 * sizeof(unsigned), s));
    // MIXW = 8: every word column as two packed DPX add-mins; the others: the
    // packed remainder's count of DPX word columns (four) and its neighbours.
    double r8 = 0, r6 = 0, r5 = 0, r4 = 0, r3 = 0;
    int rc = time_peak_packed<8>(blocks, in, out, s, &r8);
    if (!rc) rc = time_peak_packed<6>(blocks, in, out, s, &r6);
    if (!rc) rc = time_peak_packed<5>(blocks, in, out, s, &r5);
    if (!rc) rc = time_peak_packed<4>(blocks, in, out, s, &r4);
    if (!rc) rc = time_peak_packed<3>(blocks, in, out, s, &r3);
    cudaFreeAsync(in, s);
    cudaFreeAsync(out, s);
    if (rc) return rc;
    if (dpx_only) *dpx_only = r8;
    double best = r8;
    for (double r : {r6, r5, r4, r3}) best = r > best ? r : best;
    if (mixed) *mixed = best;
    return FW_OK;
}

int measure_int32_rates(double* rates, int count, cudaStream_t s) {
    int dev = 0, sms = 0;
    FW_CUDA_TRY(cudaGetDevice(&dev));
    FW_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8;
    int *in = nullptr, *out = nullptr;
    FW_CUDA_TRY(cudaMallocAsync(&in, 1024 * sizeof(int), s));
    FW_CUDA_TRY(cudaMallocAsync(&out, (size_t)blocks * 256 * sizeof(int), s));
    FW_CUDA_TRY(cudaMemsetAsync(in, 0, 1024 * sizeof(int), s));
    double r[kInt32RateCount] = {};
    // instruction classes: lane operations per second (16 per thread-iteration)
    int rc = time_rate<0>(blocks, in, out, s, 16, &r[0]);
    if (!rc) rc = time_rate<1>(blocks, in, out, s, 16, &r[1]);
    if (!rc) rc = time_rate<2>(blocks, in, out, s, 16, &r[2]);
    if (!rc) rc = time_rate<3>(blocks, in, out, s, 16, &r[3]);
    if (!rc) rc = time_rate<4>(blocks, in, out, s, 16, &r[4]);
    if (!rc) rc = time_rate<5>(blocks, in, out, s, 16, &r[5]);
    // relaxation forms: relaxations per second
    if (!rc) rc = time_rate<6>(blocks, in, out, s, 32, &r[6]);
    if (!rc) rc = time_rate<7>(blocks, in, out, s, 32, &r[7]);
    if (!rc) rc = time_rate<8>(blocks, in, out, s, 48, &r[8]);
    cudaFreeAsync(in, s);
    cudaFreeAsync(out, s);
    if (rc) return rc;
    for (int i = 0; i < count && i < kInt32RateCount; ++i) rates[i] = r[i];
    return FW_OK;
}

int measure_relax_peak(double* dpx_only, double* mixed, cudaStream_t s) {
    int dev = 0, sms = 0;
    FW_CUDA_TRY(cudaGetDevice(&dev));
    FW_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8;
    int *in = nullptr, *out = nullptr;
    FW_CUDA_TRY(cudaMallocAsync(&in, 768 * sizeof(int), s));
    FW_CUDA_TRY(cudaMallocAsync(&out, (size_t)blocks * 256 * sizeof(int), s));
    FW_CUDA_TRY(cudaMemsetAsync(in, 0, 768 * sizeof(int), s));
    // MIXA = 8: every pair as two DPX add-mins. The others: the remainder's
    // mix (kMixA) and its neighbours; the best of all is the ceiling.
    double r8 = 0, r2 = 0, r3 = 0, r4 = 0, r5 = 0;
    int rc = time_peak<8>(blocks, in, out, s, &r8);
    if (!rc) rc = time_peak<2>(blocks, in, out, s, &r2);
    if (!rc) rc = time_peak<3>(blocks, in, out, s, &r3);
    if (!rc) rc = time_peak<4>(blocks, in, out, s, &r4);
    if (!rc) rc = time_peak<5>(blocks, in, out, s, &r5);
    cudaFreeAsync(in, s);
    cudaFreeAsync(out, s);
    if (rc) return rc;
    if (dpx_only) *dpx_only = r8;
    double best = r2 > r3 ? r2 : r3;
    best = best > r4 ? best : r4;
    best = best > r5 ? best : r5;
    best = best > r8 ? best : r8;
    if (mixed) *mixed = best;
    return FW_OK;
}

}  // namespace fw

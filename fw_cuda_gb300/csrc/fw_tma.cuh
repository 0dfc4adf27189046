// Tensor-memory-accelerator helpers shared by the remainder kernels: mbarrier
// setup and bounded waits, 2-D tiled bulk tensor loads, and host-side tensor
// map encoding for the k-major panel buffers.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "fw_common.cuh"
#include "fw_internal.h"

namespace fw {

// Spins of mbarrier.try_wait (each may itself suspend for a while) before a
// wait gives up and the kernel records a copy fault instead of hanging.
constexpr int kMbarSpins = 1 << 20;

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes initialised barriers visible to the async (TMA) proxy; call from the
// initialising thread, then synchronise the CTA.
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// true once the phase with this parity has completed; false after `spins`
// unsuccessful tries.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int spins = kMbarSpins) {
    const uint32_t addr = smem_u32(bar);
    for (int i = 0; i < spins; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(addr), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// One slab wait of a copy ring, agreed by the whole CTA: true only when the
// slab's copy arrived for every thread (one thread whose bounded wait gave up
// makes it false for all). It is also the CTA barrier after which the stage
// of the previous slab may be refilled.
__device__ __forceinline__ bool ring_wait_all(uint64_t* bar, uint32_t parity) {
    const bool got = mbar_wait(bar, parity);
    return __syncthreads_or(got ? 0 : 1) == 0;
}

// After a missed slab: bounded waits for every copy already issued into the
// ring (running slab counts first .. last, stage j % stages, phase j / stages),
// so that no copy is still writing the CTA's shared memory when it stops
// using the ring. Copies that still do not arrive cannot be waited for longer.
__device__ __forceinline__ void ring_drain(uint64_t* bars, int stages, int first, int last) {
    for (int j = first; j <= last; ++j) mbar_wait(&bars[j % stages], (uint32_t)((j / stages) & 1));
}

// A missed copy: one more in the process-lifetime counter of the translation
// unit and, when the call has one, in the call's own status word.
__device__ __forceinline__ void count_copy_fault(unsigned int* process_total, unsigned int* call_word) {
    atomicAdd(process_total, 1u);
    if (call_word) atomicAdd(call_word, 1u);
}

// Box (x, y) of the 2-D map into shared memory (128-byte aligned), completing
// `bar` with its byte count. x * element size must be a multiple of 16.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// 3-D form: box (x, y, z).
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library does not link libcuda itself).
inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// 2-D map over a k-major panel of `rows` rows of `width` 32-bit elements
// (16-byte aligned base, row stride width * 4 bytes, a multiple of 16), in
// boxes of box_w x kSlab.
inline int panel_map(CUtensorMap* map, const void* base, uint64_t width, uint64_t rows, uint32_t box_w) {
    const auto fn = tensor_map_encoder();
    if (!fn) return set_error(FW_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    if ((reinterpret_cast<uintptr_t>(base) & 15u) != 0 || (width * 4) % 16 != 0)
        return set_error(FW_ERR_INTERNAL, "panel_map: base or row stride not 16-byte aligned");
    const cuuint64_t dims[2] = {width, rows};
    const cuuint64_t strides[1] = {width * 4};
    const cuuint32_t box[2] = {box_w, (cuuint32_t)kSlab};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<void*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(FW_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    return FW_OK;
}

// 2-D map over `rows` rows of `width` 32-bit elements with leading dimension
// ld (elements; ld * 4 a multiple of 16), in boxes of box_w x kSlab.
inline int panel_map_ld(CUtensorMap* map, const void* base, uint64_t width, uint64_t ld, uint64_t rows,
                        uint32_t box_w) {
    const auto fn = tensor_map_encoder();
    if (!fn) return set_error(FW_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    if ((reinterpret_cast<uintptr_t>(base) & 15u) != 0 || (ld * 4) % 16 != 0 || width > ld)
        return set_error(FW_ERR_INTERNAL, "panel_map_ld: base, leading dimension or width not valid");
    const cuuint64_t dims[2] = {width, rows};
    const cuuint64_t strides[1] = {ld * 4};
    const cuuint32_t box[2] = {box_w, (cuuint32_t)kSlab};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<void*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(FW_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    return FW_OK;
}

// 3-D map over `depth` k-major panels of `rows` x `width` 32-bit elements
// stored one after another, in boxes of box_w x kSlab x 1.
inline int panel_map_3d(CUtensorMap* map, const void* base, uint64_t width, uint64_t rows, uint64_t depth,
                        uint32_t box_w) {
    const auto fn = tensor_map_encoder();
    if (!fn) return set_error(FW_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    if ((reinterpret_cast<uintptr_t>(base) & 15u) != 0 || (width * 4) % 16 != 0)
        return set_error(FW_ERR_INTERNAL, "panel_map_3d: base or row stride not 16-byte aligned");
    const cuuint64_t dims[3] = {width, rows, depth};
    const cuuint64_t strides[2] = {width * 4, width * rows * 4};
    const cuuint32_t box[3] = {box_w, (cuuint32_t)kSlab, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, const_cast<void*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(FW_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    return FW_OK;
}

}  // namespace fw

// Second oracle and speed comparator: the reference's own GPU kernels.
//
// TEST INFRASTRUCTURE ONLY. oracle/Makefile compiles the reference's three
// GPU sources (src/fw_baseline_gpu.cu, src/fw_tiling_gpu.cu,
// src/fw_multi_layer_tiling_gpu.cu), device code only, into cubins for
// sm_103a under oracle/_ref/. This file loads those cubins through the CUDA
// driver API and replays the reference's host launch loops unchanged:
//   baseline_gpu            src/fw_baseline_gpu.cu:16-32
//   tiling_gpu              src/fw_tiling_gpu.cu:253-284
//   multi_layer_tiling_gpu  src/fw_multi_layer_tiling_gpu.cu:507-577
// (16x16 thread blocks, TILE = 32, the same grids and dynamic shared memory,
// the legacy default stream, one device-wide synchronisation at the end).
// The shipped library never loads it; tests use it for parity on the GPU and
// the benchmark's reference arm uses it to time the reference kernels.
#include <cuda.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <string>

namespace {

struct RefKernels {
    bool loaded = false;
    CUmodule mod_base = nullptr, mod_tile = nullptr, mod_ml = nullptr;
    CUfunction base = nullptr;
    CUfunction t_diag = nullptr, t_row = nullptr, t_col = nullptr, t_oth = nullptr;
    CUfunction ml_lead = nullptr, ml_row = nullptr, ml_col = nullptr;
    CUfunction ml_row_rev = nullptr, ml_col_rev = nullptr, ml_rest = nullptr;
};

RefKernels g_ref;
char g_err[512] = "";

int fail(const char* what, CUresult r) {
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    std::snprintf(g_err, sizeof(g_err), "%s: %s", what, s ? s : "unknown");
    return static_cast<int>(r) ? static_cast<int>(r) : 1;
}

#define REF_CHECK(call)                                  \
    do {                                                 \
        CUresult _r = (call);                            \
        if (_r != CUDA_SUCCESS) return fail(#call, _r);  \
    } while (0)

int launch(CUfunction f, unsigned gx, unsigned gy, unsigned smem, void** args) {
    REF_CHECK(cuLaunchKernel(f, gx, gy, 1, 16, 16, 1, smem, nullptr, args, nullptr));
    return 0;
}

}  // namespace

extern "C" {

const char* refgpu_last_error(void) { return g_err; }

// Loads the three cubins from `dir` (oracle/_ref). Returns 0 on success.
int refgpu_load(const char* dir) {
    if (g_ref.loaded) return 0;
    REF_CHECK(cuInit(0));
    CUdevice dev;
    REF_CHECK(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    REF_CHECK(cuDevicePrimaryCtxRetain(&ctx, dev));
    REF_CHECK(cuCtxSetCurrent(ctx));
    const std::string d(dir);
    REF_CHECK(cuModuleLoad(&g_ref.mod_base, (d + "/ref_fw_baseline_gpu.cubin").c_str()));
    REF_CHECK(cuModuleLoad(&g_ref.mod_tile, (d + "/ref_fw_tiling_gpu.cubin").c_str()));
    REF_CHECK(cuModuleLoad(&g_ref.mod_ml, (d + "/ref_fw_multi_layer_tiling_gpu.cubin").c_str()));
    REF_CHECK(cuModuleGetFunction(&g_ref.base, g_ref.mod_base, "_Z16fwBaselineKernelPiii"));
    REF_CHECK(cuModuleGetFunction(&g_ref.t_diag, g_ref.mod_tile, "_Z22fwTilingDiagonalKernelILi32EEvPiii"));
    REF_CHECK(cuModuleGetFunction(&g_ref.t_row, g_ref.mod_tile, "_Z17fwTilingRowKernelILi32EEvPiii"));
    REF_CHECK(cuModuleGetFunction(&g_ref.t_col, g_ref.mod_tile, "_Z20fwTilingColumnKernelILi32EEvPiii"));
    REF_CHECK(cuModuleGetFunction(&g_ref.t_oth, g_ref.mod_tile, "_Z20fwTilingOthersKernelILi32EEvPiii"));
    REF_CHECK(cuModuleGetFunction(&g_ref.ml_lead, g_ref.mod_ml, "_Z27fwMultiLayerLeadBlockKernelILi32EEvPiiii"));
    REF_CHECK(cuModuleGetFunction(&g_ref.ml_row, g_ref.mod_ml, "_Z25fwMultiLayerLeadRowKernelILi32EEvPiiiii"));
    REF_CHECK(cuModuleGetFunction(&g_ref.ml_col, g_ref.mod_ml, "_Z28fwMultiLayerLeadColumnKernelILi32EEvPiiiii"));
    REF_CHECK(cuModuleGetFunction(&g_ref.ml_row_rev, g_ref.mod_ml,
                                  "_Z32fwMultiLayerLeadRowReverseKernelILi32EEvPiiiiii"));
    REF_CHECK(cuModuleGetFunction(&g_ref.ml_col_rev, g_ref.mod_ml,
                                  "_Z35fwMultiLayerLeadColumnReverseKernelILi32EEvPiiiiii"));
    REF_CHECK(cuModuleGetFunction(&g_ref.ml_rest, g_ref.mod_ml, "_Z28fwMultiLayerRestBlocksKernelILi32EEvPiiiii"));
    g_ref.loaded = true;
    return 0;
}

// src/fw_baseline_gpu.cu:16-32: one 16x16-block grid launch per pivot k.
int refgpu_baseline_gpu(uint64_t d_D, int n) {
    if (!g_ref.loaded) return 1;
    const unsigned g = static_cast<unsigned>((n + 15) / 16);
    CUdeviceptr p = d_D;
    for (int k = 0; k < n; ++k) {
        void* args[] = {&p, &n, &k};
        if (int r = launch(g_ref.base, g, g, 0, args)) return r;
    }
    REF_CHECK(cuCtxSynchronize());
    return 0;
}

// src/fw_tiling_gpu.cu:253-284: per tile: diagonal, row, column, others.
int refgpu_tiling_gpu(uint64_t d_D, int n) {
    if (!g_ref.loaded) return 1;
    const int TILE = 32;
    const int numTiles = (n + TILE - 1) / TILE;
    const unsigned tileBytes = TILE * TILE * 4;
    CUdeviceptr p = d_D;
    for (int tile = 0; tile < numTiles; ++tile) {
        void* args[] = {&p, &n, &tile};
        if (int r = launch(g_ref.t_diag, 1, 1, tileBytes, args)) return r;
        if (numTiles > 1) {
            const unsigned m = static_cast<unsigned>(numTiles - 1);
            if (int r = launch(g_ref.t_row, m, 1, 2 * tileBytes, args)) return r;
            if (int r = launch(g_ref.t_col, m, 1, 2 * tileBytes, args)) return r;
            if (int r = launch(g_ref.t_oth, m, m, 2 * tileBytes, args)) return r;
        }
    }
    REF_CHECK(cuCtxSynchronize());
    return 0;
}

// src/fw_multi_layer_tiling_gpu.cu:507-577, including its argument
// normalisation (kappa <= 0 or > 16 becomes 4).
int refgpu_multi_layer_tiling_gpu(uint64_t d_D, int n, int kappa) {
    if (!g_ref.loaded) return 1;
    if (kappa <= 0 || kappa > 16) kappa = 4;
    const int TILE = 32;
    const int numTiles = (n + TILE - 1) / TILE;
    const unsigned tileBytes = TILE * TILE * 4;
    CUdeviceptr p = d_D;
    for (int kBlockBase = 0; kBlockBase < numTiles; kBlockBase += kappa) {
        int blocksInStage = std::min(kappa, numTiles - kBlockBase);
        for (int l = 0; l < blocksInStage; ++l) {
            void* a_lead[] = {&p, &n, &kBlockBase, &l};
            if (int r = launch(g_ref.ml_lead, 1, 1, 3 * tileBytes, a_lead)) return r;
            const int numRowColTiles = numTiles - 1;
            if (numRowColTiles > 0) {
                int nt = numTiles;
                void* a_rc[] = {&p, &n, &nt, &kBlockBase, &l};
                if (int r = launch(g_ref.ml_row, numRowColTiles, 1, 4 * tileBytes, a_rc)) return r;
                if (int r = launch(g_ref.ml_col, numRowColTiles, 1, 4 * tileBytes, a_rc)) return r;
            }
        }
        for (int l = blocksInStage - 2; l >= 0; --l) {
            const int currentK = kBlockBase + l;
            int nt = numTiles;
            void* a_rev[] = {&p, &n, &nt, &kBlockBase, &blocksInStage, &l};
            const int numRowTiles = (currentK + 1) + std::max(0, numTiles - (kBlockBase + blocksInStage));
            if (numRowTiles > 0) {
                if (int r = launch(g_ref.ml_row_rev, numRowTiles, 1, 2 * tileBytes, a_rev)) return r;
            }
            const int numColTiles = currentK + std::max(0, numTiles - (kBlockBase + blocksInStage));
            if (numColTiles > 0) {
                if (int r = launch(g_ref.ml_col_rev, numColTiles, 1, 2 * tileBytes, a_rev)) return r;
            }
        }
        if (blocksInStage < numTiles) {
            const unsigned m = static_cast<unsigned>(numTiles - blocksInStage);
            int nt = numTiles;
            void* a_rest[] = {&p, &n, &nt, &kBlockBase, &blocksInStage};
            if (int r = launch(g_ref.ml_rest, m, m, 2 * tileBytes, a_rest)) return r;
        }
    }
    REF_CHECK(cuCtxSynchronize());
    return 0;
}

}  // extern "C"

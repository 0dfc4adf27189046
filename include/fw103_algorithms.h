/*
 * C++ drop-in for the reference's algorithm registry (ddevedzic1/FW_CUDA).
 *
 * Same names, function-pointer types and argument meaning as the reference:
 *   AlgorithmFuncGPU / AlgorithmFuncCPU   include/algo_types.h:6,9
 *   GPU_ALGORITHMS, getGPUAlgorithmFunc,  src/cuda_utils.cu:7-23
 *   isGPUAlgorithm
 *   CPU_ALGORITHMS, getCPUAlgorithmFunc,  src/utils.cpp:14-24
 *   hasNegativeCycle                      src/utils.cpp:5-12
 * The three GPU functions call fw_apsp_i32 (fw103.h) on the legacy default
 * stream and return after cudaDeviceSynchronize, like the reference's
 * launchers; on a nonzero status (of the call, of the synchronisation, or of
 * fw_check_faults: a tile copy that missed its bounded wait) they print the
 * error and exit(EXIT_FAILURE), like the reference's checkCudaErrors
 * (include/cuda_utils.cuh:13-32).
 * All of it is exported by libfw103.so.
 */
#ifndef FW103_ALGORITHMS_H
#define FW103_ALGORITHMS_H

#include <map>
#include <string>

#include "fw103.h"

using WeightType = int;                                                    /* include/constants.h:9 */
using AlgorithmFuncCPU = void (*)(WeightType* D, int n, int tileSize);     /* include/algo_types.h:6 */
using AlgorithmFuncGPU = void (*)(WeightType* d_D, int n, int tileSize, int kappa); /* include/algo_types.h:9 */

constexpr int INF = FW_INF;                   /* include/constants.h:3 */
constexpr int MAX_N = FW_MAX_N;               /* include/constants.h:5 */
constexpr int MAX_EDGE_WEIGHT = FW_MAX_EDGE_WEIGHT; /* include/constants.h:7 */

/* src/fw_baseline_gpu.cu:16 */
void fwBaselineGPU(WeightType* d_D, int n, int tileSize, int kappa);
/* src/fw_tiling_gpu.cu:253 */
void fwTilingGPU(WeightType* d_D, int n, int tileSize, int kappa);
/* src/fw_multi_layer_tiling_gpu.cu:507 */
void fwMultiLayerTilingGPU(WeightType* d_D, int n, int tileSize, int kappa);
/* src/fw_baseline_cpu.cpp:3 — the host k-i-j sweep, selectable as "baseline_cpu" */
void fwBaselineCPU(WeightType* D, int n, int tileSize);

extern const std::map<std::string, AlgorithmFuncGPU> GPU_ALGORITHMS;
extern const std::map<std::string, AlgorithmFuncCPU> CPU_ALGORITHMS;

/* Throw std::out_of_range("ERROR: Unsupported GPU/CPU algorithm: <name>") when absent. */
AlgorithmFuncGPU getGPUAlgorithmFunc(const std::string& algorithmName);
AlgorithmFuncCPU getCPUAlgorithmFunc(const std::string& algorithmName);
bool isGPUAlgorithm(const std::string& algorithmName);
bool hasNegativeCycle(const WeightType* distMatrix, int n);

#endif /* FW103_ALGORITHMS_H */

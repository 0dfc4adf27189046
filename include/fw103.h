/*
 * fw103 — GB300 (sm_103a) Floyd-Warshall all-pairs shortest paths.
 *
 * C ABI of libfw103.so: plain pointers, sizes and status codes, callable from
 * C, C++, ctypes or any other FFI. Device pointers are CUDA device addresses
 * in the current device's context; `fw_stream_t` is a cudaStream_t (NULL =
 * the legacy default stream). Every entry point except the host-only ones
 * enqueues its work on the given stream and returns without synchronising;
 * the C++ shims in fw103_algorithms.h add the reference's synchronising
 * behaviour. On failure an entry point returns a nonzero fw_status and
 * fw_last_error_string() describes it (per host thread).
 *
 * Semantics follow the reference project ddevedzic1/FW_CUDA: int32 weights,
 * row-major n x n matrix, INF = 1e9 for a missing edge (include/constants.h:3),
 * relaxation D[i][j] = min(D[i][j], D[i][k] + D[k][j]) in plain int32
 * arithmetic (src/fw_baseline_cpu.cpp:9-12), 1 <= n <= 32769
 * (include/constants.h:5).
 */
#ifndef FW103_H
#define FW103_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FW_INF 1000000000       /* include/constants.h:3 */
#define FW_MAX_N 32769          /* include/constants.h:5 */
#define FW_MAX_EDGE_WEIGHT 25000 /* include/constants.h:7 */

typedef struct CUstream_st* fw_stream_t;

typedef enum fw_status {
    FW_OK = 0,
    FW_ERR_INVALID_ARGUMENT = 1, /* bad size, pointer, variant or layout */
    FW_ERR_CUDA = 2,             /* a CUDA runtime call or launch failed */
    FW_ERR_NO_MEMORY = 3,        /* workspace allocation failed */
    FW_ERR_TIMEOUT = 4,          /* a bounded device-side wait gave up */
    FW_ERR_NOT_BUILT = 5,        /* device code for this GPU is absent */
    FW_ERR_INTERNAL = 6          /* an internal consistency check failed */
} fw_status;

/* Which of the reference's three GPU algorithms a call stands in for
 * (src/cuda_utils.cu:7-11). Results are identical; the schedules differ. */
typedef enum fw_variant {
    FW_VARIANT_BASELINE = 0,    /* "baseline_gpu": one relaxation sweep per pivot */
    FW_VARIANT_TILING = 1,      /* "tiling_gpu": blocked sweep, 128-wide pivot blocks */
    FW_VARIANT_MULTI_LAYER = 2, /* "multi_layer_tiling_gpu": kappa pivot layers per pass */
    FW_VARIANT_AUTO = 3         /* n <= 2048: the int32 stripe sweep; larger: exact packed 16-bit
                                   sweep when provably identical, else MULTI_LAYER */
} fw_variant;

/* ---------------------------------------------------------------- plain APSP */

/* In-place APSP of the n x n int32 matrix at d_D.
 * Replaces AlgorithmFuncGPU (include/algo_types.h:9) as implemented by
 * fwBaselineGPU (src/fw_baseline_gpu.cu:16-32), fwTilingGPU
 * (src/fw_tiling_gpu.cu:253-284) and fwMultiLayerTilingGPU
 * (src/fw_multi_layer_tiling_gpu.cu:507-577). `tile` is accepted and ignored
 * as in the reference; `kappa` is used by FW_VARIANT_MULTI_LAYER only, with
 * the reference's normalisation (<= 0 or > 16 becomes 4,
 * src/fw_multi_layer_tiling_gpu.cu:511-513). Uses a per-(device, stream)
 * workspace that the library allocates on first use and keeps.
 * With n <= 2048, FW_VARIANT_TILING, FW_VARIANT_MULTI_LAYER and
 * FW_VARIANT_AUTO run as one cooperative launch (the stripe sweep: 8-wide
 * pivot blocks, the matrix held in registers across the SMs) when the device
 * can hold its grid and the workspace has fw_workspace_bytes_i32() bytes;
 * otherwise the 128-wide blocked sweep (or, for AUTO, the packed path) runs.
 * All give the same result. */
int fw_apsp_i32(int32_t* d_D, int64_t n, int tile, int kappa, int variant, fw_stream_t stream);

/* After a FW_VARIANT_AUTO call on `stream`: synchronises the stream and sets
 * *used_packed to 1 if the exact packed 16-bit sweep produced the result, 0 if
 * an int32 sweep ran (the stripe sweep for n <= 2048, or input outside
 * [0, 32767) u {INF}, or distances too close to the 16-bit cap to prove the
 * packed result exact). The answer lives
 * in the call's workspace: ask before freeing a caller workspace
 * (fw_apsp_i32_ws); a library workspace that a later, larger call on the
 * stream replaced makes this return FW_ERR_INVALID_ARGUMENT. */
int fw_apsp_auto_report(fw_stream_t stream, int* used_packed);

/* Bytes of device workspace fw_apsp_i32_ws needs for these arguments. */
size_t fw_workspace_bytes_i32(int64_t n, int tile, int kappa, int variant);

/* As fw_apsp_i32, with a caller-owned workspace (256-byte aligned);
 * allocates nothing. fw_workspace_bytes_i32() bytes select the fastest
 * schedule (the stripe sweep for n <= 2048, the look-ahead or two-block pass
 * of the blocked sweep above). The blocked variants also accept less, down to the 256-byte
 * status block and one pair of 128-row panels (128 x (n rounded up to 128)
 * ints each; two pairs for kappa > 4 at n >= 24576), which runs the 128-wide
 * blocked sweep without its look-ahead. */
int fw_apsp_i32_ws(int32_t* d_D, int64_t n, int tile, int kappa, int variant,
                   void* d_workspace, size_t workspace_bytes, fw_stream_t stream);

/* As fw_apsp_i32, for callers that cannot allocate device memory (a process
 * whose pool already owns the GPU's free memory, code that must not take the
 * implicit synchronisation of cudaMalloc/cudaFree, a plugin host without an
 * allocator). No counterpart in the reference. The workspace is a fixed
 * array of 8 MiB + 256 bytes inside the library's device image, held by every
 * GPU that loads the library until exit; n > 8192 is rejected with
 * FW_ERR_INVALID_ARGUMENT. FW_VARIANT_AUTO runs the int32 multi-layer sweep
 * here and kappa > 4 runs as kappa 4 (same result; after an AUTO call
 * fw_apsp_auto_report has no report for the stream). All calls share that
 * array: calls whose GPU work overlaps (other streams, other host threads)
 * race and must be serialised by the caller. The first call on each device
 * looks up the array's device address (cudaGetSymbolAddress); make it before
 * any stream capture. fw_check_faults reads the call's status word, which
 * lives in the array: check before the next call. */
int fw_apsp_i32_noalloc(int32_t* d_D, int64_t n, int tile, int kappa, int variant, fw_stream_t stream);

/* ---------------------------------------------------------------- out-of-core */

/* Solves an n x n int32 row-major matrix that stays in HOST memory, in place,
 * for matrices larger than the device's memory (the reference caps n at
 * MAX_N = 32769, include/constants.h:5, and copies the whole matrix to the
 * device, src/gpu_memory.cu:13-16). Each pass of `pass_width` pivots
 * (a multiple of 128; 0 = 2048) streams the matrix through the device in row
 * stripes of `stripe_rows` rows (a multiple of 128; 0 = chosen from the free
 * device memory), so a pass moves 8 n^2 bytes for pass_width * n^2
 * relaxations. The result is bit-identical to fw_apsp_i32. Page-locked host
 * memory gives asynchronous copies; pageable memory is registered for the
 * duration of the call when possible. Allocates its device buffers per call
 * (fw_host_solve_device_bytes) and returns when h_D holds the result; work is
 * enqueued on `stream` and two streams of its own. */
int fw_apsp_i32_host(int32_t* h_D, int64_t n, int64_t pass_width, int64_t stripe_rows, fw_stream_t stream);

/* Device bytes fw_apsp_i32_host allocates for these arguments (0 for invalid
 * ones; stripe_rows must be given, not 0). */
size_t fw_host_solve_device_bytes(int64_t n, int64_t pass_width, int64_t stripe_rows);

/* ---------------------------------------------------------------- path reconstruction */

/* int32 APSP that also records next hops, for `batch` equal-size graphs
 * (stride n*n): d_D as in fw_apsp_i32 (same distances, bit for bit), d_nh[i][j]
 * = the vertex after i on a shortest path to j (j for a direct edge when no
 * shorter path exists, i on the diagonal, -1 when j is unreachable), updated
 * on strict improvement as nh[i][j] = nh[i][k]. The distances are exact for
 * any graph without negative cycles; the next hops spell out shortest paths
 * when every cycle has positive weight (with zero-weight cycles, equal-length
 * alternatives can make recorded first hops point around such a cycle). No
 * counterpart in the reference (its sweeps keep distances only). */
int fw_apsp_paths_i32(int32_t* d_D, int32_t* d_nh, int64_t n, int64_t batch, fw_stream_t stream);

/* Host helper: walks a next-hop matrix (host copy) from i to j, writing up to
 * `cap` vertices (i first, j last) into h_path; returns the number of
 * vertices on the path, 0 when j is unreachable, a negative fw_status-like
 * error (sets the last error) when the next hops do not form a path. */
int fw_path_length_i32(const int32_t* h_nh, int64_t n, int64_t i, int64_t j, int32_t* h_path, int64_t cap);

/* ---------------------------------------------------------------- graph I/O, checks */

/* Dense n x n int32 matrix from a CSR adjacency on the device (d_rowptr: n+1
 * monotone offsets, d_col / d_w: rowptr[n] column indices and int32 weights),
 * in the reference's convention: FW_INF where there is no edge, 0 on the
 * diagonal (a negative self-loop lowers it), the smallest weight among
 * duplicate edges. Edges with a column outside [0, n) or a weight >= FW_INF
 * are skipped and counted into *d_bad when d_bad is not NULL. With d_col or
 * d_w NULL only the empty graph is written. No counterpart in the reference
 * (its generator is dense and on the host, src/graph_generator.cpp:7-46). */
int fw_dense_from_csr_i32(const int64_t* d_rowptr, const int32_t* d_col, const int32_t* d_w, int64_t n,
                          int32_t* d_D, uint32_t* d_bad, fw_stream_t stream);

/* d_flags[b] = 1 if graph b (of `batch` equal-size n x n graphs, stride n*n)
 * has a negative diagonal entry after the sweep, else 0: the reference's
 * hasNegativeCycle (src/utils.cpp:5-12) on the device. */
int fw_negative_cycle_i32(const int32_t* d_D, int64_t n, int64_t batch, int32_t* d_flags, fw_stream_t stream);

/* ---------------------------------------------------------------- batched APSP */

/* Many independent graphs solved in one persistent launch. No counterpart in
 * the reference; each graph's result is the reference's baseline_cpu sweep
 * (src/fw_baseline_cpu.cpp:6-15) of that graph. Graph g is an n_g x n_g
 * int32 row-major matrix at element offset offsets[g] of one packed device
 * buffer (1 <= n_g <= 4096, graphs must not overlap), solved in place. */
typedef struct fw_batch_plan fw_batch_plan;

/* Offsets for a dense packing with 16-byte aligned graph starts; writes
 * count offsets and the total element count of the packed buffer. */
int fw_batch_pack_offsets(const int32_t* h_sizes, int64_t count, int64_t* h_offsets, int64_t* total_elems);

/* Sorts the graphs into size buckets, uploads the work list and allocates
 * the per-CTA workspace on the current device. */
int fw_batch_plan_create(fw_batch_plan** plan, const int32_t* h_sizes, const int64_t* h_offsets, int64_t count);

/* Chooses the per-bucket schedule (graphs per CTA, CTAs per SM) by timing the
 * candidates on a scratch copy of d_packed (left unchanged). Synchronises. */
int fw_batch_plan_autotune(fw_batch_plan* plan, const int32_t* d_packed, fw_stream_t stream);

/* Solves every graph of the batch in place: one CUDA-graph launch (captured
 * on the first call for this d_packed, replayed afterwards). A plan belongs to
 * the device it was created on and holds one work counter and one workspace:
 * its solves must not overlap (one stream, or ordered by events). */
int fw_apsp_batched_i32(fw_batch_plan* plan, int32_t* d_packed, fw_stream_t stream);

/* The chosen schedule as text, and the batch's total relaxations (sum n^3). */
int fw_batch_plan_describe(const fw_batch_plan* plan, char* buf, size_t cap, double* relaxations);

void fw_batch_plan_destroy(fw_batch_plan* plan);

/* ---------------------------------------------------------------- differentiable */

/* fp32 APSP that also records next hops, for `batch` graphs of n x n stored
 * one after another (stride n*n). No counterpart in the reference. On entry
 * d_D holds the weights (+inf = no edge); on return the distances, and d_nh
 * the next hop of every shortest path (nh[i][j] = j for a direct edge, i on
 * the diagonal, -1 when j is unreachable), updated as in the sweep
 * if (D[i][k] + D[k][j] < D[i][j]) { D[i][j] = D[i][k] + D[k][j]; nh[i][j] = nh[i][k]; }. */
int fw_forward_f32(float* d_D, int32_t* d_nh, int64_t n, int64_t batch, fw_stream_t stream);

/* dL/dW for L depending on D = fw_forward_f32(W): every edge (u, v) on the
 * recorded path i -> j receives dL/dD[i][j]; d_dLdW is overwritten (zero for
 * non-edges). d_bad_walks, if not NULL, is a device int incremented by the
 * number of paths that did not reach their end within n hops (0 for a valid
 * next-hop matrix). Floating-point atomics: the summation order varies. */
int fw_backward(const float* d_dLdD, const int32_t* d_nh, float* d_dLdW, int64_t n, int64_t batch,
                int32_t* d_bad_walks, fw_stream_t stream);

/* ---------------------------------------------------------------- host side */

/* The reference's random digraph (src/graph_generator.cpp:7-46) into a host
 * buffer of n*n int32: std::mt19937(seed, or random_device when seed == 0),
 * per ordered pair in row-major order: i == j -> 0; else a
 * bernoulli(density) draw and, if it fires, a uniform integer in
 * [wmin, wmax]; else FW_INF. wmin = 0, wmax = FW_MAX_EDGE_WEIGHT reproduces
 * generateAlignedGraph1D byte for byte under the same libstdc++. */
int fw_generate_graph_i32(int32_t* h_out, int64_t n, double density, uint32_t seed,
                          int32_t wmin, int32_t wmax);

/* fw_generate_graph_i32's matrix, value for value, generated on the device
 * into d_D (n*n int32): the MT19937 word stream is produced in parallel
 * chunks whose starting states come from polynomial jump-ahead, and the
 * variable-length draws (two words per pair, one more per edge and per
 * rejection of the weight draw) are parsed in parallel. Replaces the host
 * generation of src/graph_generator.cpp:7-46 and the n*n host-to-device
 * copy of src/gpu_memory.cu:13-16. Allocates ~4 bytes per generator word
 * (about 2 + density words per pair) on `stream` and returns when d_D is
 * written. */
int fw_generate_graph_device_i32(int32_t* d_D, int64_t n, double density, uint32_t seed,
                                 int32_t wmin, int32_t wmax, fw_stream_t stream);

/* Host: `count` outputs of std::mt19937(seed) starting after the first
 * `skip` outputs, computed by the same polynomial jump-ahead (no device). */
int fw_mt19937_outputs(uint32_t seed, uint64_t skip, int64_t count, uint32_t* h_out);

/* Tile copies (TMA) of the int32 remainder kernel that did not arrive within
 * their bounded wait since the library was loaded on this device: 0 in a
 * working build. The kernel records the fault instead of waiting forever; the
 * affected tiles are then not updated. Synchronous (reads a device word). */
int fw_copy_faults(unsigned int* count);

/* Synchronises `stream` and reads the status word of the last call on it (on
 * the current device) among fw_apsp_i32, fw_apsp_i32_ws, fw_apsp_i32_noalloc,
 * fw_apsp_paths_i32 and fw_forward_f32. Their kernels wait for each tile copy
 * with a bounded wait; a copy that does not arrive in time is counted in that
 * word and the affected tiles are left as they were, instead of the kernel
 * waiting forever. Returns FW_OK when the count is 0, FW_ERR_TIMEOUT (the
 * call's result is not valid) when it is not, FW_ERR_INVALID_ARGUMENT when no
 * such call was made on the stream or its library workspace was replaced
 * since. *count (may be NULL) receives the count. The word lives in the call's
 * workspace: ask before freeing a caller workspace (fw_apsp_i32_ws).
 * The reference has no status (it prints and exits on a CUDA error,
 * include/cuda_utils.cuh:13-32); the C++ shims of fw103_algorithms.h call
 * this after every solve and keep that print-and-exit contract. */
int fw_check_faults(fw_stream_t stream, unsigned int* count);

/* Test hooks: host-side fault injection, no GPU fault involved.
 * FW_INJECT_CALL_FAULT: the next sweep call on this host thread sets its own
 * status word after its kernels, as one missed tile copy would, so that
 * fw_check_faults (and the C++ shims) report FW_ERR_TIMEOUT.
 * FW_INJECT_PACKED_FAULT: the next FW_VARIANT_AUTO call marks its packed
 * sweep as having missed a copy before the guarded decode, so the packed
 * result is refused and the int32 sweep produces the result (as it does
 * after a real miss). Kinds may be OR-ed; 0 clears pending injections. */
#define FW_INJECT_CALL_FAULT 1
#define FW_INJECT_PACKED_FAULT 2
int fw_debug_inject(int kinds);

/* Test hook: one CTA arms an mbarrier for a 16-byte transfer that is never
 * issued and waits for it with the kernels' bounded wait, limited to `spins`
 * tries (1 .. 1048576); then it completes the transfer count itself so the
 * barrier is left balanced. Returns FW_ERR_TIMEOUT when the wait gave up (the
 * expected outcome), FW_OK if it did not. Synchronous. */
int fw_debug_bounded_wait(int spins, fw_stream_t stream);

/* Test hook: one thread runs the stripe sweep's bounded flag wait (the wait
 * of the small-graph sweep for a pivot stripe another CTA publishes) on a
 * flag that nothing sets, limited to `limit_us` microseconds (1 .. 1000000),
 * then sets the flag and checks that the same wait sees it. Returns
 * FW_ERR_TIMEOUT when the first wait gave up (the expected outcome), FW_OK if
 * it did not. No counterpart in the reference. Synchronous. */
int fw_debug_flag_wait(int64_t limit_us, fw_stream_t stream);

/* Message of the last failure on this host thread ("" if none). */
const char* fw_last_error_string(void);

/* Library version string. */
const char* fw_version(void);

/* ---------------------------------------------------------------- measurement */

/* Per-kernel timing over a window: fw_profile_begin() makes the library
 * bracket each launch it issues with CUDA events on the launch stream;
 * fw_profile_end() synchronises those events and reports, per kernel class,
 * the launch count, summed device time and summed relaxations. */
typedef struct fw_kernel_stats {
    char name[32];
    int64_t launches;
    double total_ms;
    double relaxations;
} fw_kernel_stats;

int fw_profile_begin(void);
/* Writes up to `cap` entries; *count receives the number of kernel classes. */
int fw_profile_end(fw_kernel_stats* out, int cap, int* count);

/* Integer issue ceiling of this GPU for min-plus relaxations, measured with a
 * register-only kernel (no memory traffic): relaxations per second when every
 * relaxation is one DPX add-min instruction (dpx_only), and the best rate of
 * the instruction mix the blocked kernels use (mixed). */
int fw_measure_relax_peak(double* dpx_only, double* mixed, fw_stream_t stream);

/* What the int32 relaxation rate is built from, measured with register-only
 * kernels (8 CTAs of 256 threads per SM, 16 independent accumulators per
 * thread, no memory traffic). rates[0..8] (up to `count` entries):
 *   lane operations per second of one instruction class alone:
 *   [0] DPX add-min min(a + b, c)   [1] integer multiply-add a * 1 + b
 *   [2] DPX three-way min           [3] add             [4] min
 *   [5] [0] and [1] alternating (both classes counted);
 *   relaxations per second of a relaxation form:
 *   [6] two multiply-adds + one three-way min (2 relaxations)
 *   [7] two DPX add-mins (2 relaxations)
 *   [8] [6] followed by one DPX add-min (3 relaxations).
 * No counterpart in the reference. */
int fw_measure_int32_rates(double* rates, int count, fw_stream_t stream);

/* The same for the packed 16-bit form of FW_VARIANT_AUTO's fast path (two
 * 15-bit lanes per word): every relaxation pair one packed DPX add-min
 * (dpx_only), and the best rate of the packed kernels' instruction mix
 * (mixed). */
int fw_measure_relax_peak_packed(double* dpx_only, double* mixed, fw_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* FW103_H */

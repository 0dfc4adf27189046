// Oracle for the Floyd-Warshall all-pairs shortest path (APSP) path.
//
// TEST INFRASTRUCTURE ONLY. This file is the CPU restatement that the test
// suite, the smoke check and the benchmark's CPU-baseline leg use as the
// checker. Nothing in the shipped library links, loads or calls it.
//
// What is restated, and from where (paths are relative to the reference
// project ddevedzic1/FW_CUDA):
//   * oracle_generate_graph: the dense random digraph of
//     src/graph_generator.cpp:7-46 (std::mt19937 seeded with `seed`, one
//     bernoulli_distribution(density) draw per ordered pair i != j in
//     row-major order, then a uniform_int_distribution weight draw when the
//     edge exists; diagonal 0; missing edge = INF). The weight range is a
//     parameter here: [0, 25000] (include/constants.h:7) reproduces the
//     reference byte for byte when built against the same libstdc++.
//   * oracle_fw_i32: the textbook in-place k-i-j sweep of
//     src/fw_baseline_cpu.cpp:3-16, with the same int32 add and strict `<`.
//   * oracle_fw_i32_pivots: the same sweep restricted to pivots [k0, k1),
//     optionally with the i-loop split over host threads (one barrier per
//     pivot). Used to time bounded samples of a large solve.
//   * oracle_has_negative_cycle: src/utils.cpp:5-12.
//   * oracle_mt19937_outputs: std::mt19937 outputs after a discard, the
//     engine the generator draws from.
// Added checkers with no reference counterpart:
//   * oracle_sssp_dense: dense Dijkstra from one source on the same INF
//     convention (exact for non-negative weights); checks sampled rows of a
//     full-size solve that the k-i-j sweep cannot finish in test time.
//   * oracle_fw_f64_nexthop / oracle_fw_f32_nexthop: the k-i-j sweep in
//     FP64 / FP32 that also records next hops (nh[i][j] <- nh[i][k] on a
//     strict improvement); missing edges are +infinity.
//   * oracle_fw_backward: dL/dW by walking every recorded path.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <limits>
#include <random>
#include <thread>
#include <vector>
#include <atomic>

namespace {

constexpr int32_t kInf = 1000000000;  // include/constants.h:3

// Sense-reversing spin barrier for the threaded sweep (host threads only).
struct SpinBarrier {
    explicit SpinBarrier(int n) : count_(n), total_(n) {}
    void wait() {
        const int gen = gen_.load(std::memory_order_acquire);
        if (count_.fetch_sub(1, std::memory_order_acq_rel) == 1) {
            count_.store(total_, std::memory_order_relaxed);
            gen_.store(gen + 1, std::memory_order_release);
        } else {
            while (gen_.load(std::memory_order_acquire) == gen) {
                std::this_thread::yield();
            }
        }
    }
    std::atomic<int> count_;
    const int total_;
    std::atomic<int> gen_{0};
};

}  // namespace

extern "C" {

int32_t oracle_inf(void) { return kInf; }

// src/graph_generator.cpp:7-46 with the weight range as a parameter.
// Returns 0 on success, 1 on a bad argument (n <= 0 or density outside [0,1]).
int oracle_generate_graph(int32_t* out, int64_t n, double density, uint32_t seed,
                          int32_t wmin, int32_t wmax) {
    if (out == nullptr || n <= 0 || !(density >= 0.0 && density <= 1.0) || wmin > wmax) return 1;
    std::mt19937 gen(seed != 0 ? seed : std::random_device{}());
    std::uniform_int_distribution<int32_t> weight(wmin, wmax);
    std::bernoulli_distribution edge(density);
    const size_t nn = static_cast<size_t>(n);
    for (size_t i = 0; i < nn; ++i) {
        for (size_t j = 0; j < nn; ++j) {
            int32_t v;
            if (i == j) {
                v = 0;
            } else if (edge(gen)) {
                v = weight(gen);
            } else {
                v = kInf;
            }
            out[i * nn + j] = v;
        }
    }
    return 0;
}

// src/fw_baseline_cpu.cpp:6-15: for k, for i, for j: if (D[i][k]+D[k][j] < D[i][j]) store.
void oracle_fw_i32(int32_t* D, int64_t n) {
    const size_t nn = static_cast<size_t>(n);
    for (size_t k = 0; k < nn; ++k) {
        for (size_t i = 0; i < nn; ++i) {
            const int32_t dik = D[i * nn + k];
            int32_t* row = D + i * nn;
            const int32_t* rowk = D + k * nn;
            for (size_t j = 0; j < nn; ++j) {
                const int32_t cand = dik + rowk[j];
                if (cand < row[j]) row[j] = cand;
            }
        }
    }
}

// Pivots [k0, k1) of the same sweep; rows split over `threads` host threads.
// With threads == 1 this is exactly oracle_fw_i32 restricted to the pivots.
// With more threads each pivot's row k and column k are read while other
// rows are written; they do not change during pivot k while D[k][k] >= 0,
// so the result equals the single-threaded one for graphs without negative
// cycles.
void oracle_fw_i32_pivots(int32_t* D, int64_t n, int64_t k0, int64_t k1, int threads) {
    const size_t nn = static_cast<size_t>(n);
    if (k0 < 0) k0 = 0;
    if (k1 > n) k1 = n;
    if (threads <= 1) {
        for (int64_t k = k0; k < k1; ++k) {
            for (size_t i = 0; i < nn; ++i) {
                const int32_t dik = D[i * nn + k];
                int32_t* row = D + i * nn;
                const int32_t* rowk = D + static_cast<size_t>(k) * nn;
                for (size_t j = 0; j < nn; ++j) {
                    const int32_t cand = dik + rowk[j];
                    if (cand < row[j]) row[j] = cand;
                }
            }
        }
        return;
    }
    SpinBarrier barrier(threads);
    auto worker = [&](int t) {
        const size_t lo = nn * t / threads, hi = nn * (t + 1) / threads;
        for (int64_t k = k0; k < k1; ++k) {
            const int32_t* rowk = D + static_cast<size_t>(k) * nn;
            for (size_t i = lo; i < hi; ++i) {
                const int32_t dik = D[i * nn + k];
                int32_t* row = D + i * nn;
                for (size_t j = 0; j < nn; ++j) {
                    const int32_t cand = dik + rowk[j];
                    if (cand < row[j]) row[j] = cand;
                }
            }
            barrier.wait();
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(worker, t);
    worker(0);
    for (auto& th : pool) th.join();
}

// `count` outputs of std::mt19937(seed) after discarding the first `skip`
// (the engine of src/graph_generator.cpp:18), straight from the standard
// library: the checker for the jump-ahead of the device generator.
void oracle_mt19937_outputs(uint32_t seed, uint64_t skip, int64_t count, uint32_t* out) {
    std::mt19937 gen(seed);
    gen.discard(skip);
    for (int64_t i = 0; i < count; ++i) out[i] = static_cast<uint32_t>(gen());
}

// src/utils.cpp:5-12.
int oracle_has_negative_cycle(const int32_t* D, int64_t n) {
    for (int64_t i = 0; i < n; ++i) {
        if (D[i * n + i] < 0) return 1;
    }
    return 0;
}

// Dense O(n^2) Dijkstra from `src` over weights W (row-major, INF = missing),
// non-negative weights only. out[j] = min(INF, shortest path length); out[src]
// = min(W[src][src], shortest cycle through src). This is what the k-i-j
// sweep yields for such graphs, because every stored value is an exact path
// length below INF or INF itself.
void oracle_sssp_dense(const int32_t* W, int64_t n, int64_t src, int32_t* out) {
    const size_t nn = static_cast<size_t>(n);
    std::vector<int64_t> dist(nn, std::numeric_limits<int64_t>::max());
    std::vector<char> done(nn, 0);
    // Seed with the direct edges from src so that src itself can be reached
    // again only through a cycle.
    const int32_t* ws = W + static_cast<size_t>(src) * nn;
    for (size_t j = 0; j < nn; ++j) {
        if (ws[j] < kInf) dist[j] = ws[j];
    }
    for (size_t it = 0; it < nn; ++it) {
        int64_t best = std::numeric_limits<int64_t>::max();
        size_t u = nn;
        for (size_t j = 0; j < nn; ++j) {
            if (!done[j] && dist[j] < best) { best = dist[j]; u = j; }
        }
        if (u == nn) break;
        done[u] = 1;
        const int32_t* wu = W + u * nn;
        for (size_t j = 0; j < nn; ++j) {
            if (wu[j] < kInf) {
                const int64_t c = best + wu[j];
                if (c < dist[j]) dist[j] = c;
            }
        }
    }
    for (size_t j = 0; j < nn; ++j) {
        int64_t v = dist[j];
        if (j == static_cast<size_t>(src)) v = std::min<int64_t>(v, ws[j]);
        out[j] = v >= kInf ? kInf : static_cast<int32_t>(v);
    }
}

// k-i-j sweep in FP64 with next-hop recording. W: +inf = no edge. On entry
// D = W; nh is initialised here: nh[i][j] = j where W[i][j] is finite and
// i != j, nh[i][i] = i, -1 otherwise. On a strict improvement through k,
// nh[i][j] = nh[i][k].
void oracle_fw_f64_nexthop(double* D, int32_t* nh, int64_t n) {
    const size_t nn = static_cast<size_t>(n);
    for (size_t i = 0; i < nn; ++i)
        for (size_t j = 0; j < nn; ++j)
            nh[i * nn + j] = (i == j) ? static_cast<int32_t>(i)
                                      : (std::isfinite(D[i * nn + j]) ? static_cast<int32_t>(j) : -1);
    for (size_t k = 0; k < nn; ++k) {
        for (size_t i = 0; i < nn; ++i) {
            const double dik = D[i * nn + k];
            const int32_t hik = nh[i * nn + k];
            for (size_t j = 0; j < nn; ++j) {
                const double c = dik + D[k * nn + j];
                if (c < D[i * nn + j]) { D[i * nn + j] = c; nh[i * nn + j] = hik; }
            }
        }
    }
}

// The same sweep in FP32 (k-i-j order, round-to-nearest adds).
void oracle_fw_f32_nexthop(float* D, int32_t* nh, int64_t n) {
    const size_t nn = static_cast<size_t>(n);
    for (size_t i = 0; i < nn; ++i)
        for (size_t j = 0; j < nn; ++j)
            nh[i * nn + j] = (i == j) ? static_cast<int32_t>(i)
                                      : (std::isfinite(D[i * nn + j]) ? static_cast<int32_t>(j) : -1);
    for (size_t k = 0; k < nn; ++k) {
        for (size_t i = 0; i < nn; ++i) {
            const float dik = D[i * nn + k];
            const int32_t hik = nh[i * nn + k];
            for (size_t j = 0; j < nn; ++j) {
                const float c = dik + D[k * nn + j];
                if (c < D[i * nn + j]) { D[i * nn + j] = c; nh[i * nn + j] = hik; }
            }
        }
    }
}

// dL/dW for L = sum_ij G[i][j] * D[i][j], D = APSP(W): every edge (u, v) on
// the recorded path i -> j receives G[i][j]. Pairs with i == j or with no
// path (nh = -1) contribute nothing; a pair whose walk does not reach j
// within n hops is counted in the return value (0 = every walk ended).
int64_t oracle_fw_backward(const double* G, const int32_t* nh, int64_t n, double* dW) {
    const size_t nn = static_cast<size_t>(n);
    std::memset(dW, 0, sizeof(double) * nn * nn);
    int64_t bad = 0;
    for (size_t i = 0; i < nn; ++i) {
        for (size_t j = 0; j < nn; ++j) {
            if (i == j || nh[i * nn + j] < 0) continue;
            const double g = G[i * nn + j];
            size_t u = i;
            size_t steps = 0;
            while (u != j && steps < nn) {
                const int32_t v = nh[u * nn + j];
                if (v < 0) break;
                dW[u * nn + static_cast<size_t>(v)] += g;
                u = static_cast<size_t>(v);
                ++steps;
            }
            if (u != j) ++bad;
        }
    }
    return bad;
}

}  // extern "C"

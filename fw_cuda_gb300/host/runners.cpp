// Command-line runners over the fw103 engine, with the reference's command
// lines and output lines (ddevedzic1/FW_CUDA):
//   bench_runner <algorithm_name> <n_size> <density> [seed] [tile_size] [kappa]
//       src/bench_runner.cpp:7-103, src/algorithm_runner.cu:12-91
//   tests_runner <algorithm_name> [tile_size] [kappa]
//       src/tests_main.cpp:6-50, src/tests_runner.cu:12-41, src/tests.cpp, src/tests_gpu.cu
// Differences, all additive: bench_runner also prints the throughput in
// relaxations per second and times a solve of the unsolved input (the
// reference times a second solve of an already solved matrix,
// src/timer.cu:43-53; the work is the same); tests_runner exits nonzero when
// a test fails (the reference always returns 0, src/tests_runner.cu:40); the
// environment variable FW_WEIGHT_RANGE="lo,hi" changes the generator's weight
// range (default 0,25000 as in the reference).
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "fw103.h"
#include "fw103_algorithms.h"

namespace {

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        std::cerr << "CUDA Error: " << what << ": " << cudaGetErrorName(e) << " (" << cudaGetErrorString(e) << ")\n";
        std::exit(EXIT_FAILURE);
    }
}

void weight_range(int* lo, int* hi) {
    *lo = 0;
    *hi = MAX_EDGE_WEIGHT;
    if (const char* e = std::getenv("FW_WEIGHT_RANGE")) {
        int a = 0, b = 0;
        if (std::sscanf(e, "%d,%d", &a, &b) == 2 && a <= b) {
            *lo = a;
            *hi = b;
        }
    }
}

std::vector<WeightType> generate(int n, double density, unsigned seed) {
    int lo, hi;
    weight_range(&lo, &hi);
    std::vector<WeightType> g(static_cast<size_t>(n) * n);
    if (fw_generate_graph_i32(g.data(), n, density, seed, lo, hi) != FW_OK) {
        std::cerr << "ERROR: " << fw_last_error_string() << "\n";
        return {};
    }
    return g;
}

// ------------------------------------------------------------------ bench
int execute_benchmark(const std::string& name, int n, int tileSize, int kappa, double density, unsigned seed) {
    if (n <= 0 || n > MAX_N) {
        std::cerr << "ERROR: Graph size (n) must be between 1 and " << MAX_N << ". Aborting.\n";
        return 1;
    }
    const bool isGPU = isGPUAlgorithm(name);
    std::cout << "\n========================================\n";
    std::cout << "BENCHMARK: " << name << "\n";
    std::cout << "========================================\n";
    std::cout << "Graph size: " << n << " vertices\n";
    std::cout << "Edge density: " << std::fixed << std::setprecision(1) << (density * 100.0) << "%\n";
    std::cout << "Tile size: " << tileSize << "\n";
    std::cout << "Kappa: " << kappa << "\n";
    std::cout << "Algorithm type: " << (isGPU ? "GPU" : "CPU") << "\n";
    if (seed == 0)
        std::cout << "Seed: Random (Non-reproducible)\n";
    else
        std::cout << "Seed: " << seed << " (Reproducible)\n";
    std::cout << "\n";
    std::cout << "Generating graph...\n";
    std::vector<WeightType> h = generate(n, density, seed);
    if (h.empty()) {
        std::cerr << "ERROR: Failed to generate graph.\n";
        return 1;
    }
    double elapsed = 0.0;
    const size_t bytes = static_cast<size_t>(n) * n * sizeof(WeightType);
    if (isGPU) {
        AlgorithmFuncGPU fn = getGPUAlgorithmFunc(name);
        std::cout << "Warming up GPU...\n";
        check(cudaFree(nullptr), "context");
        std::cout << "Copying graph to GPU...\n";
        WeightType *d = nullptr, *pristine = nullptr;
        check(cudaMalloc(&d, bytes), "cudaMalloc");
        check(cudaMalloc(&pristine, bytes), "cudaMalloc");
        check(cudaMemcpy(pristine, h.data(), bytes, cudaMemcpyHostToDevice), "copyToDevice");
        std::cout << "Running " << name << "...\n";
        check(cudaMemcpy(d, pristine, bytes, cudaMemcpyDeviceToDevice), "restore");
        fn(d, n, tileSize, kappa);  // warm-up solve (src/timer.cu:43-46)
        check(cudaMemcpy(d, pristine, bytes, cudaMemcpyDeviceToDevice), "restore");
        cudaEvent_t a, b;
        check(cudaEventCreate(&a), "event");
        check(cudaEventCreate(&b), "event");
        check(cudaEventRecord(a), "event");
        fn(d, n, tileSize, kappa);
        check(cudaEventRecord(b), "event");
        check(cudaEventSynchronize(b), "event");
        float ms = 0.f;
        check(cudaEventElapsedTime(&ms, a, b), "event");
        elapsed = ms / 1000.0;
        check(cudaMemcpy(h.data(), d, bytes, cudaMemcpyDeviceToHost), "copyToHost");
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        cudaFree(d);
        cudaFree(pristine);
    } else {
        AlgorithmFuncCPU fn = getCPUAlgorithmFunc(name);
        std::cout << "Running " << name << "...\n";
        const auto t0 = std::chrono::steady_clock::now();
        fn(h.data(), n, tileSize);
        elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    std::cout << "\nResults:\n";
    std::cout << "--------\n";
    std::cout << "Execution time: " << std::fixed << std::setprecision(6) << elapsed << " seconds\n";
    std::cout << "Throughput: " << std::scientific << std::setprecision(4)
              << (static_cast<double>(n) * n * n / elapsed) << " relaxations/s\n";
    return 0;
}

void bench_usage(const char* p) {
    std::cerr << "Usage: " << p << " <algorithm_name> <n_size> <density> [seed] [tile_size] [kappa]\n\n";
    std::cerr << "Arguments:\n";
    std::cerr << "  algorithm_name  Name of the algorithm to run\n";
    std::cerr << "  n_size          Graph size (number of vertices, 1 to " << MAX_N << ")\n";
    std::cerr << "  density         Edge density (0.0 to 1.0)\n";
    std::cerr << "  seed            Random seed (optional, 0 for random)\n";
    std::cerr << "  tile_size       Tile size for tiling/CUDA (optional)\n";
    std::cerr << "  kappa           Number of tile-layers to group (optional, used by multi_layer_tiling_gpu)\n\n";
    std::cerr << "Examples:\n";
    std::cerr << "  " << p << " baseline_cpu 1024 0.8\n";
    std::cerr << "  " << p << " baseline_gpu 2048 0.9 42 16\n";
    std::cerr << "  " << p << " multi_layer_tiling_gpu 4096 0.9 42 32 4\n";
}

// ------------------------------------------------------------------ tests
struct Suite {
    int passed = 0, total = 0;
    void equal(const std::vector<WeightType>& actual, const std::vector<WeightType>& expected, const std::string& t) {
        ++total;
        if (actual.size() != expected.size()) {
            std::cerr << "[ FAILED ] " << t << ": Matrix size mismatch (Expected: " << expected.size()
                      << ", Actual: " << actual.size() << ")\n";
            return;
        }
        const int n = static_cast<int>(std::lround(std::sqrt(static_cast<double>(actual.size()))));
        for (size_t i = 0; i < actual.size(); ++i) {
            if (actual[i] != expected[i]) {
                std::cerr << "[ FAILED ] " << t << ": Mismatch at position [" << i / n << "][" << i % n
                          << "]. Expected: " << expected[i] << ", Actual: " << actual[i] << "\n";
                return;
            }
        }
        std::cout << "[ PASSED ] " << t << "\n";
        ++passed;
    }
};

std::vector<WeightType> run_gpu(AlgorithmFuncGPU fn, const std::vector<WeightType>& in, int n, int tile, int kappa) {
    WeightType* d = nullptr;
    const size_t bytes = in.size() * sizeof(WeightType);
    check(cudaMalloc(&d, bytes), "cudaMalloc");
    check(cudaMemcpy(d, in.data(), bytes, cudaMemcpyHostToDevice), "copyToDevice");
    fn(d, n, tile, kappa);
    std::vector<WeightType> out(in.size());
    check(cudaMemcpy(out.data(), d, bytes, cudaMemcpyDeviceToHost), "copyToHost");
    check(cudaFree(d), "cudaFree");
    return out;
}

// Runs the suite of src/tests_gpu.cu:156-185 (gpu) or src/tests.cpp:140-164
// (cpu) with `solve` standing for the algorithm under test.
template <class Solve>
int run_suite(const std::string& banner, Solve solve, bool gpu_cases) {
    Suite s;
    std::cout << "\n========================================\n";
    std::cout << banner << "\n";
    std::cout << "========================================\n";
    const WeightType I = INF;
    s.equal(solve(std::vector<WeightType>{0}, 1), {0}, "Single node (1x1)");
    s.equal(solve(std::vector<WeightType>{0, I, I, 0}, 2), {0, I, I, 0}, "No edges (2x2)");
    s.equal(solve(std::vector<WeightType>{0, 1, I, 100, I, 0, 1, I, I, I, 0, 1, I, I, I, 0}, 4),
            {0, 1, 2, 3, I, 0, 1, 2, I, I, 0, 1, I, I, I, 0}, "Simple path optimization (4x4)");
    const std::vector<WeightType> disc = {0, 1, I, I, 1, 0, I, I, I, I, 0, 2, I, I, 2, 0};
    s.equal(solve(disc, 4), disc, "Disconnected components (4x4)");
    s.equal(solve(std::vector<WeightType>{0, 5, 10, 0, 0, -1, I, I, 0}, 3), {0, 5, 4, 0, 0, -1, I, I, 0},
            "Negative weights (3x3)");
    {
        ++s.total;
        const std::vector<WeightType> r = solve(std::vector<WeightType>{0, 2, I, I, 0, 1, I, -3, 0}, 3);
        if (hasNegativeCycle(r.data(), 3)) {
            std::cout << "[ PASSED ] Negative cycle detection (3x3)\n";
            ++s.passed;
        } else {
            std::cerr << "[ FAILED ] Negative cycle detection (3x3)\n";
        }
    }
    struct Case {
        int n;
        double d;
        unsigned seed;
    };
    std::vector<Case> cases = {{128, 0.9, 42}, {256, 0.9, 123}, {512, 0.9, 456}, {1024, 0.9, 789}};
    if (gpu_cases) {
        for (Case c : {Case{128, 0.1, 101}, Case{256, 0.1, 202}, Case{512, 0.1, 303}, Case{1024, 0.1, 404}})
            cases.push_back(c);
    }
    for (const Case& c : cases) {
        std::vector<WeightType> in = generate(c.n, c.d, c.seed);
        std::vector<WeightType> expected = in;
        fwBaselineCPU(expected.data(), c.n, 0);
        std::string name = "Large graph (N=" + std::to_string(c.n);
        if (gpu_cases) name += ", density=" + std::to_string(c.d);
        name += ", seed=" + std::to_string(c.seed) + ")";
        s.equal(solve(in, c.n), expected, name);
    }
    std::cout << "========================================\n";
    std::cout << "RESULTS: " << s.passed << "/" << s.total << " passed\n";
    std::cout << "========================================\n\n";
    return s.passed == s.total ? 0 : 1;
}

int execute_tests(const std::string& name, int tileSize, int kappa) {
    if (isGPUAlgorithm(name)) {
        AlgorithmFuncGPU fn = getGPUAlgorithmFunc(name);
        std::cout << "Warming up GPU...\n";
        check(cudaFree(nullptr), "context");
        return run_suite("TESTING (GPU): " + name + " (tileSize=" + std::to_string(tileSize) +
                             ", kappa=" + std::to_string(kappa) + ")",
                         [&](const std::vector<WeightType>& in, int n) { return run_gpu(fn, in, n, tileSize, kappa); },
                         true);
    }
    AlgorithmFuncCPU fn = nullptr;
    try {
        fn = getCPUAlgorithmFunc(name);
    } catch (const std::out_of_range& e) {
        std::cerr << "ERROR: " << e.what() << "\n";
        return 1;
    }
    return run_suite("TESTING: " + name + " (tileSize=" + std::to_string(tileSize) + ")",
                     [&](std::vector<WeightType> in, int n) {
                         fn(in.data(), n, tileSize);
                         return in;
                     },
                     false);
}

void tests_usage(const char* p) {
    std::cerr << "Usage: " << p << " <algorithm_name> [tile_size] [kappa]\n\n";
    std::cerr << "Arguments:\n";
    std::cerr << "  algorithm_name  Name of the algorithm to test\n";
    std::cerr << "  tile_size       Tile size (optional, default 0)\n";
    std::cerr << "  kappa           Number of tile-layers per stage for multi-layer tiling (optional, default 0)\n\n";
    std::cerr << "Examples:\n";
    std::cerr << "  " << p << " baseline_cpu\n";
    std::cerr << "  " << p << " baseline_gpu\n";
    std::cerr << "  " << p << " multi_layer_tiling_gpu 32 4\n";
}

int bench_main(int argc, char** argv) {
    if (argc < 4 || argc > 7) {
        bench_usage(argv[0]);
        return 1;
    }
    const std::string name = argv[1];
    int n = 0, tileSize = 0, kappa = 0;
    double density = 0.0;
    unsigned seed = 0;
    try {
        n = std::stoi(argv[2]);
        if (n <= 0 || n > MAX_N) {
            std::cerr << "ERROR: Invalid graph size (" << n << "). Must be between 1 and " << MAX_N << ".\n";
            return 1;
        }
    } catch (const std::exception&) {
        std::cerr << "ERROR: Invalid N_SIZE provided (" << argv[2] << "). Must be an integer.\n";
        return 1;
    }
    try {
        density = std::stod(argv[3]);
        if (density < 0.0 || density > 1.0) {
            std::cerr << "ERROR: Invalid density (" << density << "). Must be between 0.0 and 1.0.\n";
            return 1;
        }
    } catch (const std::exception&) {
        std::cerr << "ERROR: Invalid DENSITY provided (" << argv[3] << "). Must be a floating point number.\n";
        return 1;
    }
    if (argc >= 5) {
        try {
            seed = static_cast<unsigned>(std::stoul(argv[4]));
        } catch (const std::exception&) {
            std::cerr << "ERROR: Invalid SEED provided (" << argv[4] << "). Must be an unsigned integer.\n";
            return 1;
        }
    }
    if (argc >= 6) {
        try {
            tileSize = std::stoi(argv[5]);
            if (tileSize < 0 || tileSize > n) {
                std::cerr << "ERROR: Invalid TILE_SIZE (" << tileSize << "). Must be between 0 and " << n << ".\n";
                return 1;
            }
        } catch (const std::exception&) {
            std::cerr << "ERROR: Invalid TILE_SIZE provided (" << argv[5] << "). Must be an integer.\n";
            return 1;
        }
    }
    if (argc == 7) {
        try {
            kappa = std::stoi(argv[6]);
            if (kappa < 0) {
                std::cerr << "ERROR: Invalid KAPPA (" << kappa << "). Must be non-negative.\n";
                return 1;
            }
        } catch (const std::exception&) {
            std::cerr << "ERROR: Invalid KAPPA provided (" << argv[6] << "). Must be an integer.\n";
            return 1;
        }
    }
    try {
        return execute_benchmark(name, n, tileSize, kappa, density, seed);
    } catch (const std::exception& e) {
        std::cerr << "RUNTIME ERROR: " << e.what() << "\n";
        return 1;
    } catch (...) {
        std::cerr << "RUNTIME ERROR: An unknown error occurred.\n";
        return 1;
    }
}

int tests_main(int argc, char** argv) {
    if (argc < 2 || argc > 4) {
        tests_usage(argv[0]);
        return 1;
    }
    const std::string name = argv[1];
    int tileSize = 0, kappa = 0;
    if (argc >= 3) {
        try {
            tileSize = std::stoi(argv[2]);
        } catch (const std::exception&) {
            std::cerr << "ERROR: Invalid TILE_SIZE provided (" << argv[2] << "). Must be an integer.\n";
            return 1;
        }
    }
    if (argc == 4) {
        try {
            kappa = std::stoi(argv[3]);
        } catch (const std::exception&) {
            std::cerr << "ERROR: Invalid KAPPA provided (" << argv[3] << "). Must be an integer.\n";
            return 1;
        }
    }
    return execute_tests(name, tileSize, kappa);
}

}  // namespace

int main(int argc, char** argv) {
    // One binary, two names (bench_runner / tests_runner), chosen by argv[0].
    const char* base = std::strrchr(argv[0], '/');
    base = base ? base + 1 : argv[0];
    if (std::strstr(base, "tests_runner")) return tests_main(argc, argv);
    return bench_main(argc, argv);
}

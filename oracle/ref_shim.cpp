// C entry points over the reference's own CPU code, for pinning the oracle.
//
// TEST INFRASTRUCTURE ONLY. oracle/Makefile compiles this file together with
// the reference sources, in place under the reference checkout
// (src/fw_baseline_cpu.cpp, src/graph_generator.cpp, src/utils.cpp,
// src/tests.cpp), into oracle/_ref/libfwref.so. Nothing here is shipped; the
// golden-vector script in tests/golden/ and the oracle tests load it when it
// exists (it can only be built where the reference checkout is present).
#include <cstdint>
#include <cstring>
#include <vector>

#include "fw_baseline_cpu.h"   // src/fw_baseline_cpu.cpp:3
#include "graph_generator.h"   // src/graph_generator.cpp:48
#include "tests.h"             // src/tests.cpp:140
#include "utils.h"             // src/utils.cpp:5

extern "C" {

// generateGraph1D(n, density, seed) copied out into a caller buffer of n*n ints.
int ref_generate_graph(int32_t* out, int n, double density, unsigned int seed) {
    std::vector<WeightType> g = generateGraph1D(n, density, seed);
    if (g.empty()) return 1;
    std::memcpy(out, g.data(), g.size() * sizeof(WeightType));
    return 0;
}

// fwBaselineCPU(D, n, 0), in place.
void ref_fw_baseline_cpu(int32_t* D, int n) { fwBaselineCPU(D, n, 0); }

int ref_has_negative_cycle(const int32_t* D, int n) { return hasNegativeCycle(D, n) ? 1 : 0; }

// The reference's own CPU test suite run on baseline_cpu against itself.
void ref_run_tests_cpu(void) { runTestsCPU(fwBaselineCPU, fwBaselineCPU, "baseline_cpu", 0); }

}  // extern "C"

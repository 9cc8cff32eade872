// C++ caller of the reference-shaped interface (include/ghcm_eikonal.hpp),
// written the way the reference harness drives eikonal_hcm_opencl_ex
// (src/test_runner.cpp:169-223, 226-291): build a setup, bind a SolverFn,
// run it on a cost field from one seed.
//
// Exit status: 0 = solved and checked, 2 = no usable GPU (setup returned
// nullopt), 1 = a check failed.
#include <cmath>
#include <cstdio>

#include "ghcm_eikonal.hpp"

int main() {
    ghcm::HcmConfig config;
    config.block_size = 16;
    config.kernel = ghcm::HcmConfig::Kernel::Systolic;
    auto setup = ghcm::eikonal_hcm_cuda_setup(config);
    if (!setup) {
        std::puts("no device");
        return 2;
    }
    ghcm::SolverFn solve = ghcm::bind_solver(*setup);
    // constant cost 1 (field_cost_constant, src/test_runner.cpp:47-48), seed (3, 5)
    ghcm::Field2D<float> cost({37, 29}, 1.f);
    auto const r = solve(cost, {{3, 5}});
    // along the seed's row and column the Godunov solution is the L1 distance
    for (uint32_t x = 0; x < 37; ++x)
        if (r.field(x, 5) != std::fabs(float(x) - 3.f)) return 1;
    for (uint32_t y = 0; y < 29; ++y)
        if (r.field(3, y) != std::fabs(float(y) - 5.f)) return 1;
    if (r.stats.block_solves == 0 || r.duration_total.count() <= 0) return 1;
    // errors surface as exceptions, not exits
    try {
        solve(cost, {{37, 0}});
        return 1;
    } catch (ghcm::Error const& e) {
        if (e.status() != GHCM_ERR_BAD_ARG) return 1;
    }
    std::printf("ok %llu block-solves\n", static_cast<unsigned long long>(r.stats.block_solves));
    return 0;
}

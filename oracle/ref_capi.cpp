// C entry points over the reference's own CPU solvers, compiled from the
// reference sources where they lie (see oracle/Makefile, target `ref`).
//
//   ghcm_ref_fim -> eikonal_fim_sequential  (src/eikonal_fim.cpp:13-107)
//   ghcm_ref_fmm -> eikonal_fmm_sequential  (src/eikonal_fmm.cpp:13-71)
//
// Inputs follow the reference convention: a row-major W x H COST field
// (x fastest, src/util_dim.h:17-21; cost = h / speed, src/test_runner.cpp:38-42)
// and seed cells as (x, y) pairs. The output is the FP32 arrival-time field and
// the solver's own high_resolution_clock duration in microseconds.
//
// TEST INFRASTRUCTURE ONLY: used by tests/ and by the CPU-baseline legs of
// bench.py to pin the oracle restatement against the real reference.
#include "eikonal.h"

#include <cstdint>
#include <cstring>

namespace {

Field2D<float> make_field(const float* cost, std::uint32_t w, std::uint32_t h) {
    return Field2D<float>(glm::u32vec2(w, h), cost);
}

std::vector<uint2> make_seeds(const std::uint32_t* xy, std::uint32_t n) {
    std::vector<uint2> seeds;
    seeds.reserve(n);
    for (std::uint32_t i = 0; i < n; ++i) seeds.emplace_back(xy[2 * i], xy[2 * i + 1]);
    return seeds;
}

int copy_out(EikonalResult const& r, float* out, std::int64_t* us) {
    std::memcpy(out, r.field.backing_store().data(), r.field.size_flat() * sizeof(float));
    if (us) *us = static_cast<std::int64_t>(r.duration_total.count());
    return 0;
}

}  // namespace

extern "C" int ghcm_ref_fim(float eps, const float* cost, std::uint32_t w, std::uint32_t h,
                            const std::uint32_t* seeds_xy, std::uint32_t n_seeds, float* time_out,
                            std::int64_t* elapsed_us) {
    if (!cost || !time_out || w == 0 || h == 0) return -1;
    auto const r = eikonal_fim_sequential(eps, make_field(cost, w, h), make_seeds(seeds_xy, n_seeds));
    return copy_out(r, time_out, elapsed_us);
}

extern "C" int ghcm_ref_fmm(const float* cost, std::uint32_t w, std::uint32_t h,
                            const std::uint32_t* seeds_xy, std::uint32_t n_seeds, float* time_out,
                            std::int64_t* elapsed_us) {
    if (!cost || !time_out || w == 0 || h == 0) return -1;
    auto const r = eikonal_fmm_sequential(make_field(cost, w, h), make_seeds(seeds_xy, n_seeds));
    return copy_out(r, time_out, elapsed_us);
}

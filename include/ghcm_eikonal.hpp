// ghcm_eikonal.hpp - header-only C++ interface over the C ABI (ghcm.h), in the
// shape of the reference's solver interface src/eikonal.h:12-67, so that a
// caller of eikonal_hcm_opencl{,_setup,_ex} can switch to the GB300 solver by
// renaming the calls:
//
//   reference (src/eikonal.h)                  here
//   HcmConfig                                  ghcm::HcmConfig (same fields + GB300 knobs)
//   EikonalResult                              ghcm::EikonalResult (+ solver stats)
//   eikonal_hcm_opencl_setup(device, config)   ghcm::eikonal_hcm_cuda_setup(config, device)
//   eikonal_hcm_opencl_ex(setup, cost, seeds)  ghcm::eikonal_hcm_cuda_ex(setup, cost, seeds)
//   eikonal_hcm_opencl(device, config, ...)    ghcm::eikonal_hcm_cuda(config, ..., device)
//   SolverFn (src/test_runner.cpp:123)         ghcm::SolverFn
//
// Differences, by design: errors throw ghcm::Error instead of exiting the
// process (src/eikonal_hcm.cpp:181-182, src/util_opencl.h:48-57); setup
// returns std::nullopt on failure as the reference's optional does.
#pragma once

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <functional>
#include <memory>
#include <optional>
#include <stdexcept>
#include <string>
#include <vector>

#include "ghcm.h"

namespace ghcm {

struct uint2 {
    uint32_t x, y;
};

// Row-major field, x fastest (Field2D, src/util_field.h; dim_idx, src/util_dim.h:17-21).
template <typename T>
class Field2D {
public:
    Field2D() = default;
    Field2D(uint2 size, T fill = T()) : size_(size), data_(static_cast<size_t>(size.x) * size.y, fill) {}
    Field2D(uint2 size, const T* values) : size_(size), data_(values, values + static_cast<size_t>(size.x) * size.y) {}

    uint2 size() const { return size_; }
    size_t size_flat() const { return data_.size(); }
    bool in_bounds(int64_t x, int64_t y) const { return x >= 0 && y >= 0 && x < size_.x && y < size_.y; }
    T& operator()(uint32_t x, uint32_t y) { return data_[x + static_cast<size_t>(y) * size_.x]; }
    const T& operator()(uint32_t x, uint32_t y) const { return data_[x + static_cast<size_t>(y) * size_.x]; }
    T& operator[](size_t i) { return data_[i]; }
    const T& operator[](size_t i) const { return data_[i]; }
    std::vector<T>& backing_store() { return data_; }
    const std::vector<T>& backing_store() const { return data_; }

private:
    uint2 size_{0, 0};
    std::vector<T> data_;
};

class Error : public std::runtime_error {
public:
    Error(int status, const std::string& what)
        : std::runtime_error(what + ": " + ghcm_status_string(status)), status_(status) {}
    int status() const { return status_; }

private:
    int status_;
};

struct HcmConfig {
    enum class Kernel { Systolic, FIM };
    enum class CacheMode { None, Time, Cost, Both };

    // the reference's fields and defaults (src/eikonal.h:17-26)
    uint8_t block_size = 8;               // 8, 16 or 32
    float workers_overload = 1.f;         // the thread count follows the tile size
    float compute_unit_overload = 1.f;    // n = compute_unit_overload x SM count
    float fim_minimum_change = 1e-5f;
    CacheMode cache_mode = CacheMode::Both;  // tiles always live in shared memory / registers
    Kernel kernel = Kernel::Systolic;
    // GB300 knobs
    uint32_t max_jobs = 0;                // explicit n; overrides compute_unit_overload when > 0
    uint32_t key_mode = GHCM_KEY_BOUNDARY_MIN;
    uint32_t max_sweeps = 0;
    uint32_t max_waves = 0;
    uint32_t wait_timeout_ms = 2000;
    bool use_tma = true;
    uint32_t refresh_solves = 0;          // quiet solves per tile that may raise cells (0 = 1, GHCM_REFRESH_*)
};

struct EikonalResult {
    using duration_t = std::chrono::microseconds;

    Field2D<float> field;
    duration_t duration_total{0}, duration_device{0};
    ghcm_stats stats{};
};

struct HcmSetup {
    HcmConfig config;
    std::shared_ptr<ghcm_ctx> ctx;
};

using SolverFn = std::function<EikonalResult(Field2D<float> const&, std::vector<uint2> const&)>;

namespace detail {
inline ghcm_config to_c(HcmConfig const& c, uint32_t sms, int device) {
    ghcm_config out;
    ghcm_config_default(&out);
    out.block_size = c.block_size;
    out.max_jobs = c.max_jobs ? c.max_jobs
                              : static_cast<uint32_t>(std::max(1.f, c.compute_unit_overload * static_cast<float>(sms)));
    out.eps = c.fim_minimum_change;
    out.kernel = c.kernel == HcmConfig::Kernel::FIM ? GHCM_KERNEL_FIM : GHCM_KERNEL_SYSTOLIC;
    out.key_mode = c.key_mode;
    out.max_sweeps = c.max_sweeps;
    out.max_waves = c.max_waves;
    out.wait_timeout_ms = c.wait_timeout_ms;
    out.device = device;
    out.use_tma = c.use_tma ? 1u : 0u;
    out.refresh_solves = c.refresh_solves;
    return out;
}

inline std::shared_ptr<ghcm_ctx> make_ctx(ghcm_config const& c, int* status) {
    ghcm_ctx* raw = nullptr;
    *status = ghcm_create(&c, &raw);
    if (*status != GHCM_OK) return nullptr;
    return std::shared_ptr<ghcm_ctx>(raw, [](ghcm_ctx* p) { ghcm_destroy(p); });
}
}  // namespace detail

// Builds a solver context (eikonal_hcm_opencl_setup, src/eikonal_hcm.cpp:137-175).
inline std::optional<HcmSetup> eikonal_hcm_cuda_setup(HcmConfig const& config, int device = -1) {
    int status = 0;
    auto probe = detail::make_ctx(detail::to_c(config, 1, device), &status);
    if (!probe) return std::nullopt;
    uint32_t sms = 0;
    ghcm_device_sm_count(probe.get(), &sms);
    auto ctx = detail::make_ctx(detail::to_c(config, sms, device), &status);
    if (!ctx) return std::nullopt;
    return HcmSetup{config, ctx};
}

// Solves a COST field (cost = h / speed, as the reference takes it) from the
// seed cells (eikonal_hcm_opencl_ex, src/eikonal_hcm.cpp:186-529).
inline EikonalResult eikonal_hcm_cuda_ex(HcmSetup const& setup, Field2D<float> const& field_cost,
                                         std::vector<uint2> const& seed_points) {
    auto const t0 = std::chrono::high_resolution_clock::now();
    EikonalResult r;
    r.field = Field2D<float>(field_cost.size(), 0.f);
    std::vector<uint32_t> seeds;
    seeds.reserve(seed_points.size() * 2);
    for (auto const& p : seed_points) {
        seeds.push_back(p.x);
        seeds.push_back(p.y);
    }
    int const rc = ghcm_solve(setup.ctx.get(), field_cost.backing_store().data(), 0, field_cost.size().x,
                              field_cost.size().y, 1.f, seeds.data(), static_cast<uint32_t>(seed_points.size()),
                              r.field.backing_store().data(), &r.stats);
    if (rc != GHCM_OK) throw Error(rc, "ghcm_solve");
    auto const t1 = std::chrono::high_resolution_clock::now();
    r.duration_total = std::chrono::duration_cast<EikonalResult::duration_t>(t1 - t0);
    r.duration_device = EikonalResult::duration_t(static_cast<int64_t>(r.stats.device_ms * 1e3));
    return r;
}

// One-shot setup + solve (eikonal_hcm_opencl, src/eikonal_hcm.cpp:177-184).
inline EikonalResult eikonal_hcm_cuda(HcmConfig const& config, Field2D<float> const& field_cost,
                                      std::vector<uint2> const& seed_points, int device = -1) {
    auto setup = eikonal_hcm_cuda_setup(config, device);
    if (!setup) throw Error(GHCM_ERR_UNSUPPORTED, "eikonal_hcm_cuda_setup");
    return eikonal_hcm_cuda_ex(*setup, field_cost, seed_points);
}

// A SolverFn bound to a setup, as the reference harness binds
// eikonal_hcm_opencl_ex (src/test_runner.cpp:249-252).
inline SolverFn bind_solver(HcmSetup setup) {
    return [setup](Field2D<float> const& f, std::vector<uint2> const& s) { return eikonal_hcm_cuda_ex(setup, f, s); };
}

}  // namespace ghcm

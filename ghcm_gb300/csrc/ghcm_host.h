// Host-side pieces shared by the C-ABI files (ghcm_capi.cpp, ghcm_batch.cpp):
// the context, device buffers and status mapping. Not part of the public
// interface.
#pragma once

#include "../../include/ghcm.h"
#include "ghcm_internal.h"

#include <cstddef>
#include <algorithm>
#include <cstdint>
#include <cstdio>

namespace ghcm {

// A growable device allocation.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    bool reserve(size_t need) {
        if (need <= bytes) return true;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (cudaMalloc(&p, need) != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            return false;
        }
        bytes = need;
        return true;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

static_assert(kParams == GHCM_MLP_PARAMS && kFeatures == GHCM_MLP_FEATURES && kHidden == GHCM_MLP_HIDDEN,
              "MLP shape differs from the C ABI");
static_assert(sizeof(TraceRec) == sizeof(ghcm_trace_record), "trace record layout differs from the C ABI");

// Bytes of the per-tile learning arrays (tstat | kmax | nsolve | last_change | vetoes | the scores of the
// entries of the two active lists).
inline size_t learn_bytes(uint32_t tiles) {
    return align_up(16ull * tiles, 256) + 6 * align_up(4ull * tiles, 256);
}

// Points s.learn's per-tile arrays into `base` (learn_bytes(tiles) bytes).
inline void bind_learn_arrays(Learn& L, char* base, uint32_t tiles) {
    size_t const a = align_up(16ull * tiles, 256), b = align_up(4ull * tiles, 256);
    L.tstat = reinterpret_cast<float4*>(base);
    L.kmax = reinterpret_cast<uint32_t*>(base + a);
    L.nsolve = reinterpret_cast<uint32_t*>(base + a + b);
    L.last_change = reinterpret_cast<uint32_t*>(base + a + 2 * b);
    L.vetoes = reinterpret_cast<uint32_t*>(base + a + 3 * b);
    L.lscore[0] = reinterpret_cast<float*>(base + a + 4 * b);
    L.lscore[1] = reinterpret_cast<float*>(base + a + 5 * b);
}

inline int map_cuda(cudaError_t e) {
    if (e == cudaSuccess) return GHCM_OK;
    if (e == cudaErrorMemoryAllocation) return GHCM_ERR_OOM;
    return GHCM_ERR_CUDA;
}

// Largest field side the solver accepts. Tile origins and staged-box
// coordinates are 32-bit signed in the kernels, and a side this size keeps
// side + B - 1 and every coordinate far from overflowing them.
constexpr uint32_t kMaxSide = 1u << 30;

// Ctl::error bits -> status, most specific first.
inline int status_from_error(uint32_t error) {
    if (error & kErrBadSeed) return GHCM_ERR_BAD_ARG;
    if (error & kErrBadInput) return GHCM_ERR_BAD_INPUT;
    if (error & kErrTimeout) return GHCM_ERR_TIMEOUT;
    if (error & (kErrInternal | kErrChecked)) return GHCM_ERR_INTERNAL;
    if (error & kErrNotConverged) return GHCM_ERR_NOT_CONVERGED;
    return GHCM_OK;
}

// Algorithmic HBM bytes of one block-solve of a B x B tile, FP32: speed read
// (B^2) + time tile with its edge halo, no corners, read ((B+2)^2 - 4) + time
// write (B^2).
inline uint32_t bytes_per_solve(uint32_t b) { return 4u * b * b + 4u * ((b + 2u) * (b + 2u) - 4u) + 4u * b * b; }

// The cost cap of a config (+inf when off).
inline float cost_cap_of(const ghcm_config& cfg) {
    return cfg.cost_cap > 0.f ? cfg.cost_cap : __builtin_huge_valf();
}

// GHCM_PROFILE builds: the per-phase counters of a finished solve, on stderr.
// GHCM_CHECKED builds: names a failed index check on stderr (the solve also
// returns GHCM_ERR_INTERNAL).
inline void report_checks(const Ctl& c) {
#ifdef GHCM_CHECKED
    if (c.error & kErrChecked)
        std::fprintf(stderr, "[ghcm-checked] an index check failed; largest failing site id %u\n", c.check_site);
#else
    (void)c;
#endif
}

inline void print_profile(const Ctl& c, int grid) {
#ifdef GHCM_PROFILE
    std::fprintf(stderr,
                 "[ghcm-prof] grid %d solves %llu waves %u residual_passes %u kernel_us %.1f | per wave: "
                 "decide %.2f us, span %.2f us, release seen after %.2f us, max sweeps %.1f | sweeps/solve %.1f\n",
                 grid, c.block_solves, c.waves, c.residual_passes, c.prof[5] / 1e3,
                 c.prof[2] / 1e3 / std::max(1ull, c.prof[9]), c.prof[6] / 1e3 / std::max(1ull, c.prof[9]),
                 c.prof[7] / 1e3 / std::max(1ull, c.prof[9]) / std::max(1, grid - 1),
                 double(c.prof[8]) / std::max(1ull, c.prof[9]), double(c.prof[3]) / std::max(1ull, c.block_solves));
    if (c.prof[9])
        std::fprintf(stderr, "[ghcm-prof] per wave, after the release: latest first-job start %.2f us, latest job end "
                     "%.2f us, longest block-solve %.2f us\n",
                     c.prof[17] / 1e3 / c.prof[9], c.prof[15] / 1e3 / c.prof[9], c.prof[19] / 1e3 / c.prof[9]);
    if (c.prof[9])
        std::fprintf(stderr, "[ghcm-prof] per wave, decision: control loads %.2f us, job planning %.2f us; "
                     "%.0f%% of waves ran the top-n select\n",
                     c.prof[20] / 1e3 / c.prof[9], c.prof[21] / 1e3 / c.prof[9], 100.0 * c.prof[22] / c.prof[9]);
    if (c.prof[22])
        std::fprintf(stderr, "[ghcm-prof] per top-n select: histogram %.2f us, scan %.2f us, gather %.2f us; "
                     "per wave, decision end to release %.2f us\n",
                     c.prof[24] / 1e3 / c.prof[22], c.prof[25] / 1e3 / c.prof[22], c.prof[26] / 1e3 / c.prof[22],
                     c.prof[27] / 1e3 / std::max(1ull, c.prof[9]));
    if (c.prof[13])
        std::fprintf(stderr, "[ghcm-prof] per CTA block-solve: stage %.2f us, sweeps %.2f us (%.3f us/sweep), "
                     "probe+commit+activate %.2f us\n",
                     c.prof[10] / 1e3 / c.prof[13], c.prof[11] / 1e3 / c.prof[13],
                     c.prof[11] / 1e3 / std::max(1ull, c.prof[3]), c.prof[12] / 1e3 / c.prof[13]);
#else
    (void)c;
    (void)grid;
#endif
}

// Scheduler parameters of a config on a device with `sms` SMs.
inline void fill_sched_params(Sched& s, const ghcm_config& cfg, int sms, uint32_t tiles) {
    uint32_t const B = cfg.block_size;
    s.max_jobs = cfg.max_jobs ? cfg.max_jobs : 8u * static_cast<uint32_t>(sms);
    if (s.max_jobs > tiles) s.max_jobs = tiles;
    s.key_mode = cfg.key_mode;
    s.max_sweeps = cfg.max_sweeps ? cfg.max_sweeps : 4u * B * B;
    s.max_waves = cfg.max_waves;
    s.eps = cfg.eps;
    bool const off = cfg.refresh_solves == GHCM_REFRESH_OFF;
    bool const in_only = cfg.refresh_solves == GHCM_REFRESH_IN_SOLVE;
    s.refresh = static_cast<uint16_t>(off || in_only ? 0u : (cfg.refresh_solves ? cfg.refresh_solves : kDefaultRefresh));
    s.in_solve = off ? 0u : 1u;
    s.learn.fallback_jobs = cfg.fallback_jobs ? cfg.fallback_jobs : s.max_jobs;
    s.timeout_ns = static_cast<uint64_t>(cfg.wait_timeout_ms ? cfg.wait_timeout_ms : 2000u) * 1000000ull;
}

}  // namespace ghcm

struct ghcm_ctx {
    ghcm_config cfg;
    int device = 0;
    int sms = 0;
    ghcm::LaunchInfo launch{};
    ghcm::LaunchInfo wide{};    // the build with more CTAs per SM for waves of many jobs (blocks_per_sm 0: none)
    ghcm::EncodeTiledFn encode = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
    // scheduler workspace: flags | key | tmin | list0 | list1 | jobs | ctl | insts
    ghcm::DevBuf ws;
    // field buffers used by ghcm_solve (host-pointer entry)
    ghcm::DevBuf d_in, d_time, d_seeds;
    // pinned staging for the instance record and the control block readback
    ghcm::Inst* h_inst = nullptr;
    ghcm::Ctl* h_ctl = nullptr;
    // learned schedule and trace recorder
    ghcm::DevBuf d_learn;          // per-tile learning arrays
    ghcm::DevBuf d_trace;          // trace records
    uint32_t trace_cap = 0;
    uint32_t trace_total = 0;      // records the last solve produced (may exceed trace_cap)
    ghcm::DevBuf d_model;          // MLP parameters
    bool has_model = false;
    float threshold = 0.5f;
    uint32_t policy = GHCM_POLICY_SCORE;
    uint32_t max_vetoes = 2;
    uint32_t counters[4] = {0, 0, 0, 0};
};

// Batches: many independent eikonal instances solved by one persistent launch.
//
// The reference solves one field per call (eikonal_hcm_opencl_ex,
// src/eikonal_hcm.cpp:186-529) and its harness calls it once per trial
// (src/test_runner.cpp:226-291). Small fields cannot fill a GPU: a 64 x 64
// field at block 16 has 16 tiles for 152 SMs. A batch gives the tiles of all
// its instances one global tile numbering (instance i owns the tiles
// [tile_base_i, tile_base_i + tiles_i)), one active set and one persistent
// grid; the device scheduler (ghcm_sched.cuh) and the tile solvers are the
// single-field ones, reading the instance of a tile from a per-tile index and
// its TMA tensor maps from a device table.
//
// The launch sequence - control-block reset, the two init kernels, the
// cooperative persistent kernel and the status readback into pinned memory -
// is captured once into a CUDA graph at ghcm_batch_create and replayed by
// ghcm_batch_run. If the capture is refused the batch launches the same
// sequence directly (ghcm_batch_info.graph = 0).
#include "ghcm_host.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

using namespace ghcm;

struct ghcm_batch {
    ghcm_config cfg{};
    int device = 0;
    int sms = 0;
    int grid = 0;
    LaunchInfo launch{};
    uint32_t count = 0;
    uint32_t tiles = 0;
    uint64_t cells = 0;
    uint64_t max_cells = 0;
    uint32_t max_seeds = 0;
    uint32_t tma_insts = 0;
    DevBuf ws;
    Sched s{};
    Ctl* h_ctl = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

int check_instance(const ghcm_instance& in) {
    if (!in.field || !in.time_out || in.width == 0 || in.height == 0) return GHCM_ERR_BAD_ARG;
    if (in.n_seeds && !in.seeds_xy) return GHCM_ERR_BAD_ARG;
    if (!(in.h > 0.f) || !std::isfinite(in.h) || in.reserved != 0u) return GHCM_ERR_BAD_ARG;
    if (in.width > kMaxSide || in.height > kMaxSide || static_cast<uint64_t>(in.width) * in.height > (1ull << 34))
        return GHCM_ERR_UNSUPPORTED;
    return GHCM_OK;
}

// The launch sequence of one solve of the batch on `st`.
cudaError_t enqueue(ghcm_batch* b, cudaStream_t st) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(b->s.ctl, 0, sizeof(Ctl), st)) != cudaSuccess) return e;
    if ((e = launch_init(b->s, b->count, b->max_cells, b->max_seeds, static_cast<int>(b->cfg.block_size), b->sms, st)) !=
        cudaSuccess)
        return e;
    if ((e = launch_persistent(static_cast<int>(b->cfg.block_size), b->cfg.kernel == GHCM_KERNEL_FIM, b->s, b->grid,
                               st, b->launch.wide)) != cudaSuccess)
        return e;
    return cudaMemcpyAsync(b->h_ctl, b->s.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st);
}

// Captures the launch sequence into b->exec; leaves the batch graph-less if
// the runtime refuses any step.
void capture(ghcm_batch* b) {
    cudaStream_t cs = nullptr;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    cudaGraph_t g = nullptr;
    bool ok = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
        cudaError_t const e = enqueue(b, cs);
        ok = cudaStreamEndCapture(cs, &g) == cudaSuccess && e == cudaSuccess && g != nullptr;
    }
    if (ok && cudaGraphInstantiate(&b->exec, g, 0) == cudaSuccess) {
        b->graph = g;
    } else {
        if (g) cudaGraphDestroy(g);
        b->exec = nullptr;
    }
    cudaGetLastError();
    cudaStreamDestroy(cs);
}

void destroy_batch(ghcm_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->ws.release();
    if (b->h_ctl) cudaFreeHost(b->h_ctl);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    delete b;
}

}  // namespace

extern "C" {

int ghcm_batch_create(ghcm_ctx* ctx, const ghcm_instance* insts, uint32_t count, ghcm_batch** out) {
    if (!out) return GHCM_ERR_BAD_ARG;
    *out = nullptr;
    if (!ctx || !insts || count == 0u) return GHCM_ERR_BAD_ARG;
    if (count > 65535u) return GHCM_ERR_UNSUPPORTED;
    uint32_t const B = ctx->cfg.block_size;
    std::vector<Inst> h(count);
    uint64_t tiles = 0, cells = 0, max_cells = 0;
    uint32_t max_seeds = 0;
    for (uint32_t i = 0; i < count; ++i) {
        int const rc = check_instance(insts[i]);
        if (rc != GHCM_OK) return rc;
        Inst& I = h[i];
        std::memset(&I, 0, sizeof(I));
        I.in = insts[i].field;
        I.time = insts[i].time_out;
        I.w = insts[i].width;
        I.h = insts[i].height;
        I.tiles_x = (I.w + B - 1) / B;
        I.tiles_y = (I.h + B - 1) / B;
        I.tile_base = static_cast<uint32_t>(tiles);
        I.spacing = insts[i].h;
        I.in_is_speed = insts[i].input_is_speed ? 1u : 0u;
        I.seeds = insts[i].seeds_xy;
        I.n_seeds = insts[i].n_seeds;
        I.cost_cap = cost_cap_of(ctx->cfg);
        tiles += static_cast<uint64_t>(I.tiles_x) * I.tiles_y;
        uint64_t const c = static_cast<uint64_t>(I.w) * I.h;
        cells += c;
        max_cells = std::max(max_cells, c);
        max_seeds = std::max(max_seeds, I.n_seeds);
        if (tiles >= (1ull << 31)) return GHCM_ERR_UNSUPPORTED;
    }
    bool const learned = ctx->cfg.schedule == GHCM_SCHEDULE_LEARNED;
    if (learned && !ctx->has_model) return GHCM_ERR_BAD_ARG;  // no schedule model set
    if (cudaSetDevice(ctx->device) != cudaSuccess) return GHCM_ERR_CUDA;

    ghcm_batch* b = new (std::nothrow) ghcm_batch();
    if (!b) return GHCM_ERR_OOM;
    b->cfg = ctx->cfg;
    b->device = ctx->device;
    b->sms = ctx->sms;
    if (query_persistent(static_cast<int>(ctx->cfg.block_size), ctx->cfg.kernel == GHCM_KERNEL_FIM, &b->launch, true) !=
            0 ||
        b->launch.blocks_per_sm <= 0)
        b->launch = ctx->launch;
    b->count = count;
    b->tiles = static_cast<uint32_t>(tiles);
    b->cells = cells;
    b->max_cells = max_cells;
    b->max_seeds = max_seeds;

    // tensor maps: instances whose rows and buffers are 16-byte aligned
    std::vector<CUtensorMap> maps(2u * count);
    std::memset(maps.data(), 0, maps.size() * sizeof(CUtensorMap));
    for (uint32_t i = 0; i < count && ctx->cfg.use_tma; ++i) {
        Inst& I = h[i];
        bool const aligned = (I.w % 4u == 0u) && (reinterpret_cast<uintptr_t>(I.in) % 16u == 0u) &&
                             (reinterpret_cast<uintptr_t>(I.time) % 16u == 0u);
        if (aligned && encode_tile_map(ctx->encode, &maps[2u * i], I.time, I.w, I.h, B) &&
            encode_tile_map(ctx->encode, &maps[2u * i + 1u], I.in, I.w, I.h, B)) {
            I.tma = 1;
            ++b->tma_insts;
        }
    }

    // workspace: flags | key | tmin | list0 | list1 | tile_inst | jobs | ctl | insts | maps
    Sched& s = b->s;
    std::memset(&s, 0, sizeof(s));
    s.num_tiles = b->tiles;
    s.num_insts = count;
    fill_sched_params(s, b->cfg, b->sms, b->tiles);
    b->grid = persistent_grid(b->launch, b->sms, s.max_jobs);
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t const at = o;
        o = align_up(o + bytes, 256);
        return at;
    };
    size_t const t4 = sizeof(uint32_t) * b->tiles;
    size_t const o_flags = take(t4), o_key = take(t4), o_tmin = take(t4), o_l0 = take(t4), o_l1 = take(t4);
    size_t const o_epoch = take(t4);
    size_t const o_ti = take(t4), o_jobs = take(sizeof(uint32_t) * std::max<uint32_t>(s.max_jobs, 1u));
    size_t const o_ctl = take(sizeof(Ctl)), o_insts = take(sizeof(Inst) * count);
    size_t const o_maps = take(sizeof(CUtensorMap) * 2u * count);
    size_t const o_learn = learned ? take(learn_bytes(b->tiles)) : 0;
    size_t const o_model = learned ? take(sizeof(float) * kParams) : 0;
    int rc = GHCM_OK;
    if (!b->ws.reserve(o)) rc = GHCM_ERR_OOM;
    if (rc == GHCM_OK && cudaMallocHost(reinterpret_cast<void**>(&b->h_ctl), sizeof(Ctl)) != cudaSuccess)
        rc = GHCM_ERR_OOM;
    if (rc == GHCM_OK && (cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess))
        rc = GHCM_ERR_CUDA;
    if (rc != GHCM_OK) {
        cudaGetLastError();
        destroy_batch(b);
        return rc;
    }
    char* base = b->ws.as<char>();
    s.flags = reinterpret_cast<uint32_t*>(base + o_flags);
    s.key = reinterpret_cast<uint32_t*>(base + o_key);
    s.tmin = reinterpret_cast<float*>(base + o_tmin);
    s.epoch = reinterpret_cast<uint32_t*>(base + o_epoch);
    s.list[0] = reinterpret_cast<uint32_t*>(base + o_l0);
    s.list[1] = reinterpret_cast<uint32_t*>(base + o_l1);
    s.tile_inst = reinterpret_cast<const uint32_t*>(base + o_ti);
    s.jobs = reinterpret_cast<uint32_t*>(base + o_jobs);
    s.ctl = reinterpret_cast<Ctl*>(base + o_ctl);
    s.insts = reinterpret_cast<const Inst*>(base + o_insts);
    s.maps = b->tma_insts ? reinterpret_cast<const CUtensorMap*>(base + o_maps) : nullptr;
    cudaError_t e = cudaSuccess;
    if (learned) {
        bind_learn_arrays(s.learn, base + o_learn, b->tiles);
        s.learn.params = reinterpret_cast<const float*>(base + o_model);
        s.learn.threshold = ctx->threshold;
        s.learn.veto = ctx->policy == GHCM_POLICY_VETO ? 1u : 0u;
        s.learn.max_vetoes = ctx->max_vetoes;
        e = cudaMemcpy(base + o_model, ctx->d_model.p, sizeof(float) * kParams, cudaMemcpyDeviceToDevice);
    }
    if (e == cudaSuccess) e = cudaMemcpy(base + o_insts, h.data(), sizeof(Inst) * count, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(base + o_maps, maps.data(), sizeof(CUtensorMap) * 2u * count, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        destroy_batch(b);
        return map_cuda(e);
    }
    capture(b);
    *out = b;
    return GHCM_OK;
}

int ghcm_batch_run(ghcm_batch* b, void* stream, ghcm_stats* stats) {
    if (!b) return GHCM_ERR_BAD_ARG;
    if (cudaSetDevice(b->device) != cudaSuccess) return GHCM_ERR_CUDA;
    auto const t0 = std::chrono::steady_clock::now();
    cudaStream_t const st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaEventRecord(b->ev0, st);
    if (e == cudaSuccess) e = b->exec ? cudaGraphLaunch(b->exec, st) : enqueue(b, st);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev1, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return map_cuda(e);
    Ctl const& c = *b->h_ctl;
    report_checks(c);
    print_profile(c, b->grid);
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, b->ev0, b->ev1);
        stats->block_solves = c.block_solves;
        stats->cells = b->cells;
        stats->bytes_alg = c.block_solves * static_cast<uint64_t>(bytes_per_solve(b->cfg.block_size));
        stats->waves = c.waves;
        stats->residual_passes = c.residual_passes;
        stats->max_active = c.max_active;
        stats->tiles = b->tiles;
        stats->device_ms = ms;
        stats->kernel_ms = ms;
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return status_from_error(c.error);
}

int ghcm_batch_query(const ghcm_batch* b, ghcm_batch_info* out) {
    if (!b || !out) return GHCM_ERR_BAD_ARG;
    std::memset(out, 0, sizeof(*out));
    out->instances = b->count;
    out->tiles = b->tiles;
    out->cells = b->cells;
    out->block_size = b->cfg.block_size;
    out->max_jobs = b->s.max_jobs;
    out->max_sweeps = b->s.max_sweeps;
    out->graph = b->exec ? 1u : 0u;
    out->grid = static_cast<uint32_t>(b->grid);
    out->tma_instances = b->tma_insts;
    return GHCM_OK;
}

int ghcm_batch_destroy(ghcm_batch* b) {
    destroy_batch(b);
    return GHCM_OK;
}

int ghcm_solve_batched(ghcm_ctx* ctx, const ghcm_instance* insts, uint32_t count, void* stream, ghcm_stats* stats) {
    ghcm_batch* b = nullptr;
    int rc = ghcm_batch_create(ctx, insts, count, &b);
    if (rc != GHCM_OK) return rc;
    rc = ghcm_batch_run(b, stream, stats);
    destroy_batch(b);
    return rc;
}

// Wave cap of one autotuner trial (a wave takes at least ~10 us, so a trial
// ends within seconds even on a config that would not converge).
constexpr uint32_t kTuneWaveCap = 200000u;

int ghcm_autotune_batch(const ghcm_config* base, const ghcm_instance* insts, uint32_t count, void* stream,
                        uint32_t reps, ghcm_config* best, ghcm_tune_trial* trials, uint32_t max_trials,
                        uint32_t* n_trials) {
    int rc = check_config(base);
    if (rc != GHCM_OK) return rc;
    if (!best || !insts || count == 0u) return GHCM_ERR_BAD_ARG;
    if (n_trials) *n_trials = 0;
    reps = std::max<uint32_t>(reps, 1u);
    uint32_t ran = 0;
    int sms = 0;
    {
        ghcm_ctx* probe = nullptr;
        if ((rc = ghcm_create(base, &probe)) != GHCM_OK) return rc;
        sms = probe->sms;
        ghcm_destroy(probe);
    }
    struct Pick {
        ghcm_config cfg;
        double ms;
        bool ok;
    } pick{*base, 0.0, false};

    // one trial: fresh context and batch, a warm-up replay, then the best of reps
    auto trial = [&](uint32_t B, uint32_t n, uint32_t sweeps, uint32_t kernel) {
        ghcm_config c = *base;
        c.block_size = B;
        c.max_jobs = n;
        c.max_sweeps = sweeps;
        c.kernel = kernel;
        // a trial may not run unbounded: a config that cannot finish fails with
        // GHCM_ERR_NOT_CONVERGED and is skipped
        if (c.max_waves == 0u) c.max_waves = kTuneWaveCap;
        ghcm_tune_trial t{B, n, sweeps, GHCM_OK, 0.0, 0ull, kernel, 0u};
        ghcm_ctx* ctx = nullptr;
        ghcm_batch* b = nullptr;
        int r = ghcm_create(&c, &ctx);
        if (r == GHCM_OK) r = ghcm_batch_create(ctx, insts, count, &b);
        ghcm_stats st{};
        if (r == GHCM_OK) r = ghcm_batch_run(b, stream, &st);
        double bestms = 0.0;
        for (uint32_t k = 0; k < reps && r == GHCM_OK; ++k) {
            r = ghcm_batch_run(b, stream, &st);
            if (k == 0 || st.device_ms < bestms) bestms = st.device_ms;
        }
        t.status = r;
        t.ms = bestms;
        t.block_solves = st.block_solves;
        if (b) ghcm_batch_destroy(b);
        if (ctx) ghcm_destroy(ctx);
        if (trials && ran < max_trials) trials[ran] = t;
        ++ran;
        if (r == GHCM_OK && (!pick.ok || bestms < pick.ms)) pick = Pick{c, bestms, true};
        return r;
    };

    // stage 1: tile size x n on a coarse grid; stage 2: n halved and doubled
    // around the best; stage 3: inner-sweep caps; stage 4: the other tile
    // kernel (systolic <-> block-FIM, data/eikonal_ghcm_fim.cl:214-392)
    uint32_t const S = static_cast<uint32_t>(sms);
    uint32_t const K = base->kernel;
    for (uint32_t B : {8u, 16u, 32u})
        for (uint32_t m : {4u, 16u, 64u}) trial(B, m * S, 0u, K);
    if (!pick.ok) {
        if (n_trials) *n_trials = ran;
        return GHCM_ERR_INTERNAL;
    }
    uint32_t const bB = pick.cfg.block_size;
    uint32_t const n1 = pick.cfg.max_jobs;
    for (uint32_t n : {n1 / 2u, n1 * 2u}) trial(bB, n, 0u, K);
    uint32_t const bN = pick.cfg.max_jobs;
    for (uint32_t sw : {bB / 2u, bB, 2u * bB}) trial(bB, bN, sw, K);
    trial(bB, bN, pick.cfg.max_sweeps, K == GHCM_KERNEL_FIM ? GHCM_KERNEL_SYSTOLIC : GHCM_KERNEL_FIM);
    // leave the fastest config's solve in the outputs
    ghcm_ctx* ctx = nullptr;
    rc = ghcm_create(&pick.cfg, &ctx);
    if (rc == GHCM_OK) rc = ghcm_solve_batched(ctx, insts, count, stream, nullptr);
    if (ctx) ghcm_destroy(ctx);
    *best = pick.cfg;
    best->max_waves = base->max_waves;
    if (n_trials) *n_trials = ran;
    return rc;
}

}  // extern "C"

// C-ABI layer of libghcm.so: contexts, device workspace, argument checks,
// tensor-map setup and the launch sequence of one solve.
//
// Replaces the host half of the reference's gHCM path:
//   eikonal_hcm_opencl_setup (src/eikonal_hcm.cpp:137-175) -> ghcm_create
//   eikonal_hcm_opencl_ex    (src/eikonal_hcm.cpp:186-529) -> ghcm_solve / ghcm_solve_device
// The reference's per-wave host loop (priority queue, job upload, blocking
// status read, neighbour activation) has no host counterpart here: it runs on
// the device inside one persistent kernel (ghcm_solver.cu).
#include "ghcm_host.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>

using namespace ghcm;

namespace ghcm {

int check_config(const ghcm_config* c) {
    if (!c) return GHCM_ERR_BAD_ARG;
    if (c->block_size != 8 && c->block_size != 16 && c->block_size != 32) return GHCM_ERR_BAD_ARG;
    if (c->kernel > GHCM_KERNEL_FIM || c->schedule > GHCM_SCHEDULE_LEARNED || c->key_mode > GHCM_KEY_BLOCK_MIN)
        return GHCM_ERR_BAD_ARG;
    if (!(c->eps >= 0.f) || !std::isfinite(c->eps)) return GHCM_ERR_BAD_ARG;
    if (!(c->cost_cap >= 0.f)) return GHCM_ERR_BAD_ARG;  // NaN or negative
    if (c->refresh_solves > kMaxRefresh && c->refresh_solves != GHCM_REFRESH_OFF &&
        c->refresh_solves != GHCM_REFRESH_IN_SOLVE)
        return GHCM_ERR_BAD_ARG;
    for (uint32_t r : c->reserved)
        if (r != 0) return GHCM_ERR_BAD_ARG;
    return GHCM_OK;
}

EncodeTiledFn tensor_map_encoder() {
    static EncodeTiledFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<EncodeTiledFn>(p);
        cudaGetLastError();
        return static_cast<EncodeTiledFn>(nullptr);
    }();
    return fn;
}

bool encode_tile_map(EncodeTiledFn encode, CUtensorMap* map, const float* base, uint32_t w, uint32_t h,
                     uint32_t block) {
    if (!encode) return false;
    cuuint64_t const dims[2] = {w, h};
    cuuint64_t const strides[1] = {static_cast<cuuint64_t>(w) * sizeof(float)};
    uint32_t bw = 0, bh = 0;
    tile_box(static_cast<int>(block), &bw, &bh);  // the tile with its halo, x from ox-4 (16-byte aligned)
    cuuint32_t const box[2] = {bw, bh};
    cuuint32_t const estr[2] = {1, 1};
    CUresult const r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace ghcm

namespace {

struct Layout {
    size_t flags, key, tmin, epoch, list0, list1, jobs, ctl, insts, total;
};

Layout layout_for(uint32_t tiles, uint32_t jobs) {
    Layout l{};
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t const at = o;
        o = align_up(o + bytes, 256);
        return at;
    };
    l.flags = take(sizeof(uint32_t) * tiles);
    l.key = take(sizeof(uint32_t) * tiles);
    l.tmin = take(sizeof(float) * tiles);
    l.epoch = take(sizeof(uint32_t) * tiles);
    l.list0 = take(sizeof(uint32_t) * tiles);
    l.list1 = take(sizeof(uint32_t) * tiles);
    l.jobs = take(sizeof(uint32_t) * std::max<uint32_t>(jobs, 1));
    l.ctl = take(sizeof(Ctl));
    l.insts = take(sizeof(Inst));
    l.total = o;
    return l;
}

int run_solve(ghcm_ctx* ctx, const float* d_field, int input_is_speed, uint32_t w, uint32_t h, float spacing,
              const uint32_t* d_seeds, uint32_t n_seeds, float* d_time, cudaStream_t st, ghcm_stats* stats) {
    uint32_t const B = ctx->cfg.block_size;
    if (w > kMaxSide || h > kMaxSide) return GHCM_ERR_UNSUPPORTED;
    uint32_t const tx = (w + B - 1) / B, ty = (h + B - 1) / B;  // no wrap: w, h <= kMaxSide
    uint64_t const tiles64 = static_cast<uint64_t>(tx) * ty;
    if (tiles64 >= (1ull << 31)) return GHCM_ERR_UNSUPPORTED;
    uint32_t const tiles = static_cast<uint32_t>(tiles64);
    uint32_t const max_jobs = ctx->cfg.max_jobs ? ctx->cfg.max_jobs : 8u * static_cast<uint32_t>(ctx->sms);
    uint32_t const jobs_cap = std::min(max_jobs, tiles);
    Layout const L = layout_for(tiles, jobs_cap);
    if (!ctx->ws.reserve(L.total)) return GHCM_ERR_OOM;
    char* base = ctx->ws.as<char>();

    Sched s;
    std::memset(&s, 0, sizeof(s));
    Inst& I = *ctx->h_inst;
    std::memset(&I, 0, sizeof(I));
    I.in = d_field;
    I.time = d_time;
    I.w = w;
    I.h = h;
    I.tiles_x = tx;
    I.tiles_y = ty;
    I.tile_base = 0;
    I.spacing = spacing;
    I.in_is_speed = input_is_speed ? 1u : 0u;
    I.seeds = d_seeds;
    I.n_seeds = n_seeds;
    I.cost_cap = cost_cap_of(ctx->cfg);
    bool const aligned = (w % 4u == 0u) && (reinterpret_cast<uintptr_t>(d_field) % 16u == 0u) &&
                         (reinterpret_cast<uintptr_t>(d_time) % 16u == 0u);
    I.tma = 0;
    if (ctx->cfg.use_tma && aligned && encode_tile_map(ctx->encode, &s.tmap_time, d_time, w, h, B) &&
        encode_tile_map(ctx->encode, &s.tmap_in, d_field, w, h, B))
        I.tma = 1;

    s.insts = reinterpret_cast<const Inst*>(base + L.insts);
    s.tile_inst = nullptr;
    s.flags = reinterpret_cast<uint32_t*>(base + L.flags);
    s.key = reinterpret_cast<uint32_t*>(base + L.key);
    s.tmin = reinterpret_cast<float*>(base + L.tmin);
    s.epoch = reinterpret_cast<uint32_t*>(base + L.epoch);
    s.list[0] = reinterpret_cast<uint32_t*>(base + L.list0);
    s.list[1] = reinterpret_cast<uint32_t*>(base + L.list1);
    s.jobs = reinterpret_cast<uint32_t*>(base + L.jobs);
    s.ctl = reinterpret_cast<Ctl*>(base + L.ctl);
    s.num_tiles = tiles;
    s.num_insts = 1;
    fill_sched_params(s, ctx->cfg, ctx->sms, tiles);
    bool const learned = ctx->cfg.schedule == GHCM_SCHEDULE_LEARNED;
    if (learned && !ctx->has_model) return GHCM_ERR_BAD_ARG;  // no schedule model set
    if (learned || ctx->trace_cap) {
        if (!ctx->d_learn.reserve(learn_bytes(tiles))) return GHCM_ERR_OOM;
        bind_learn_arrays(s.learn, ctx->d_learn.as<char>(), tiles);
        if (learned) {
            s.learn.params = ctx->d_model.as<float>();
            s.learn.threshold = ctx->threshold;
            s.learn.veto = ctx->policy == GHCM_POLICY_VETO ? 1u : 0u;
            s.learn.max_vetoes = ctx->max_vetoes;
        }
        if (ctx->trace_cap) {
            s.learn.trace = ctx->d_trace.as<TraceRec>();
            s.learn.trace_cap = ctx->trace_cap;
        }
    }

    cudaError_t e;
    if ((e = cudaMemcpyAsync(base + L.insts, &I, sizeof(Inst), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return map_cuda(e);
    if ((e = cudaMemsetAsync(s.ctl, 0, sizeof(Ctl), st)) != cudaSuccess) return map_cuda(e);
    cudaEventRecord(ctx->ev0, st);
    if ((e = launch_init(s, 1, static_cast<uint64_t>(w) * h, n_seeds, static_cast<int>(B), ctx->sms, st)) != cudaSuccess)
        return map_cuda(e);
    // the wide build for waves of many jobs. A learned schedule's waves hold
    // at least its fill (fallback_jobs) and up to max_jobs: it goes wide only
    // when the fill alone is that large (on the 4096^2 noise field, cap 4096
    // and fill 1024, its scoring ran 7.2 ms on the 4-CTA build against 9.0 ms
    // on the wide one)
    uint32_t const wide_jobs = learned ? s.learn.fallback_jobs : s.max_jobs;
    bool const wide = wide_for(ctx->launch, ctx->sms, wide_jobs) && ctx->wide.blocks_per_sm > 0;
    LaunchInfo const& li = wide ? ctx->wide : ctx->launch;
    int const grid = persistent_grid(li, ctx->sms, s.max_jobs);
    cudaEventRecord(ctx->ev2, st);
    if ((e = launch_persistent(static_cast<int>(B), ctx->cfg.kernel == GHCM_KERNEL_FIM, s, grid, st, li.wide)) != cudaSuccess)
        return map_cuda(e);
    cudaEventRecord(ctx->ev1, st);
    if ((e = cudaMemcpyAsync(ctx->h_ctl, s.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return map_cuda(e);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return map_cuda(e);

    Ctl const& c = *ctx->h_ctl;
    ctx->trace_total = c.trace_count;
    ctx->counters[0] = c.score_waves;
    ctx->counters[1] = c.fallback_waves;
    ctx->counters[2] = c.trace_count;
    ctx->counters[3] = c.vetoes;
    report_checks(c);
    print_profile(c, grid);
    if (stats) {
        float ms = 0.f, kms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        cudaEventElapsedTime(&kms, ctx->ev2, ctx->ev1);
        stats->kernel_ms = kms;
        stats->block_solves = c.block_solves;
        stats->cells = static_cast<uint64_t>(w) * h;
        stats->bytes_alg = c.block_solves * static_cast<uint64_t>(bytes_per_solve(B));
        stats->waves = c.waves;
        stats->residual_passes = c.residual_passes;
        stats->max_active = c.max_active;
        stats->tiles = tiles;
        stats->device_ms = ms;
    }
    return status_from_error(c.error);
}

int check_field_args(ghcm_ctx* ctx, const void* field, uint32_t w, uint32_t h, float spacing, const void* seeds,
                     uint32_t n_seeds, const void* out) {
    if (!ctx || !field || !out || w == 0 || h == 0) return GHCM_ERR_BAD_ARG;
    if (n_seeds && !seeds) return GHCM_ERR_BAD_ARG;
    if (!(spacing > 0.f) || !std::isfinite(spacing)) return GHCM_ERR_BAD_ARG;
    if (w > kMaxSide || h > kMaxSide || static_cast<uint64_t>(w) * h > (1ull << 34)) return GHCM_ERR_UNSUPPORTED;
    return GHCM_OK;
}

}  // namespace

extern "C" {

int ghcm_abi_version(void) { return GHCM_ABI_VERSION; }

const char* ghcm_status_string(int status) {
    switch (status) {
        case GHCM_OK: return "ok";
        case GHCM_ERR_BAD_ARG: return "bad argument";
        case GHCM_ERR_BAD_INPUT: return "input field holds a NaN or negative value";
        case GHCM_ERR_OOM: return "out of memory";
        case GHCM_ERR_CUDA: return "CUDA error";
        case GHCM_ERR_TIMEOUT: return "a bounded device wait timed out";
        case GHCM_ERR_NOT_CONVERGED: return "wave cap reached before convergence";
        case GHCM_ERR_UNSUPPORTED: return "unsupported device or size";
        case GHCM_ERR_INTERNAL: return "internal error";
        case GHCM_ERR_TOO_LARGE: return "field exceeds the no-alloc scratch limit (GHCM_NOALLOC_MAX_TILES tiles)";
        default: return "unknown status";
    }
}

int ghcm_config_default(ghcm_config* cfg) {
    if (!cfg) return GHCM_ERR_BAD_ARG;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->block_size = 16;
    cfg->max_jobs = 0;
    cfg->eps = 1e-5f;
    cfg->kernel = GHCM_KERNEL_SYSTOLIC;
    cfg->schedule = GHCM_SCHEDULE_PLAIN;
    cfg->key_mode = GHCM_KEY_BOUNDARY_MIN;
    cfg->max_sweeps = 0;
    cfg->max_waves = 0;
    cfg->wait_timeout_ms = 2000;
    cfg->device = -1;
    cfg->use_tma = 1;
    return GHCM_OK;
}

int ghcm_create(const ghcm_config* cfg, ghcm_ctx** out) {
    if (!out) return GHCM_ERR_BAD_ARG;
    *out = nullptr;
    int rc = check_config(cfg);
    if (rc != GHCM_OK) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return GHCM_ERR_UNSUPPORTED;
    }
    int dev = cfg->device;
    if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) return GHCM_ERR_CUDA;
    if (dev >= ndev) return GHCM_ERR_BAD_ARG;
    if (cudaSetDevice(dev) != cudaSuccess) return GHCM_ERR_CUDA;
    int coop = 0, sms = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (!coop || sms <= 0) return GHCM_ERR_UNSUPPORTED;

    ghcm_ctx* ctx = new (std::nothrow) ghcm_ctx();
    if (!ctx) return GHCM_ERR_OOM;
    ctx->cfg = *cfg;
    ctx->device = dev;
    ctx->sms = sms;
    if (query_persistent(static_cast<int>(cfg->block_size), cfg->kernel == GHCM_KERNEL_FIM, &ctx->wide, true) != 0)
        ctx->wide.blocks_per_sm = 0;  // no wide build: every solve uses ctx->launch
    if (query_persistent(static_cast<int>(cfg->block_size), cfg->kernel == GHCM_KERNEL_FIM, &ctx->launch) != 0 ||
        ctx->launch.blocks_per_sm <= 0) {
        delete ctx;
        return GHCM_ERR_UNSUPPORTED;
    }
    ctx->encode = tensor_map_encoder();
    if (cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
        cudaEventCreate(&ctx->ev2) != cudaSuccess ||
        cudaMallocHost(reinterpret_cast<void**>(&ctx->h_inst), sizeof(Inst)) != cudaSuccess ||
        cudaMallocHost(reinterpret_cast<void**>(&ctx->h_ctl), sizeof(Ctl)) != cudaSuccess) {
        ghcm_destroy(ctx);
        return GHCM_ERR_OOM;
    }
    *out = ctx;
    return GHCM_OK;
}

int ghcm_destroy(ghcm_ctx* ctx) {
    if (!ctx) return GHCM_OK;
    cudaSetDevice(ctx->device);
    ctx->ws.release();
    ctx->d_in.release();
    ctx->d_time.release();
    ctx->d_seeds.release();
    ctx->d_learn.release();
    ctx->d_trace.release();
    ctx->d_model.release();
    if (ctx->h_inst) cudaFreeHost(ctx->h_inst);
    if (ctx->h_ctl) cudaFreeHost(ctx->h_ctl);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->ev2) cudaEventDestroy(ctx->ev2);
    delete ctx;
    return GHCM_OK;
}

int ghcm_device_sm_count(const ghcm_ctx* ctx, uint32_t* out) {
    if (!ctx || !out) return GHCM_ERR_BAD_ARG;
    *out = static_cast<uint32_t>(ctx->sms);
    return GHCM_OK;
}

int ghcm_solve_device(ghcm_ctx* ctx, const float* d_field, int input_is_speed, uint32_t width, uint32_t height,
                      float h, const uint32_t* d_seeds_xy, uint32_t n_seeds, float* d_time_out, void* stream,
                      ghcm_stats* stats) {
    int rc = check_field_args(ctx, d_field, width, height, h, d_seeds_xy, n_seeds, d_time_out);
    if (rc != GHCM_OK) return rc;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return GHCM_ERR_CUDA;
    auto const t0 = std::chrono::steady_clock::now();
    rc = run_solve(ctx, d_field, input_is_speed, width, height, h, d_seeds_xy, n_seeds, d_time_out,
                   static_cast<cudaStream_t>(stream), stats);
    if (stats) stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

int ghcm_solve(ghcm_ctx* ctx, const float* field, int input_is_speed, uint32_t width, uint32_t height, float h,
               const uint32_t* seeds_xy, uint32_t n_seeds, float* time_out, ghcm_stats* stats) {
    int rc = check_field_args(ctx, field, width, height, h, seeds_xy, n_seeds, time_out);
    if (rc != GHCM_OK) return rc;
    for (uint32_t i = 0; i < n_seeds; ++i)
        if (seeds_xy[2 * i] >= width || seeds_xy[2 * i + 1] >= height) return GHCM_ERR_BAD_ARG;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return GHCM_ERR_CUDA;
    auto const t0 = std::chrono::steady_clock::now();
    size_t const bytes = static_cast<size_t>(width) * height * sizeof(float);
    if (!ctx->d_in.reserve(bytes) || !ctx->d_time.reserve(bytes) ||
        !ctx->d_seeds.reserve(std::max<size_t>(8, 8ull * n_seeds)))
        return GHCM_ERR_OOM;
    cudaStream_t const st = nullptr;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(ctx->d_in.p, field, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return map_cuda(e);
    if (n_seeds &&
        (e = cudaMemcpyAsync(ctx->d_seeds.p, seeds_xy, 8ull * n_seeds, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return map_cuda(e);
    rc = run_solve(ctx, ctx->d_in.as<float>(), input_is_speed, width, height, h, ctx->d_seeds.as<uint32_t>(),
                   n_seeds, ctx->d_time.as<float>(), st, stats);
    if (rc == GHCM_OK || rc == GHCM_ERR_NOT_CONVERGED) {
        if ((e = cudaMemcpy(time_out, ctx->d_time.p, bytes, cudaMemcpyDeviceToHost)) != cudaSuccess)
            return map_cuda(e);
    }
    if (stats) stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

int ghcm_trace_enable(ghcm_ctx* ctx, uint32_t capacity) {
    if (!ctx) return GHCM_ERR_BAD_ARG;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return GHCM_ERR_CUDA;
    if (capacity == 0u) {
        ctx->d_trace.release();
        ctx->trace_cap = 0u;
        return GHCM_OK;
    }
    if (!ctx->d_trace.reserve(static_cast<size_t>(capacity) * sizeof(TraceRec))) return GHCM_ERR_OOM;
    ctx->trace_cap = capacity;
    ctx->trace_total = 0u;
    return GHCM_OK;
}

int ghcm_trace_read(ghcm_ctx* ctx, ghcm_trace_record* out, uint32_t max_records, uint32_t* n_records,
                    uint32_t* n_total) {
    if (!ctx || !n_records || (max_records && !out)) return GHCM_ERR_BAD_ARG;
    uint32_t const have = std::min(ctx->trace_total, ctx->trace_cap);
    uint32_t const n = std::min(have, max_records);
    *n_records = 0u;
    if (n_total) *n_total = ctx->trace_total;
    if (n == 0u) return GHCM_OK;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return GHCM_ERR_CUDA;
    cudaError_t const e = cudaMemcpy(out, ctx->d_trace.p, static_cast<size_t>(n) * sizeof(TraceRec),
                                     cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return map_cuda(e);
    *n_records = n;
    return GHCM_OK;
}

int ghcm_set_schedule_model(ghcm_ctx* ctx, const float* params, uint32_t n_params, float threshold) {
    if (!ctx) return GHCM_ERR_BAD_ARG;
    if (!params) {
        ctx->has_model = false;
        return GHCM_OK;
    }
    if (n_params != GHCM_MLP_PARAMS || !(threshold > 0.f && threshold < 1.f)) return GHCM_ERR_BAD_ARG;
    for (uint32_t i = 0; i < n_params; ++i)
        if (!std::isfinite(params[i])) return GHCM_ERR_BAD_ARG;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return GHCM_ERR_CUDA;
    if (!ctx->d_model.reserve(sizeof(float) * GHCM_MLP_PARAMS)) return GHCM_ERR_OOM;
    cudaError_t const e = cudaMemcpy(ctx->d_model.p, params, sizeof(float) * GHCM_MLP_PARAMS, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return map_cuda(e);
    ctx->has_model = true;
    ctx->threshold = threshold;
    return GHCM_OK;
}

int ghcm_set_schedule_policy(ghcm_ctx* ctx, uint32_t policy, uint32_t max_vetoes) {
    if (!ctx || policy > GHCM_POLICY_VETO || max_vetoes > 1000u) return GHCM_ERR_BAD_ARG;
    ctx->policy = policy;
    ctx->max_vetoes = max_vetoes ? max_vetoes : 2u;
    return GHCM_OK;
}

int ghcm_schedule_counters(const ghcm_ctx* ctx, uint32_t out[4]) {
    if (!ctx || !out) return GHCM_ERR_BAD_ARG;
    for (int i = 0; i < 4; ++i) out[i] = ctx->counters[i];
    return GHCM_OK;
}

int ghcm_selftest_wait_timeout(ghcm_ctx* ctx, uint32_t timeout_ms) {
    if (!ctx || timeout_ms == 0 || timeout_ms > 60000) return GHCM_ERR_BAD_ARG;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return GHCM_ERR_CUDA;
    DevBuf buf;
    if (!buf.reserve(align_up(sizeof(Ctl), 256) + 256)) return GHCM_ERR_OOM;
    Ctl* ctl = buf.as<Ctl>();
    uint32_t* flag = reinterpret_cast<uint32_t*>(buf.as<char>() + align_up(sizeof(Ctl), 256));
    cudaError_t e = cudaMemset(buf.p, 0, buf.bytes);
    if (e == cudaSuccess) e = launch_wait_selftest(flag, ctl, static_cast<uint64_t>(timeout_ms) * 1000000ull, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    Ctl host{};
    if (e == cudaSuccess) e = cudaMemcpy(&host, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost);
    buf.release();
    if (e != cudaSuccess) return map_cuda(e);
    return (host.error & kErrTimeout) ? GHCM_ERR_TIMEOUT : GHCM_OK;
}

int ghcm_selftest_sqrt(ghcm_ctx* ctx, unsigned long long* mismatches) {
    if (!ctx || !mismatches) return GHCM_ERR_BAD_ARG;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return GHCM_ERR_CUDA;
    DevBuf buf;
    if (!buf.reserve(256)) return GHCM_ERR_OOM;
    unsigned long long* d_count = buf.as<unsigned long long>();
    cudaError_t e = cudaMemset(d_count, 0, sizeof(*d_count));
    if (e == cudaSuccess) e = launch_sqrt_selftest(d_count, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(mismatches, d_count, sizeof(*d_count), cudaMemcpyDeviceToHost);
    buf.release();
    return e == cudaSuccess ? GHCM_OK : map_cuda(e);
}

}  // extern "C"

// The gHCM block eikonal solve on the device.
//
// One persistent, co-resident grid (a few CTAs per SM, each CTA a tile
// worker) runs the whole solve; the host only launches it:
//
//   wave loop (replaces the host loop of src/eikonal_hcm.cpp:343-482)
//     barrier  every CTA arrives; the last to arrive picks the n active tiles
//              with the smallest keys (a histogram select over the keys:
//              the device form of the priority-queue pop,
//              src/eikonal_hcm.cpp:344-358) and releases the grid;
//     solve    each CTA takes jobs in turn: stages the tile plus a two-cell
//              halo into shared memory (TMA when the field allows it), solves
//              it to convergence, probes the four neighbour edge rows, writes
//              the tile back and activates the neighbours that would improve
//              (src/eikonal_hcm.cpp:434-469);
//   when no tile is active, a global Godunov residual pass over every cell
//   re-activates any tile not at the fixed point; the solve ends when that
//   pass activates nothing. The reference has no such check
//   (src/eikonal_hcm.cpp:343, 486-488).
//
// Every wait (grid barrier, TMA completion) is bounded by Sched::timeout_ns.
#include "ghcm_device.cuh"
#include "ghcm_internal.h"

// GHCM_PROFILE builds accumulate per-phase times (thread 0 of each CTA) into
// Ctl::prof: [0] barrier waits, [1] solve phases, [3] sweeps, [4] residual
// phases, [5] kernel wall time (CTA 0). They change no result.
#ifdef GHCM_PROFILE
#define GHCM_PROF_BEGIN(var) uint64_t var = (threadIdx.x == 0) ? global_ns() : 0ull
#define GHCM_PROF_END(ctl, idx, var) \
    if (threadIdx.x == 0) atomicAdd(&(ctl)->prof[idx], static_cast<unsigned long long>(global_ns() - (var)))
#define GHCM_PROF_COUNT(ctl, idx, n) \
    if (threadIdx.x == 0) atomicAdd(&(ctl)->prof[idx], static_cast<unsigned long long>(n))
#else
#define GHCM_PROF_BEGIN(var)
#define GHCM_PROF_END(ctl, idx, var)
#define GHCM_PROF_COUNT(ctl, idx, n)
#endif

#include "ghcm_tile.cuh"
#include "ghcm_warp_tile.cuh"

#include <algorithm>

namespace ghcm {

// CTAs per SM for the persistent grid: more CTAs keep more tiles in flight,
// fewer make the per-wave grid barrier cheaper.
template <int B>
constexpr int max_ctas_per_sm() {
    return B == 8 ? 12 : 4;
}

// Systolic B=16 and B=32 tiles also have a build for 8 CTAs per SM (32
// registers a thread, a few spills outside the sweep loop) for waves that hold
// many jobs per CTA: batches, and single fields whose n is more than twice the
// 4-CTA grid (wide_for). The extra tiles in flight per SM took a 512-instance
// batch from 29.5 to 27.4 ms at B=16 and from 32.1 to 28.2 ms at B=32, the
// 16384^2 maze (B=32, n=4096) from 98.5 to 95.5 ms and the 4096^2 rings at
// n=4096 from 19.7 to 19.0 ms. With fewer jobs per CTA the smaller register
// budget costs more than the extra tiles bring (rings at n=256: 13.8 -> 14.4
// ms, at n=1024: 16.2 -> 16.5 ms), so those keep the 4-CTA build.
constexpr int kWideCtas = 8;

// List entries per thread the top-n select keeps in registers between its
// passes (ids and bins; a list of up to 256 x this many is read once): 7 in
// the 64-register systolic builds of tiles of 16 (8 spills), 6 in the other
// 64-register builds, 4 in the 32-register wide builds.
template <int B, bool FIM, int CTAS>
__host__ __device__ constexpr int select_regs() {
    return CTAS > 4 ? 4 : ((FIM || B == 32) ? 6 : 7);
}

template <int B, bool FIM, int CTAS = max_ctas_per_sm<B>()>
__global__ void __launch_bounds__(TileGeom<B>::THREADS, CTAS) k_solve(const __grid_constant__ Sched s) {
    using G = TileGeom<B>;
    __shared__ TileSmem<B> sm;
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ uint32_t s_hist[SELECT_BINS];
    __shared__ uint32_t s_sel[16];
    __shared__ uint32_t s_state[8];
    __shared__ uint32_t s_word[8];
    __shared__ float s_red[G::THREADS / 32];
    __shared__ uint32_t s_krange[2];
    int const tid = threadIdx.x;
    Ctl* ctl = s.ctl;
    if (ld_relaxed(&ctl->error) != 0u) return;  // the init kernels rejected the input

    if (tid == 0) mbar_init(&s_bar, 1);
    if (FIM)
        for (int i = tid; i < B * B; i += G::THREADS) sm.check[i] = 0;
    if (tid < 8) s_state[tid] = 0u;  // INIT, generation 0, no waves yet
    if (tid == 0) {
        s_krange[0] = inf_bits();  // keys this CTA activates in a phase: {min, max}
        s_krange[1] = 0u;
    }
    if (s.learn.params)  // learned schedule: the model in shared memory for scoring
        for (int i = tid; i < kParams; i += G::THREADS) g_mlp_params[i] = __ldg(&s.learn.params[i]);
    __shared__ uint32_t s_slot[2];
    if (tid == 0) sm_enter(ctl, s_slot);
    __syncthreads();
    GHCM_PROF_BEGIN(t_kernel);
    uint32_t parity = 0u;
    bool tma_pending = false;
    unsigned long long solves = 0ull;
    uint32_t const warps_per_cta = G::THREADS / 32;
    uint32_t const gw = blockIdx.x * warps_per_cta + static_cast<uint32_t>(tid >> 5);
    uint32_t const nwarps = gridDim.x * warps_per_cta;
    uint32_t rank = blockIdx.x;
    bool ranked = false;
    for (;;) {
        GHCM_PROF_BEGIN(t_bar);
        bool const ok = wave_barrier<G::THREADS, select_regs<B, FIM, CTAS>()>(s, s_hist, s_sel, s_state, s_krange);
        GHCM_PROF_END(ctl, 0, t_bar);
        if (!ok) break;
        if (!ranked) {  // the first barrier follows every CTA's sm_enter
            rank = sm_rank<G::THREADS>(ctl, s_slot, reinterpret_cast<uint32_t*>(s_red));
            ranked = true;
        }
        uint32_t const phase = s_state[kStPhase];
        uint32_t const cur = s_state[kStCur];
        if (phase == kPhaseJobs) {
            GHCM_PROF_BEGIN(t_solve);
            uint32_t const nj = s_state[kStJobs];
            uint32_t const wave = s_state[kStWaves];
            const uint32_t* jobs = s_state[kStInList] ? s.list[cur] : s.jobs;
#ifdef GHCM_PROFILE
            if (tid == 0 && rank < nj) {  // the latest first-job start of the wave
                unsigned long long const rel = ld_relaxed_u64(&ctl->release_ns);
                atomicMax(&ctl->prof[16], static_cast<unsigned long long>(global_ns() - rel));
            }
#endif
            for (uint32_t j = rank; j < nj; j += gridDim.x) {
                uint32_t const job = __ldcg(&jobs[j]);
                if (job >= s.num_tiles) {  // never written by a correct decision: stop the grid
                    if (tid == 0) atomicOr(&ctl->error, kErrInternal);
                    break;
                }
                int const r = solve_tile<B, FIM, (CTAS <= 4)>(s, job, cur ^ 1u, sm, &s_bar, parity, tma_pending, s_word,
                                                              s_red, s_krange, wave, s_state[kStResid] + 1u,
                                                              act_phase_bit(s_state[kStGen]));
                if (r == kJobFailed) break;
                solves += (r == kJobSolved) ? 1u : 0u;
            }
#ifdef GHCM_PROFILE
            if (tid == 0 && rank < nj) {  // the latest job end of the wave
                unsigned long long const rel = ld_relaxed_u64(&ctl->release_ns);
                atomicMax(&ctl->prof[14], static_cast<unsigned long long>(global_ns() - rel));
            }
#endif
            GHCM_PROF_END(ctl, 1, t_solve);
        } else if (phase == kPhaseResidual) {
            GHCM_PROF_BEGIN(t_res);
            residual_warp<B>(s, cur ^ 1u, gw, nwarps, s_krange, s_state[kStResid]);
            GHCM_PROF_END(ctl, 4, t_res);
        } else {
            break;  // done or stopped
        }
    }
    if (tid == 0 && solves) atomicAdd(&ctl->block_solves, solves);
    if (blockIdx.x == 0) {
        GHCM_PROF_END(ctl, 5, t_kernel);
    }
    // A TMA copy still in flight after a timed-out wait: give it a bounded
    // chance to land before the CTA's shared memory is released.
    if (tid == 0 && tma_pending) (void)mbar_wait(&s_bar, parity ^ 1u, s.timeout_ns);
}

// The same wave loop with one warp per tile (systolic, B = 8 or 16).
template <int B>
__global__ void __launch_bounds__(WarpTileGeom<B>::THREADS, 3) k_solve_warp(const __grid_constant__ Sched s) {
    using W = WarpTileGeom<B>;
    __shared__ WarpTileSmem<B> wsm[W::NW];
    __shared__ uint32_t s_hist[SELECT_BINS];
    __shared__ uint32_t s_sel[16];
    __shared__ uint32_t s_state[8];
    __shared__ uint32_t s_krange[2];
    int const tid = threadIdx.x;
    int const warp = tid >> 5;
    int const lane = tid & 31;
    WarpTileSmem<B>& sm = wsm[warp];
    Ctl* ctl = s.ctl;
    if (ld_relaxed(&ctl->error) != 0u) return;  // the init kernels rejected the input

    if (lane == 0) mbar_init(&sm.bar, 1);
    if (tid < 8) s_state[tid] = 0u;  // INIT, generation 0, no waves yet
    if (tid == 0) {
        s_krange[0] = inf_bits();
        s_krange[1] = 0u;
    }
    if (s.learn.params)
        for (int i = tid; i < kParams; i += W::THREADS) g_mlp_params[i] = __ldg(&s.learn.params[i]);
    __shared__ uint32_t s_slot[2];
    __shared__ uint32_t s_tmp[W::NW];
    if (tid == 0) sm_enter(ctl, s_slot);
    __syncthreads();
    GHCM_PROF_BEGIN(t_kernel);
    uint32_t parity = 0u;
    bool tma_pending = false;
    unsigned long long solves = 0ull;
    uint32_t const gw = blockIdx.x * W::NW + static_cast<uint32_t>(warp);
    uint32_t const nwarps = gridDim.x * W::NW;
    uint32_t worker = gw;  // job order: warp 0 of every CTA (by SM rank) first, then warp 1, ...
    bool ranked = false;
    for (;;) {
        GHCM_PROF_BEGIN(t_bar);
        bool const ok = wave_barrier<W::THREADS, 8>(s, s_hist, s_sel, s_state, s_krange);
        GHCM_PROF_END(ctl, 0, t_bar);
        if (!ok) break;
        if (!ranked) {
            worker = static_cast<uint32_t>(warp) * gridDim.x + sm_rank<W::THREADS>(ctl, s_slot, s_tmp);
            ranked = true;
        }
        uint32_t const phase = s_state[kStPhase];
        uint32_t const cur = s_state[kStCur];
        if (phase == kPhaseJobs) {
            GHCM_PROF_BEGIN(t_solve);
            uint32_t const nj = s_state[kStJobs];
            uint32_t const wave = s_state[kStWaves];
            const uint32_t* jobs = s_state[kStInList] ? s.list[cur] : s.jobs;
            for (uint32_t j = worker; j < nj; j += nwarps) {
                uint32_t const job = __ldcg(&jobs[j]);
                if (job >= s.num_tiles) {
                    if (lane == 0) atomicOr(&ctl->error, kErrInternal);
                    break;
                }
                int const r = solve_tile_warp<B>(s, job, cur ^ 1u, sm, parity, tma_pending, s_krange, wave,
                                                 s_state[kStResid] + 1u, act_phase_bit(s_state[kStGen]));
                if (r == kJobFailed) break;
                solves += (r == kJobSolved) ? 1u : 0u;
            }
            GHCM_PROF_END(ctl, 1, t_solve);
        } else if (phase == kPhaseResidual) {
            GHCM_PROF_BEGIN(t_res);
            residual_warp<B>(s, cur ^ 1u, gw, nwarps, s_krange, s_state[kStResid]);
            GHCM_PROF_END(ctl, 4, t_res);
        } else {
            break;  // done or stopped
        }
    }
    if (lane == 0 && solves) atomicAdd(&ctl->block_solves, solves);
    if (blockIdx.x == 0) {
        GHCM_PROF_END(ctl, 5, t_kernel);
    }
    if (lane == 0 && tma_pending) (void)mbar_wait(&sm.bar, parity ^ 1u, s.timeout_ns);
}

// ---------------------------------------------------------------------------
// Initialisation kernels (src/eikonal_hcm.cpp:189-238). blockIdx.y is the
// instance; a single solve is a batch of one.
// ---------------------------------------------------------------------------

// Per-tile scheduler state and instance index, time = +inf everywhere; rejects
// NaN or negative inputs.
__global__ void k_init_inst(Sched s) {
    Inst const I = s.insts[blockIdx.y];
    uint32_t const stride = gridDim.x * blockDim.x;
    uint32_t const first = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t const n_tiles = I.tiles_x * I.tiles_y;
    for (uint32_t t = first; t < n_tiles; t += stride) {
        uint32_t const g = I.tile_base + t;
        s.flags[g] = 0u;
        s.epoch[g] = 0u;
        s.key[g] = inf_bits();
        s.tmin[g] = f_inf();
        if (s.tile_inst) const_cast<uint32_t*>(s.tile_inst)[g] = blockIdx.y;
        if (s.learn.tstat) {
            s.learn.kmax[g] = 0u;
            s.learn.nsolve[g] = 0u;
            s.learn.last_change[g] = 0u;
            s.learn.vetoes[g] = 0u;
        }
    }
    size_t const n = static_cast<size_t>(I.w) * I.h;
    bool bad = false;
    for (size_t i = first; i < n; i += stride) {
        float const v = __ldg(&I.in[i]);
        bad |= !(v >= 0.f);
        I.time[i] = f_inf();
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&s.ctl->error, kErrBadInput);
}

// Seeds: time 0, and the tiles of their 4-neighbours become active with key 0
// (seed_map and the initial heap, src/eikonal_hcm.cpp:198-238).
__global__ void k_init_seeds(Sched s, int block) {
    constexpr int dir[4][2] = {{-1, 0}, {0, -1}, {1, 0}, {0, 1}};
    Inst const I = s.insts[blockIdx.y];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < I.n_seeds; i += gridDim.x * blockDim.x) {
        uint32_t const ux = I.seeds[2 * i], uy = I.seeds[2 * i + 1];
        if (ux >= I.w || uy >= I.h) {
            atomicOr(&s.ctl->error, kErrBadSeed);
            continue;
        }
        I.time[static_cast<size_t>(uy) * I.w + ux] = 0.f;
        int const x = static_cast<int>(ux), y = static_cast<int>(uy);
        for (auto const& d : dir) {
            int const px = x + d[0], py = y + d[1];
            if (px < 0 || py < 0 || px >= static_cast<int>(I.w) || py >= static_cast<int>(I.h)) continue;
            uint32_t const tile = I.tile_base + static_cast<uint32_t>(py / block) * I.tiles_x + px / block;
            s.tmin[tile] = 0.f;
            activate(s, tile, 0u, 0.f, 0u, nullptr, 0u);  // key range of list 0: {0, 0} from the zeroed Ctl
        }
    }
}

// Per-tile speed statistics for the learned features, one warp per tile.
template <int B>
__global__ void k_tile_stats(Sched s) {
    uint32_t const warps = gridDim.x * (blockDim.x / 32);
    for (uint32_t t = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); t < s.num_tiles; t += warps)
        tile_speed_stats<B>(s, t);
}

__global__ void k_wait_selftest(const uint32_t* flag, Ctl* ctl, uint64_t timeout_ns) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint64_t const t0 = global_ns();
    while (ld_acquire(flag) == 0u) {
        __nanosleep(1000);
        if (global_ns() - t0 > timeout_ns) {
            atomicOr(&ctl->error, kErrTimeout);
            return;
        }
    }
}

// Every 32-bit pattern from `base` on (one per thread) through sqrt_rn and
// through __fsqrt_rn, and those in [2^-100, +inf) also through
// sqrt_rn_normal; adds the number of inputs whose results differ (NaN results
// compare equal) to *mismatches.
__global__ void k_sqrt_selftest(uint32_t base, unsigned long long* mismatches) {
    uint32_t const i = base + blockIdx.x * blockDim.x + threadIdx.x;
    float const a = __uint_as_float(i);
    float const r = sqrt_rn(a), e = __fsqrt_rn(a);
    bool same = __float_as_uint(r) == __float_as_uint(e) || (isnan(r) && isnan(e));
    if (a >= 0x1p-100f && a < f_inf()) same &= __float_as_uint(sqrt_rn_normal(a)) == __float_as_uint(e);
    int const bad = __syncthreads_count(!same);
    if (threadIdx.x == 0 && bad) atomicAdd(mismatches, static_cast<unsigned long long>(bad));
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
template <int B, bool FIM>
static void* kernel_ptr() {
    return reinterpret_cast<void*>(&k_solve<B, FIM>);
}

// Systolic B = 8 runs one warp per tile; everything else one CTA per tile (for
// B = 16 the 8-warp CTA per tile measured 1.8x faster than a warp per tile on
// the 4096^2 rings: a wave waits for its slowest tile, and a tile's sweeps are
// shorter spread over 8 warps).
static bool warp_tiles(int block, int fim) { return !fim && block == 8; }

static void* select_kernel(int block, int fim, bool wide) {
    if (wide && block == 16 && !fim) return reinterpret_cast<void*>(&k_solve<16, false, kWideCtas>);
    if (wide && block == 32 && !fim) return reinterpret_cast<void*>(&k_solve<32, false, kWideCtas>);
    switch (block) {
        case 8: return fim ? kernel_ptr<8, true>() : reinterpret_cast<void*>(&k_solve_warp<8>);
        case 16: return fim ? kernel_ptr<16, true>() : kernel_ptr<16, false>();
        case 32: return fim ? kernel_ptr<32, true>() : kernel_ptr<32, false>();
        default: return nullptr;
    }
}

static int threads_for(int block, int fim) {
    if (warp_tiles(block, fim)) return WarpTileGeom<8>::THREADS;
    switch (block) {
        case 8: return TileGeom<8>::THREADS;
        case 16: return TileGeom<16>::THREADS;
        case 32: return TileGeom<32>::THREADS;
        default: return 0;
    }
}

static int cap_for(int block, int fim, bool wide) {
    if (warp_tiles(block, fim)) return 4;
    if (wide && (block == 16 || block == 32) && !fim) return kWideCtas;
    switch (block) {
        case 8: return max_ctas_per_sm<8>();
        case 16: return max_ctas_per_sm<16>();
        case 32: return max_ctas_per_sm<32>();
        default: return 1;
    }
}

void tile_box(int block, uint32_t* width, uint32_t* height) {
    switch (block) {
        case 8: *width = TileGeom<8>::BW; *height = TileGeom<8>::BH; break;
        case 16: *width = TileGeom<16>::BW; *height = TileGeom<16>::BH; break;
        default: *width = TileGeom<32>::BW; *height = TileGeom<32>::BH; break;
    }
}

int query_persistent(int block, int fim, LaunchInfo* info, bool wide) {
    void* k = select_kernel(block, fim, wide);
    if (!k) return -1;
    int const threads = threads_for(block, fim);
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, threads, 0) != cudaSuccess) return -3;
    info->threads = threads;
    info->blocks_per_sm = std::min(bps, cap_for(block, fim, wide));
    info->wide = wide && (block == 16 || block == 32) && !fim;
    info->workers = warp_tiles(block, fim) ? WarpTileGeom<8>::NW : 1;
    return 0;
}

// A single field runs the wide build when a full wave holds more than twice
// as many jobs as the narrow build's grid has CTAs (see kWideCtas).
bool wide_for(const LaunchInfo& narrow, int sms, uint32_t max_jobs) {
    return static_cast<uint64_t>(max_jobs) >
           2u * static_cast<uint64_t>(std::max(1, narrow.blocks_per_sm)) * static_cast<uint64_t>(std::max(1, sms));
}

// Enough CTAs per SM that every job of a full wave has a worker of its own,
// within the occupancy cap. Fewer CTAs make the per-wave grid barrier cheaper
// and crowd an SM's tile solves less: on the 4096^2 seven-ring field with
// n = 256, 2 CTAs per SM solved in 13.7 ms against 15.6 ms with 4, while
// n = 1024, the noise field and batches want all 4.
int persistent_grid(const LaunchInfo& info, int sms, uint32_t max_jobs) {
    uint64_t const per_round = static_cast<uint64_t>(std::max(1, info.workers)) * static_cast<uint64_t>(sms);
    uint64_t const want = (static_cast<uint64_t>(max_jobs) + per_round - 1u) / per_round;
    int const per_sm = static_cast<int>(std::min<uint64_t>(std::max(1, info.blocks_per_sm), std::max<uint64_t>(1u, want)));
    return per_sm * sms;
}

cudaError_t launch_init(const Sched& s, uint32_t n_insts, uint64_t max_cells, uint32_t max_seeds, int block, int sms,
                        cudaStream_t st) {
    if (n_insts == 0u || n_insts > 65535u || sms <= 0) return cudaErrorInvalidValue;
    unsigned const tb = 256;
    // about 16 CTAs per SM over the whole batch, at least 8 per instance
    uint64_t const want = (max_cells + tb - 1) / tb;
    unsigned const per = static_cast<unsigned>(std::max<uint64_t>(8u, static_cast<uint64_t>(sms) * 16u * 4u / n_insts));
    unsigned const gx = static_cast<unsigned>(std::max<uint64_t>(1u, std::min<uint64_t>(want, per)));
    k_init_inst<<<dim3(gx, n_insts), tb, 0, st>>>(s);
    if (s.learn.tstat) {
        unsigned const g = static_cast<unsigned>(std::min<uint32_t>((s.num_tiles + 7u) / 8u, static_cast<uint32_t>(sms) * 16u));
        switch (block) {
            case 8: k_tile_stats<8><<<g, tb, 0, st>>>(s); break;
            case 16: k_tile_stats<16><<<g, tb, 0, st>>>(s); break;
            default: k_tile_stats<32><<<g, tb, 0, st>>>(s); break;
        }
    }
    if (max_seeds) {
        unsigned const sb = 128;
        unsigned const gs = std::min<unsigned>((max_seeds + sb - 1) / sb, 64u);
        k_init_seeds<<<dim3(gs, n_insts), sb, 0, st>>>(s, block);
    }
    return cudaGetLastError();
}

cudaError_t launch_persistent(int block, int fim, const Sched& s, int grid, cudaStream_t st, bool wide) {
    void* k = select_kernel(block, fim, wide);
    if (!k) return cudaErrorInvalidValue;
    void* args[] = {const_cast<Sched*>(&s)};
    // A learned-schedule launch stages the model in dynamic shared memory; its
    // grid is capped at what stays co-resident with that.
    size_t const dyn = s.learn.params ? kParams * sizeof(float) : 0u;
    if (dyn) {
        int dev = 0, sms = 0, bps = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, threads_for(block, fim), dyn);
        if (e != cudaSuccess) return e;
        if (bps <= 0) return cudaErrorInvalidConfiguration;
        grid = std::min(grid, bps * sms);
    }
    // A cooperative launch guarantees the co-residency the grid barrier needs;
    // through cudaLaunchKernelExC it can also be captured into a CUDA graph.
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(threads_for(block, fim));
    cfg.dynamicSmemBytes = dyn;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, k, args);
}

cudaError_t launch_sqrt_selftest(unsigned long long* mismatches, cudaStream_t st) {
    constexpr uint32_t kThreads = 256, kPerLaunch = 1u << 28;
    for (uint64_t base = 0; base < (1ull << 32); base += kPerLaunch)
        k_sqrt_selftest<<<kPerLaunch / kThreads, kThreads, 0, st>>>(static_cast<uint32_t>(base), mismatches);
    return cudaGetLastError();
}

cudaError_t launch_wait_selftest(uint32_t* flag, Ctl* ctl, uint64_t timeout_ns, cudaStream_t st) {
    k_wait_selftest<<<1, 32, 0, st>>>(flag, ctl, timeout_ns);
    return cudaGetLastError();
}

}  // namespace ghcm

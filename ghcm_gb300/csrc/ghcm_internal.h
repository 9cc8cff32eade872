// Internal types shared by the C-ABI layer (ghcm_capi.cpp) and the kernels
// (ghcm_solver.cu). Not part of the public interface.
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#include "ghcm.h"

namespace ghcm {

// Error bits written to Ctl::error by device code; the host maps them to
// GHCM_ERR_* codes.
enum : uint32_t {
    kErrTimeout      = 1u << 0,  // a bounded wait ran out
    kErrBadInput     = 1u << 1,  // NaN or negative speed / cost
    kErrNotConverged = 1u << 2,  // wave cap reached
    kErrInternal     = 1u << 3,  // list overflow or an impossible state
    kErrBadSeed      = 1u << 4,  // a device-resident seed lies outside its field
    kErrChecked      = 1u << 5,  // GHCM_CHECKED builds: an index check failed (Ctl::check_site)
};

// Per-tile scheduler flags.
enum : uint32_t {
    kActive   = 1u << 0,   // tile is in the active set (queued or about to be)
    kFull     = 1u << 1,   // re-solve every cell (residual check, sweep cap)
    kEdgeBit0 = 1u << 4,   // edge e of the tile received new boundary values: kEdgeBit0 << e
    kEdgeMask = 0xFu << 4,
    kSolveOne = 1u << 8,   // bits 8-11: the tile's block-solves so far, counted up to Sched::refresh
    kSolveMask = 0xFu << 8,
    kActPhase0 = 1u << 12, // bits 12-15: a neighbour's solve activated the tile in a jobs phase whose
    kActPhaseMask = 0xFu << 12,  // barrier generation is 0-3 mod 4 (kActPhase0 << gen % 4)
};
__host__ __device__ __forceinline__ uint32_t act_phase_bit(uint32_t gen) { return kActPhase0 << (gen & 3u); }
constexpr uint32_t kMaxRefresh = 15;  // largest Sched::refresh the 4-bit solve count holds
constexpr uint32_t kDefaultRefresh = 1;

__host__ __device__ __forceinline__ uint32_t solve_count(uint32_t flags) { return (flags & kSolveMask) >> 8; }

// One eikonal instance: a row-major W x H field and its block tiling.
struct Inst {
    const float* in;       // speed (in_is_speed) or cost
    float*       time;     // arrival times (in/out)
    uint32_t     w, h;
    uint32_t     tiles_x, tiles_y;
    uint32_t     tile_base;  // first global tile id of this instance
    float        spacing;    // h: cost = h / speed
    uint32_t     in_is_speed;
    int32_t      tma;        // 1: tiles of this instance are staged by TMA (maps in Sched)
    const uint32_t* seeds;   // n_seeds (x, y) pairs on the device
    uint32_t     n_seeds;
    float        cost_cap;   // cost = min(cost, cost_cap); +inf = no cap
};

// Device-side control block of one solve.
struct Ctl {
    unsigned long long release;    // wave-barrier release word: generation + the decided phase
    uint32_t bar_count;            // CTAs arrived at the current wave barrier
    uint32_t error;                // kErr* bits
    uint32_t count[2];             // sizes of the two active lists
    uint32_t krange[2][2];         // per list: {min, max} key bits of its tiles (a superset range)
    float    wave_front;           // smallest key of the set being scheduled this wave
    float    wave_span;            // its key range (max - min, > 0)
    uint32_t trace_count;          // trace records written (may exceed the capacity)
    uint32_t score_waves;          // learned schedule: waves chosen by score
    uint32_t fallback_waves;       // learned schedule: waves that fell back to the plain top-n
    uint32_t vetoes;               // learned schedule, veto mode: claims deferred by the model
    uint32_t waves;
    uint32_t residual_passes;
    uint32_t max_active;
    unsigned long long block_solves;
    unsigned long long prof[32];   // GHCM_PROFILE builds: per-phase nanoseconds and sweep counts
    unsigned long long release_ns; // GHCM_PROFILE builds: when the last barrier was released
    uint32_t wave_max_sweeps;      // GHCM_PROFILE builds: most sweeps of one block-solve in this wave
    uint32_t check_site;           // GHCM_CHECKED builds: largest id of a failed index check
    uint32_t sm_far;               // a CTA ran on an SM id >= kMaxSms: jobs go by block index
    uint32_t sm_ctas[256];         // CTAs of the persistent grid on each SM (by %smid)
};
constexpr uint32_t kMaxSms = 256;

// Learned block schedule and trace recorder (see ghcm_learn.cuh).
constexpr int kFeatures = 12;
constexpr int kHidden = 64;
// MLP parameters, flat: W1 [in][hidden], b1, W2 [hidden][hidden] (in-major),
// b2, W3 [hidden], b3.
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kFeatures * kHidden;
constexpr int kOffW2 = kOffB1 + kHidden;
constexpr int kOffB2 = kOffW2 + kHidden * kHidden;
constexpr int kOffW3 = kOffB2 + kHidden;
constexpr int kOffB3 = kOffW3 + kHidden;
constexpr int kParams = kOffB3 + 1;

// One block-solve of a trace: the features the scheduler saw when it chose
// the tile, and what the solve did. Layout = ghcm_trace_record.
struct TraceRec {
    float    f[kFeatures];
    uint32_t tile;
    uint32_t wave;
    uint32_t useful;   // 1: the solve moved some cell by more than eps
    uint32_t sweeps;
};

struct Learn {
    float4*   tstat;       // per tile: feature 4-6 (log speeds), set at init; nullptr: learning off
    uint32_t* kmax;        // per tile: largest activation key since its last claim (float bits)
    uint32_t* nsolve;      // per tile: block-solves so far
    uint32_t* last_change; // per tile: wave of its last useful solve + 1 (0: none)
    uint32_t* vetoes;      // per tile: consecutive vetoes (veto mode)
    float*    lscore[2];   // per entry of active list L: the tile's model logit (score mode), written by the
                           // solve that queued it; +inf for tiles re-queued in full, -inf until scored
    const float* params;   // MLP parameters (kParams floats); nullptr: plain schedule
    TraceRec* trace;       // trace records; nullptr: no trace
    uint32_t  trace_cap;
    float     threshold;   // take a tile when its score >= threshold
    uint32_t  fallback_jobs;  // n of the plain top-n when no tile qualifies
    uint32_t  veto;           // 1: the plain top-n proposes and the model vetoes at claim time
    uint32_t  max_vetoes;     // consecutive vetoes allowed per tile before it must be solved
};

// Everything the persistent kernel needs; passed by value as a
// __grid_constant__ parameter so that the tensor maps sit in parameter space.
struct Sched {
    CUtensorMap tmap_time;         // box (B+8) x (B+4) over the time field of instance 0
    CUtensorMap tmap_in;           // same box over the speed/cost field of instance 0
    const CUtensorMap* maps;       // batches: {time, in} maps of instance i at [2i], [2i+1]; nullptr: the two above
    const Inst* insts;
    const uint32_t* tile_inst;     // per-tile instance index (nullptr: a single instance)
    uint32_t* flags;               // per-tile kActive | kFull | edge bits
    uint32_t* key;                 // per-tile priority key (float bits; +inf = none)
    float*    tmin;                // per-tile smallest time after the last solve
    uint32_t* epoch;               // per tile: the residual pass its last changing solve came before (0: none)
    uint32_t* list[2];             // active lists, capacity num_tiles each
    uint32_t* jobs;                // selected jobs, capacity max_jobs
    Ctl*      ctl;
    uint32_t  num_tiles;
    uint32_t  num_insts;
    uint32_t  max_jobs;
    uint32_t  key_mode;
    uint32_t  max_sweeps;
    uint32_t  max_waves;
    float     eps;
    uint16_t  refresh;             // quiet block-solves per tile that may raise cells (kUpdFresh)
    uint16_t  in_solve;            // 1: the other solves recompute cells up to their staged value (kUpdInSolve)
    uint64_t  timeout_ns;
    Learn     learn;
};

// Launch configuration chosen by the host for a (block size, kernel) pair.
struct LaunchInfo {
    int threads;
    int blocks_per_sm;  // most CTAs per SM the grid may use (occupancy, capped)
    int workers;        // tile workers per CTA: 1, or 8 for one warp per tile
    bool wide;          // the 8-CTA-per-SM build of k_solve<16 or 32, systolic>
};

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Host helpers implemented in ghcm_capi.cpp.
int check_config(const ghcm_config* c);
EncodeTiledFn tensor_map_encoder();
bool encode_tile_map(EncodeTiledFn encode, CUtensorMap* map, const float* base, uint32_t w, uint32_t h,
                     uint32_t block);

// Host entry points implemented in ghcm_solver.cu.
// wide: the build for batches with more CTAs per SM, where there is one.
int query_persistent(int block, int fim, LaunchInfo* info, bool wide = false);
// CTAs of the persistent grid for waves of up to max_jobs tiles.
int persistent_grid(const LaunchInfo& info, int sms, uint32_t max_jobs);
// Whether a single field with waves of up to max_jobs tiles runs the wide
// build (more CTAs per SM) rather than `narrow`.
bool wide_for(const LaunchInfo& narrow, int sms, uint32_t max_jobs);
// The staged box (elements) of a tile: the TMA tensor maps use it as their box.
void tile_box(int block, uint32_t* width, uint32_t* height);
// Initialises the per-tile state, the time fields (+inf, inputs checked) and
// the seeds of every instance. max_cells / max_seeds: the largest instance.
cudaError_t launch_init(const Sched& s, uint32_t n_insts, uint64_t max_cells, uint32_t max_seeds, int block, int sms,
                        cudaStream_t st);
cudaError_t launch_persistent(int block, int fim, const Sched& s, int grid, cudaStream_t st, bool wide = false);
cudaError_t launch_wait_selftest(uint32_t* flag, Ctl* ctl, uint64_t timeout_ns, cudaStream_t st);
// Every 32-bit float through the solver's square root and __fsqrt_rn; adds the
// number of differing results to *mismatches (device memory).
cudaError_t launch_sqrt_selftest(unsigned long long* mismatches, cudaStream_t st);

}  // namespace ghcm

/*
 * ghcm.h - C ABI of the GB300 gHCM eikonal solver (libghcm.so).
 *
 * Replaces the reference's solver interface src/eikonal.h:12-67 for the gHCM
 * path (HcmConfig, EikonalResult, eikonal_hcm_opencl{,_setup,_ex}); the block
 * scheduler of src/eikonal_hcm.cpp:186-529 and the tile kernels of
 * data/eikonal_ghcm_systolic.cl / data/eikonal_ghcm_fim.cl run on the device.
 *
 * Plain C: pointers and sizes only. Every call returns an int status
 * (GHCM_OK or a negative GHCM_ERR_*); nothing exits or throws across the ABI,
 * unlike the reference's cl_do/exit paths (src/util_opencl.h:48-57,
 * src/eikonal_hcm.cpp:181-182).
 *
 * Fields are row-major float32 with x fastest: cell (x, y) is element
 * x + y * width (src/util_dim.h:17-21). Seeds are width/height-bounded
 * (x, y) pairs of uint32 with arrival time 0.
 *
 * Threading: a context may be used by one host thread at a time; calls on a
 * context are serialised. Different contexts are independent.
 */
#ifndef GHCM_H
#define GHCM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GHCM_ABI_VERSION 1

/* status codes */
#define GHCM_OK                 0
#define GHCM_ERR_BAD_ARG       -1  /* null pointer, zero size, seed outside the field, bad config */
#define GHCM_ERR_BAD_INPUT     -2  /* a speed/cost value is NaN or negative */
#define GHCM_ERR_OOM           -3  /* device or pinned allocation failed */
#define GHCM_ERR_CUDA          -4  /* a CUDA runtime call failed */
#define GHCM_ERR_TIMEOUT       -5  /* a bounded device-side wait ran out */
#define GHCM_ERR_NOT_CONVERGED -6  /* the wave cap was reached before convergence */
#define GHCM_ERR_UNSUPPORTED   -7  /* no usable GPU, or a size the build does not support */
#define GHCM_ERR_INTERNAL      -8  /* an internal invariant failed (a bug) */
#define GHCM_ERR_TOO_LARGE     -9  /* the field needs more tiles than ghcm_solve_device_noalloc's scratch holds */

/* ghcm_config.kernel - the tile solver (HcmConfig::Kernel, src/eikonal.h:13) */
#define GHCM_KERNEL_SYSTOLIC 0     /* sweep every cell until the tile converges */
#define GHCM_KERNEL_FIM      1     /* block-FIM: open-set cells only */

/* ghcm_config.schedule */
#define GHCM_SCHEDULE_PLAIN   0    /* lowest-key-first top-n (the reference's priority queue) */
#define GHCM_SCHEDULE_LEARNED 1    /* learned block-scheduling score */

/* ghcm_config.refresh_solves, special values:
 *   GHCM_REFRESH_OFF      the reference's form everywhere: every update keeps min(T_old, update)
 *   GHCM_REFRESH_IN_SOLVE sweeps recompute cells up to their value at the start of the block-solve;
 *                         no block-solve raises a cell */
#define GHCM_REFRESH_OFF      0xFFFFFFFFu
#define GHCM_REFRESH_IN_SOLVE 0xFFFFFFFEu

/* ghcm_config.key_mode - the plain priority key */
#define GHCM_KEY_BOUNDARY_MIN 0    /* min arrival time among the boundary values that activated the tile */
#define GHCM_KEY_BLOCK_MIN    1    /* min smallest_time over the tile and its 4 neighbours
                                      (BlockWrapper::calc_min_time, src/eikonal_hcm.cpp:58-70) */

typedef struct ghcm_config {
    uint32_t block_size;      /* tile side: 8, 16 or 32 (HcmConfig::block_size) */
    uint32_t max_jobs;        /* n, tiles solved per wave; 0 = 8 x SM count
                                 (HcmConfig::compute_unit_overload x compute units) */
    float    eps;             /* convergence threshold on |dT| (HcmConfig::fim_minimum_change) */
    uint32_t kernel;          /* GHCM_KERNEL_* */
    uint32_t schedule;        /* GHCM_SCHEDULE_* */
    uint32_t key_mode;        /* GHCM_KEY_* */
    uint32_t max_sweeps;      /* cap on inner sweeps per block-solve; 0 = 4 * block_size^2 */
    uint32_t max_waves;       /* cap on waves per solve; 0 = no cap */
    uint32_t wait_timeout_ms; /* limit of every device-side wait; 0 = 2000 */
    int32_t  device;          /* CUDA device ordinal; -1 = the current device */
    uint32_t use_tma;         /* 1 = stage tiles with TMA when the field allows it; 0 = plain loads */
    uint32_t fallback_jobs;   /* learned schedule: n of the plain top-n of a wave in which no tile
                                 qualifies; 0 = max_jobs */
    float    cost_cap;        /* > 0: cost = min(cost, cost_cap), the reference's permeable-wall
                                 transform field_cost_as_permeable (src/test_runner.cpp:70-75,
                                 default there 1e3); 0 = no cap */
    uint32_t refresh_solves;  /* rounding makes the update slightly non-monotone, and keeping
                                 min(T_old, update) of every evaluation (data/eikonal_common.cl:
                                 288-308) lets ulps drift low along a front. Sweeps therefore
                                 recompute each cell, bounded by its value at the start of the
                                 block-solve; the first refresh_solves quiet block-solves of a tile
                                 drop that bound (cells may rise, neighbours are told).
                                 0 = the default (1); 1..15; GHCM_REFRESH_IN_SOLVE; GHCM_REFRESH_OFF */
    uint32_t reserved[2];     /* must be zero */
} ghcm_config;

typedef struct ghcm_stats {
    uint64_t block_solves;    /* tile dispatches (the reference's profiling_info.size()) */
    uint64_t cells;           /* total cells solved for */
    uint64_t bytes_alg;       /* block_solves x algorithmic bytes per block-solve */
    uint32_t waves;           /* scheduler iterations */
    uint32_t residual_passes; /* global residual checks run */
    uint32_t max_active;      /* largest active-tile set seen */
    uint32_t tiles;           /* tiles in the tiling */
    double   device_ms;       /* device time from device-resident input to converged field */
    double   total_ms;        /* host wall time of the call, copies included */
    double   kernel_ms;       /* device time of the persistent solve kernel alone */
} ghcm_stats;

typedef struct ghcm_ctx ghcm_ctx;

/* Fills *cfg with the defaults (HcmConfig defaults, src/eikonal.h:17-26,
 * except block_size 16 and max_jobs 0). */
int ghcm_config_default(ghcm_config* cfg);

/* Creates a solver context on cfg->device. Replaces
 * eikonal_hcm_opencl_setup (src/eikonal_hcm.cpp:137-175). */
int ghcm_create(const ghcm_config* cfg, ghcm_ctx** out);

/* Releases a context and all its device memory. NULL is accepted. */
int ghcm_destroy(ghcm_ctx* ctx);

/* Solves for the arrival-time field with host buffers. Replaces
 * eikonal_hcm_opencl_ex (src/eikonal_hcm.cpp:186-529).
 *   field:      width*height values, speed (input_is_speed = 1, cost = h / speed)
 *               or cost (input_is_speed = 0, as the reference takes it)
 *   seeds_xy:   n_seeds (x, y) pairs
 *   time_out:   width*height arrival times (written)
 *   stats:      optional */
int ghcm_solve(ghcm_ctx* ctx, const float* field, int input_is_speed, uint32_t width, uint32_t height,
               float h, const uint32_t* seeds_xy, uint32_t n_seeds, float* time_out, ghcm_stats* stats);

/* Same with device-resident buffers on `stream` (a cudaStream_t; NULL = the
 * legacy default stream). d_seeds_xy is a device array. Returns when the
 * solve has finished on the stream. */
int ghcm_solve_device(ghcm_ctx* ctx, const float* d_field, int input_is_speed, uint32_t width,
                      uint32_t height, float h, const uint32_t* d_seeds_xy, uint32_t n_seeds,
                      float* d_time_out, void* stream, ghcm_stats* stats);

/* ---- batches: many independent instances in one persistent launch ----
 * No counterpart in the reference, which solves one field per call
 * (src/eikonal_hcm.cpp:186-529). Every instance is one reference solve
 * (eikonal_hcm_opencl_ex) with its own field, seeds and spacing; the tiles of
 * all instances share one device scheduler (one active set ordered by key,
 * n = cfg.max_jobs jobs per wave over the whole batch) and one persistent grid,
 * so small instances no longer leave the GPU idle. The launch sequence is
 * captured once in a CUDA graph and replayed by ghcm_batch_run. */

typedef struct ghcm_instance {
    const float*    field;          /* device: width*height speed (input_is_speed = 1) or cost */
    float*          time_out;       /* device: width*height arrival times (written) */
    const uint32_t* seeds_xy;       /* device: n_seeds (x, y) pairs */
    uint32_t        n_seeds;
    uint32_t        width, height;
    float           h;              /* grid spacing: cost = h / speed */
    int32_t         input_is_speed;
    uint32_t        reserved;       /* must be zero */
} ghcm_instance;

typedef struct ghcm_batch_info {
    uint32_t instances;
    uint32_t tiles;                 /* tiles over all instances */
    uint64_t cells;                 /* cells over all instances */
    uint32_t block_size;
    uint32_t max_jobs;              /* n per wave over the whole batch */
    uint32_t max_sweeps;
    uint32_t graph;                 /* 1: ghcm_batch_run replays a CUDA graph; 0: it launches directly */
    uint32_t grid;                  /* CTAs of the persistent launch */
    uint32_t tma_instances;         /* instances staged by TMA (the rest use plain loads) */
    uint32_t reserved[2];
} ghcm_batch_info;

typedef struct ghcm_batch ghcm_batch;

/* Validates the instances, allocates the batch's scheduler workspace and
 * captures its launch sequence (init + persistent solve + status readback)
 * into a CUDA graph. The instance buffers are the caller's and must stay
 * valid until ghcm_batch_destroy. Up to 65535 instances. Uses ctx's config
 * and device; the batch is independent of later calls on ctx. */
int ghcm_batch_create(ghcm_ctx* ctx, const ghcm_instance* insts, uint32_t count, ghcm_batch** out);

/* Solves every instance of the batch on `stream` (a cudaStream_t) and returns
 * when it has finished. stats (optional) cover the whole batch:
 * cells = sum of instance cells, device_ms = time of the replay. */
int ghcm_batch_run(ghcm_batch* batch, void* stream, ghcm_stats* stats);

int ghcm_batch_query(const ghcm_batch* batch, ghcm_batch_info* out);

/* Releases a batch. NULL is accepted. */
int ghcm_batch_destroy(ghcm_batch* batch);

/* create + run + destroy. */
int ghcm_solve_batched(ghcm_ctx* ctx, const ghcm_instance* insts, uint32_t count, void* stream, ghcm_stats* stats);

/* One autotuner trial. */
typedef struct ghcm_tune_trial {
    uint32_t block_size;
    uint32_t max_jobs;
    uint32_t max_sweeps;            /* 0 = to convergence (4 * block_size^2 cap) */
    int32_t  status;                /* GHCM_OK or the failing status */
    double   ms;                    /* best device time of the replays */
    uint64_t block_solves;
    uint32_t kernel;                /* GHCM_KERNEL_* */
    uint32_t reserved;
} ghcm_tune_trial;

/* Picks tile size (8, 16, 32), n, the inner-sweep cap and the tile kernel
 * for a batch by timing CUDA-graph replays of it, starting from `base` (its
 * kernel): tile size x n on the grid {8, 16, 32} x {4, 16, 64} x SMs, then n
 * halved and doubled around the best, then the inner-sweep caps B/2, B, 2B,
 * then the best config with the other tile kernel (15 trials).
 * Writes the fastest config to *best and the trials run to
 * trials[0..max_trials) (*n_trials = how many ran; trials may be NULL). The
 * instances' time_out fields hold a converged solve on return. reps >= 1
 * timed replays per trial after one warm-up. No counterpart in the reference
 * (its harness sweeps block sizes by hand, src/test_runner.cpp:226-291). */
int ghcm_autotune_batch(const ghcm_config* base, const ghcm_instance* insts, uint32_t count, void* stream,
                        uint32_t reps, ghcm_config* best, ghcm_tune_trial* trials, uint32_t max_trials,
                        uint32_t* n_trials);

/* ---- learned block schedule ----
 * No counterpart in the reference, whose only order is the min-time priority
 * queue (src/eikonal_hcm.cpp:47-80, 344-358). A 12 -> 64 -> 64 -> 1 FP32 MLP
 * (ReLU, sigmoid output) scores each active tile with P(its solve moves some
 * cell by more than eps). With cfg.schedule = GHCM_SCHEDULE_LEARNED and a
 * model set, every wave solves the tiles scoring >= threshold (plus tiles
 * re-queued by the residual check or a sweep cap), up to cfg.max_jobs; a wave
 * in which none qualifies falls back to the plain top-n. The global Godunov
 * residual check still decides convergence.
 *
 * Features (in this order, each roughly in [-1, 1]): the tile's key relative
 * to the wave's key range; the spread of its activation keys; never solved;
 * its smallest time above its key; log2 min / max / mean speed / 8; active
 * neighbours / 4; waves since its last useful solve / 64; log2(1 + solves) / 8;
 * re-queued in full; edges with new boundary values / 4.
 *
 * Parameters, flat float32 (GHCM_MLP_PARAMS): W1[12][64] (input-major), b1[64],
 * W2[64][64] (input-major), b2[64], W3[64], b3. */
#define GHCM_MLP_FEATURES 12
#define GHCM_MLP_HIDDEN   64
#define GHCM_MLP_PARAMS   5057

/* One block-solve of a trace: the features of the tile when the solve was
 * scheduled and whether it moved some cell by more than eps. */
typedef struct ghcm_trace_record {
    float    features[GHCM_MLP_FEATURES];
    uint32_t tile;
    uint32_t wave;
    uint32_t useful;    /* 1: some cell moved by more than eps */
    uint32_t sweeps;    /* inner sweeps of the solve */
} ghcm_trace_record;

/* Records a trace of every block-solve of the following solves on ctx, up to
 * `capacity` records per solve (0 turns tracing off). */
int ghcm_trace_enable(ghcm_ctx* ctx, uint32_t capacity);

/* Copies the last solve's trace: up to max_records to out; *n_records = how
 * many were copied, *n_total (optional) = solves the trace saw (more than the
 * capacity when it overflowed). */
int ghcm_trace_read(ghcm_ctx* ctx, ghcm_trace_record* out, uint32_t max_records, uint32_t* n_records,
                    uint32_t* n_total);

/* Sets the model of the learned schedule (host parameters, copied) and its
 * threshold in (0, 1). NULL params clear it. */
int ghcm_set_schedule_model(ghcm_ctx* ctx, const float* params, uint32_t n_params, float threshold);

/* How the learned schedule uses the model:
 *   GHCM_POLICY_SCORE (default): the CTA that queues a tile for the next wave
 *     scores it right after its own solve; the next wave solves the tiles
 *     scoring at or above the threshold, filled up to cfg.fallback_jobs tiles
 *     in plain key order (tiles queued without a score - the seeds' and, at
 *     block_size 8, every tile - go by key).
 *   GHCM_POLICY_VETO: the plain top-n proposes the wave; a CTA that
 *     claims a tile scores it first and defers it (back into the active set,
 *     key and edge bits kept) when the score is below the threshold, at most
 *     max_vetoes times in a row per tile (0 = 2). */
#define GHCM_POLICY_SCORE 0
#define GHCM_POLICY_VETO  1
int ghcm_set_schedule_policy(ghcm_ctx* ctx, uint32_t policy, uint32_t max_vetoes);

/* Learned-schedule counters of the last solve on ctx: out[0] waves chosen by
 * score, out[1] waves that fell back to the plain top-n, out[2] trace
 * records seen, out[3] claims deferred by a veto. */
int ghcm_schedule_counters(const ghcm_ctx* ctx, uint32_t out[4]);

/* Inference kernel: d_prob[i] = sigmoid(MLP(d_x[i*12 .. i*12+12))) on the
 * device, on `stream`; asynchronous. */
int ghcm_mlp_forward(const float* d_params, const float* d_x, uint32_t n, float* d_prob, void* stream);

/* Gradient kernel: adds the gradient of the summed weighted BCE loss of
 * samples (d_x, d_y in {0, 1}) to d_grad (GHCM_MLP_PARAMS floats) and the
 * summed loss to *d_loss_sum; asynchronous. */
int ghcm_mlp_grad(const float* d_params, const float* d_x, const float* d_y, uint32_t n, float pos_weight,
                  float* d_grad, float* d_loss_sum, void* stream);

typedef struct ghcm_train_config {
    uint32_t epochs;
    uint32_t batch;           /* samples per Adam step */
    float    lr;
    float    beta1, beta2, adam_eps;
    float    pos_weight;      /* weight of the positive (useful) class in the loss */
    uint32_t reserved[5];     /* must be zero */
} ghcm_train_config;

int ghcm_train_config_default(ghcm_train_config* cfg);

/* Trains the parameters in place (d_params, device) on n samples with Adam,
 * mini-batches taken in order (shuffle the samples beforehand). Blocks until
 * done. epoch_losses (optional, host, cfg->epochs floats) receives the mean
 * loss of each epoch. */
int ghcm_mlp_train(const float* d_x, const float* d_y, uint32_t n, float* d_params, const ghcm_train_config* cfg,
                   void* stream, float* epoch_losses);

/* Number of SMs of the context's device (the reference's compute units). */
int ghcm_device_sm_count(const ghcm_ctx* ctx, uint32_t* out);

/* Human-readable text for a status code. Never NULL. */
const char* ghcm_status_string(int status);

/* ABI version (GHCM_ABI_VERSION). */
int ghcm_abi_version(void);

/* Largest tiling (tiles of cfg->block_size) ghcm_solve_device_noalloc accepts:
 * 4096 x 4096 cells at block 8, 8192 x 8192 at block 16. */
#define GHCM_NOALLOC_MAX_TILES 262144u

/* ghcm_solve_device without a context and without allocating: no cudaMalloc,
 * cudaFree, pinned or library allocation of any kind. It has no counterpart in
 * the reference. For callers that cannot allocate GPU memory themselves or let
 * a library do it - a host whose pool owns every device allocation, a path that
 * must not synchronise the device the way cudaMalloc/cudaFree can, a service
 * whose footprint must not grow after start-up. The scheduler's scratch is one
 * static device array of about 7 MiB that every GPU loading the library holds
 * until exit; fields whose tiling exceeds GHCM_NOALLOC_MAX_TILES are rejected
 * with GHCM_ERR_TOO_LARGE. Runs on the current device (cfg->device must be -1
 * or that device) on `stream` and returns when the solve has finished: it
 * reads the solve's status back and synchronises `stream`, so it cannot be
 * captured into a CUDA graph. All calls share the one scratch array: calls
 * that overlap on the GPU (other streams or host threads) race and must be
 * serialised by the caller. No statistics are returned. Plain schedule only
 * (cfg->schedule must be GHCM_SCHEDULE_PLAIN). */
int ghcm_solve_device_noalloc(const ghcm_config* cfg, const float* d_field, int input_is_speed, uint32_t width,
                              uint32_t height, float h, const uint32_t* d_seeds_xy, uint32_t n_seeds,
                              float* d_time_out, void* stream);

/* Self-test of the bounded-wait path: launches a kernel that waits on a flag
 * nothing sets, with a limit of timeout_ms, and returns its status
 * (GHCM_ERR_TIMEOUT when the limit works). No counterpart in the reference,
 * whose device asserts spin forever (data/util_common.cl:26-30). */
int ghcm_selftest_wait_timeout(ghcm_ctx* ctx, uint32_t timeout_ms);

/* Self-test of the square root inside the device Godunov update: runs every
 * 32-bit float through it (both forms: the general one, and the short one
 * used on [2^-100, +inf) for tiles of normal costs) and through CUDA's IEEE
 * __fsqrt_rn on ctx's device and stores the number of inputs whose results
 * differ (NaN results compare equal) in *mismatches; 0 means the update's
 * square root is the correctly rounded one that the reference's update uses
 * (src/eikonal.h:121-137).
 * Takes about 10 ms. */
int ghcm_selftest_sqrt(ghcm_ctx* ctx, unsigned long long* mismatches);

#ifdef __cplusplus
}
#endif

#endif /* GHCM_H */

// Device-side block scheduler: tile addressing, neighbour activation, the
// top-n radix select and the wave barrier whose last arriving CTA decides the
// next phase. Replaces the host priority queue and activation loop of
// src/eikonal_hcm.cpp:343-469.
#pragma once

#include "ghcm_device.cuh"

namespace ghcm {

// Scheduler phases (Ctl::phase).
enum : uint32_t { kPhaseInit = 0, kPhaseJobs = 1, kPhaseResidual = 2, kPhaseDone = 3, kPhaseStop = 4 };

struct TileCoord {
    uint32_t tx, ty;
    int ox, oy;  // origin
    int sx, sy;  // size clipped at the field edge
};

__device__ __forceinline__ uint32_t inst_of(const Sched& s, uint32_t tile) {
    return s.tile_inst ? __ldg(&s.tile_inst[tile]) : 0u;
}

// Block id -> origin and clipped size (data/eikonal_ghcm_systolic.cl:65-97).
template <int B>
__device__ __forceinline__ TileCoord tile_coord(const Inst& I, uint32_t tile) {
    TileCoord c;
    uint32_t const local = tile - I.tile_base;
    c.tx = local % I.tiles_x;
    c.ty = local / I.tiles_x;
    c.ox = static_cast<int>(c.tx) * B;
    c.oy = static_cast<int>(c.ty) * B;
    c.sx = min(B, static_cast<int>(I.w) - c.ox);
    c.sy = min(B, static_cast<int>(I.h) - c.oy);
    return c;
}

// Neighbour tile across edge e (0: -x, 1: -y, 2: +x, 3: +y; the reference's
// Border order, data/eikonal_common.cl:361, src/eikonal_hcm.cpp:18), or -1.
__device__ __forceinline__ int neighbour_tile(const Inst& I, uint32_t tx, uint32_t ty, int e) {
    int const nx = static_cast<int>(tx) + (e == 0 ? -1 : (e == 2 ? 1 : 0));
    int const ny = static_cast<int>(ty) + (e == 1 ? -1 : (e == 3 ? 1 : 0));
    if (nx < 0 || ny < 0 || nx >= static_cast<int>(I.tiles_x) || ny >= static_cast<int>(I.tiles_y)) return -1;
    return static_cast<int>(I.tile_base) + ny * static_cast<int>(I.tiles_x) + nx;
}

// cost = h / speed (src/test_runner.cpp:38-42), IEEE-rounded like the host's.
__device__ __forceinline__ float to_cost(const Inst& I, float v) {
    return I.in_is_speed ? __fdiv_rn(I.spacing, v) : v;
}

// Puts `tile` into the next active set: lowers its key to `key`, ORs `bits`
// into its flags and appends it to list[nxt] unless it is already active.
// The device form of the dirty-set test + heap push + border-mask OR of
// src/eikonal_hcm.cpp:451-462.
__device__ __forceinline__ void activate(const Sched& s, uint32_t tile, uint32_t bits, float key, uint32_t nxt) {
    atomicMin(&s.key[tile], __float_as_uint(key));
    uint32_t const old = atomicOr(&s.flags[tile], kActive | bits);
    if (!(old & kActive)) {
        uint32_t const pos = atomicAdd(&s.ctl->count[nxt], 1u);
        if (pos < s.num_tiles)
            s.list[nxt][pos] = tile;
        else
            atomicOr(&s.ctl->error, kErrInternal);
    }
}

// Priority key of an active tile (smaller = solved first), as float bits.
__device__ __forceinline__ uint32_t tile_key(const Sched& s, uint32_t tile) {
    if (s.key_mode == 0u) return __ldcg(&s.key[tile]);
    // Block-min key: smallest_time of the tile and of its 4 neighbours
    // (BlockWrapper::calc_min_time, src/eikonal_hcm.cpp:58-70).
    const Inst& I = s.insts[inst_of(s, tile)];
    uint32_t const local = tile - I.tile_base;
    uint32_t const tx = local % I.tiles_x, ty = local / I.tiles_x;
    float k = __ldcg(&s.tmin[tile]);
    for (int e = 0; e < 4; ++e) {
        int const nb = neighbour_tile(I, tx, ty, e);
        if (nb >= 0) k = fminf(k, __ldcg(&s.tmin[nb]));
    }
    return __float_as_uint(k);
}

// Radix select of the `n` smallest keys among the m tiles of `list`, by the
// whole CTA: selected tiles go to s.jobs, the rest to `carry`. Keys are
// non-negative floats, so their bit patterns order like their values.
// Returns the number of carried tiles.
template <int THREADS>
__device__ uint32_t select_top_n(const Sched& s, const uint32_t* list, uint32_t m, uint32_t n, uint32_t* carry,
                                 uint32_t* s_hist, uint32_t* s_sel) {
    int const tid = threadIdx.x;
    uint32_t prefix = 0u, pmask = 0u, rank = n;
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int i = tid; i < 256; i += THREADS) s_hist[i] = 0u;
        __syncthreads();
        for (uint32_t i = tid; i < m; i += THREADS) {
            uint32_t const k = tile_key(s, __ldcg(&list[i]));
            if ((k & pmask) == prefix) atomicAdd(&s_hist[(k >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (tid < 32) {
            uint32_t part[8];
            uint32_t tot = 0u;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                part[j] = s_hist[tid * 8 + j];
                tot += part[j];
            }
            uint32_t incl = tot;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t const v = __shfl_up_sync(0xffffffffu, incl, o);
                if (tid >= o) incl += v;
            }
            uint32_t below = incl - tot;
            if (below < rank && rank <= incl) {
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    if (below + part[j] >= rank) {
                        s_sel[0] = static_cast<uint32_t>(tid * 8 + j);
                        s_sel[1] = below;
                        break;
                    }
                    below += part[j];
                }
            }
        }
        __syncthreads();
        rank -= s_sel[1];
        prefix |= s_sel[0] << shift;
        pmask |= 255u << shift;
        // every key equal to the prefix so far is taken: no need to refine
        if (s_hist[s_sel[0]] == rank) break;
        __syncthreads();
    }
    // take every key below the boundary prefix and `rank` keys that match it
    __syncthreads();
    if (tid == 0) {
        s_sel[2] = 0u;
        s_sel[3] = 0u;
        s_sel[4] = 0u;
    }
    __syncthreads();
    for (uint32_t i = tid; i < m; i += THREADS) {
        uint32_t const t = __ldcg(&list[i]);
        uint32_t const k = tile_key(s, t);
        bool take = (k & pmask) < prefix;
        if (!take && (k & pmask) == prefix) take = atomicAdd(&s_sel[2], 1u) < rank;
        if (take)
            s.jobs[atomicAdd(&s_sel[3], 1u)] = t;
        else
            carry[atomicAdd(&s_sel[4], 1u)] = t;
    }
    __syncthreads();
    return s_sel[4];
}

// Decides the next phase; run by the whole of the last CTA to reach the wave
// barrier while every other CTA waits.
//   after INIT / JOBS / RESIDUAL, the set to process is list[act]:
//     non-empty          -> JOBS on its n lowest keys (the rest carried over)
//     empty after JOBS   -> RESIDUAL: the global fixed-point check
//     empty after RESID. -> DONE
template <int THREADS>
__device__ void decide_phase(const Sched& s, uint32_t* s_hist, uint32_t* s_sel) {
    Ctl* ctl = s.ctl;
    int const tid = threadIdx.x;
    uint32_t const prev = ld_relaxed(&ctl->phase);
    uint32_t const cur = ld_relaxed(&ctl->cur);
    uint32_t const act = (prev == kPhaseInit) ? 0u : (cur ^ 1u);
    uint32_t const m = ld_relaxed(&ctl->count[act]);
    if (m == 0u) {
        if (tid == 0) {
            if (prev == kPhaseResidual) {
                ctl->phase = kPhaseDone;
            } else {
                ctl->phase = kPhaseResidual;
                ctl->cur = act ^ 1u;  // residual activations go to list[act], now empty
                ctl->count[act] = 0u;
                ctl->residual_passes += 1u;
            }
        }
        return;
    }
    if (s.max_waves != 0u && ld_relaxed(&ctl->waves) >= s.max_waves) {
        if (tid == 0) {
            atomicOr(&ctl->error, kErrNotConverged);
            ctl->phase = kPhaseStop;
        }
        return;
    }
    uint32_t carried = 0u;
    bool const all = m <= s.max_jobs;
    if (!all) carried = select_top_n<THREADS>(s, s.list[act], m, s.max_jobs, s.list[act ^ 1u], s_hist, s_sel);
    if (tid == 0) {
        ctl->job_count = all ? m : m - carried;
        ctl->jobs_in_list = all ? 1u : 0u;
        ctl->count[act ^ 1u] = carried;
        ctl->cur = act;
        ctl->phase = kPhaseJobs;
        ctl->waves += 1u;
        if (m > ctl->max_active) ctl->max_active = m;
    }
}

// Grid-wide wave barrier. Every CTA arrives; the last one to arrive decides
// the next phase (decide_phase) before releasing the others. The waits are
// bounded. On return, s_state holds {phase, cur, job_count, jobs_in_list};
// returns false when the grid must stop (timeout or error).
template <int THREADS>
__device__ bool wave_barrier(const Sched& s, uint32_t* s_hist, uint32_t* s_sel, uint32_t* s_state) {
    __shared__ uint32_t s_last;
    Ctl* ctl = s.ctl;
    BarrierWords* bw = reinterpret_cast<BarrierWords*>(ctl);
    __syncthreads();
    uint32_t gen = 0u;
    if (threadIdx.x == 0) {
        gen = ld_relaxed(&bw->gen);
        __threadfence();
        uint32_t const arrived = atomicAdd(&bw->count, 1u) + 1u;
        __threadfence();
        s_last = (arrived == gridDim.x) ? 1u : 0u;
    }
    __syncthreads();
    if (s_last) {
        if (threadIdx.x == 0) bw->count = 0u;
        if (ld_relaxed(&ctl->error) == 0u) decide_phase<THREADS>(s, s_hist, s_sel);
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(&bw->gen, 1u);
        }
    } else if (threadIdx.x == 0) {
        uint64_t const t0 = global_ns();
        uint32_t spins = 0;
        while (ld_acquire(&bw->gen) == gen) {
            if (++spins > 32) {
                __nanosleep(32);
                if (global_ns() - t0 > s.timeout_ns) {
                    atomicOr(&ctl->error, kErrTimeout);
                    break;
                }
            }
        }
    }
    if (threadIdx.x == 0) {
        __threadfence();
        s_state[0] = ld_relaxed(&ctl->phase);
        s_state[1] = ld_relaxed(&ctl->cur);
        s_state[2] = ld_relaxed(&ctl->job_count);
        s_state[3] = ld_relaxed(&ctl->jobs_in_list);
        s_state[4] = ld_relaxed(&ctl->error);
    }
    __syncthreads();
    return s_state[4] == 0u;
}

}  // namespace ghcm

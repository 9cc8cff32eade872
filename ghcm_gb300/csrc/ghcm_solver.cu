// The gHCM block eikonal solve on the device.
//
// One persistent, co-resident grid runs the whole solve:
//
//   wave loop (replaces the host loop of src/eikonal_hcm.cpp:343-482):
//     select   CTA 0 picks the n active tiles with the smallest keys (radix
//              select over the float-bit keys) - the device form of the host
//              priority queue pop (src/eikonal_hcm.cpp:344-358);
//     barrier
//     solve    every CTA takes jobs from a shared counter; a job stages its
//              tile plus a one-cell halo into shared memory (TMA when the field
//              allows it), iterates Godunov updates to convergence (systolic:
//              data/eikonal_ghcm_systolic.cl:130-153, or block-FIM:
//              data/eikonal_ghcm_fim.cl:347-372), probes the four neighbour
//              edge rows (check_border, data/eikonal_ghcm_systolic.cl:8-41,
//              probe-only as in data/eikonal_ghcm_fim.cl:175-194), writes the
//              tile back and activates improved neighbours with atomics
//              (src/eikonal_hcm.cpp:434-469);
//     barrier
//   when no tile is active, a global Godunov residual pass over every cell
//   re-activates any tile that is not at the fixed point; the solve ends when
//   that pass activates nothing. The reference has no such judge
//   (src/eikonal_hcm.cpp:343, 486-488).
//
// Tiles are B x B cells of the row-major field (block id = tx + ty * tiles_x,
// origin = (tx, ty) * B, size clipped at the field edge:
// data/eikonal_ghcm_systolic.cl:65-97). Every wait is bounded.
#include "ghcm_device.cuh"
#include "ghcm_internal.h"

#include <algorithm>

// GHCM_PROFILE builds accumulate per-phase times (thread 0 of each CTA) into
// Ctl::prof: [0] barrier waits, [1] block-solves, [2] select, [3] sweeps,
// [4] residual passes, [5] kernel wall time (CTA 0). They change no result.
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

namespace ghcm {

template <int B>
struct TileGeom {
    static constexpr int THREADS = (B * B < 64) ? 64 : (B * B > 256 ? 256 : B * B);
    static constexpr int CPT = (B * B) / THREADS;  // cells per thread
    static constexpr int BW = B + 8;               // staged box width: x in [ox-4, ox+B+4)
    static constexpr int BH = B + 2;               // staged box height: y in [oy-1, oy+B+1)
    static constexpr int BOX = BW * BH;
    static constexpr int BOXP = (BOX + 31) / 32 * 32;  // keeps each staged box 128-byte aligned for TMA
    static constexpr int RING = (B + 2) * (B + 2);  // the tile and its one-cell halo
    static_assert(4 * B % 32 == 0, "edge probes need whole warps");
    static_assert(B * B % THREADS == 0, "cells must divide evenly");
};

struct TileCoord {
    uint32_t tx, ty;
    int ox, oy;  // origin
    int sx, sy;  // clipped size
};

__device__ __forceinline__ uint32_t inst_of(const Sched& s, uint32_t tile) {
    return s.tile_inst ? __ldg(&s.tile_inst[tile]) : 0u;
}

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

__device__ __forceinline__ float to_cost(const Inst& I, float v) {
    return I.in_is_speed ? __fdiv_rn(I.spacing, v) : v;
}

// Puts `tile` into the next active set: lowers its key to `key`, ORs `bits`
// into its flags and appends it to list[nxt] if it was not already active.
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

// Priority key of an active tile (smaller = solved first).
__device__ __forceinline__ uint32_t tile_key(const Sched& s, uint32_t tile) {
    if (s.key_mode == 0u) return __ldcg(&s.key[tile]);
    // Block-min key: smallest_time of the tile and its 4 neighbours
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

// ---------------------------------------------------------------------------
// Select phase, run by CTA 0 alone while the grid waits at the barrier.
// ---------------------------------------------------------------------------
template <int THREADS>
__device__ void select_phase(const Sched& s, uint32_t cur, uint32_t* s_hist, uint32_t* s_sel) {
    Ctl* ctl = s.ctl;
    int const tid = threadIdx.x;
    uint32_t const nxt = cur ^ 1u;
    uint32_t const m = ld_relaxed(&ctl->count[cur]);
    if (m == 0u) {
        if (tid == 0) {
            ctl->job_next = 0u;
            ctl->job_count = 0u;
            ctl->count[nxt] = 0u;
        }
        return;
    }
    if (s.max_waves != 0u && ld_relaxed(&ctl->waves) >= s.max_waves) {
        if (tid == 0) {
            atomicOr(&ctl->error, kErrNotConverged);
            ctl->stop = 1u;
        }
        return;
    }
    if (m <= s.max_jobs) {
        if (tid == 0) {
            ctl->job_next = 0u;
            ctl->job_count = m;
            ctl->jobs_in_list = 1u;
            ctl->count[nxt] = 0u;
            ctl->waves += 1u;
            if (m > ctl->max_active) ctl->max_active = m;
        }
        return;
    }

    // Radix select of the n smallest keys, 8 bits per pass from the top.
    const uint32_t* list = s.list[cur];
    uint32_t prefix = 0u, pmask = 0u, rank = s.max_jobs;
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
        __syncthreads();
    }
    // prefix is the n-th smallest key; take every smaller key and `rank` of the equal ones.
    if (tid == 0) {
        s_sel[2] = 0u;
        s_sel[3] = 0u;
        s_sel[4] = 0u;
    }
    __syncthreads();
    uint32_t* carry = s.list[nxt];
    for (uint32_t i = tid; i < m; i += THREADS) {
        uint32_t const t = __ldcg(&list[i]);
        uint32_t const k = tile_key(s, t);
        bool take = k < prefix;
        if (!take && k == prefix) take = atomicAdd(&s_sel[2], 1u) < rank;
        if (take)
            s.jobs[atomicAdd(&s_sel[3], 1u)] = t;
        else
            carry[atomicAdd(&s_sel[4], 1u)] = t;
    }
    __syncthreads();
    if (tid == 0) {
        ctl->job_next = 0u;
        ctl->job_count = s_sel[3];
        ctl->jobs_in_list = 0u;
        ctl->count[nxt] = s_sel[4];
        ctl->waves += 1u;
        if (m > ctl->max_active) ctl->max_active = m;
    }
}

// ---------------------------------------------------------------------------
// Global residual judge: re-activates every tile holding a cell whose Godunov
// update would still lower it by more than eps.
// ---------------------------------------------------------------------------
template <int B>
__device__ void residual_pass(const Sched& s, uint32_t nxt) {
    using G = TileGeom<B>;
    __shared__ float s_kmin;
    int const tid = threadIdx.x;
    for (uint32_t tile = blockIdx.x; tile < s.num_tiles; tile += gridDim.x) {
        const Inst& I = s.insts[inst_of(s, tile)];
        TileCoord const tc = tile_coord<B>(I, tile);
        if (tid == 0) s_kmin = f_inf();
        bool bad = false;
        float kmin = f_inf();
#pragma unroll
        for (int k = 0; k < G::CPT; ++k) {
            int const id = tid + k * G::THREADS;
            int const lx = id % B, ly = id / B;
            if (lx >= tc.sx || ly >= tc.sy) continue;
            int const gx = tc.ox + lx, gy = tc.oy + ly;
            size_t const gi = static_cast<size_t>(gy) * I.w + gx;
            float const c = to_cost(I, __ldg(&I.in[gi]));
            if (!(c < f_inf())) continue;
            float const t = __ldcg(&I.time[gi]);
            float const xl = gx > 0 ? __ldcg(&I.time[gi - 1]) : f_inf();
            float const xr = gx + 1 < static_cast<int>(I.w) ? __ldcg(&I.time[gi + 1]) : f_inf();
            float const yu = gy > 0 ? __ldcg(&I.time[gi - I.w]) : f_inf();
            float const yd = gy + 1 < static_cast<int>(I.h) ? __ldcg(&I.time[gi + I.w]) : f_inf();
            float const nt = godunov(fminf(xl, xr), fminf(yu, yd), c, t);
            if (time_diff(nt, t) < -s.eps) {
                bad = true;
                kmin = fminf(kmin, nt);
            }
        }
        __syncthreads();
        if (bad) atomicMin(reinterpret_cast<unsigned int*>(&s_kmin), __float_as_uint(kmin));
        if (__syncthreads_or(bad) && tid == 0) activate(s, tile, kFull, s_kmin, nxt);
    }
}

// ---------------------------------------------------------------------------
// One block-solve.
// ---------------------------------------------------------------------------
template <int B>
struct TileSmem {
    float time[TileGeom<B>::BOXP];
    float cost[TileGeom<B>::BOXP];
};

template <int B, bool FIM>
__device__ void solve_tile(const Sched& s, uint32_t tile, uint32_t nxt, TileSmem<B>& sm, uint64_t* bar,
                           uint32_t& parity, bool& tma_pending, uint8_t* s_check, uint32_t* s_word,
                           float* s_red) {
    using G = TileGeom<B>;
    constexpr int BW = G::BW;
    int const tid = threadIdx.x;
    const Inst& I = s.insts[inst_of(s, tile)];
    TileCoord const tc = tile_coord<B>(I, tile);
    bool const use_tma = I.tma != 0;

    // Claim the tile: clear its activation state (a later activation re-queues
    // it) and stage the tile with its halo.
    if (tid == 0) {
        uint32_t const f = atomicAnd(&s.flags[tile], ~(kActive | kFull | kEdgeMask));
        atomicExch(&s.key[tile], inf_bits());
        __threadfence();
        s_word[0] = f;
        s_word[1] = 0u;  // abort flag
        if (use_tma) {
            fence_proxy_async();
            mbar_arrive_expect_tx(bar, static_cast<uint32_t>(2 * G::BOX * sizeof(float)));
            tma_load_2d(sm.time, &s.tmap_time, bar, tc.ox - 4, tc.oy - 1);
            tma_load_2d(sm.cost, &s.tmap_in, bar, tc.ox - 4, tc.oy - 1);
            tma_pending = true;
        }
    }
    __syncthreads();
    uint32_t const flags = s_word[0];
    if (use_tma) {
        if (!mbar_wait(bar, parity, s.timeout_ns)) {
            atomicOr(&s.ctl->error, kErrTimeout);
            s_word[1] = 1u;  // acted on after the barrier below, by every thread
        } else if (tid == 0) {
            tma_pending = false;
        }
        parity ^= 1u;
        for (int r = tid; r < G::RING; r += G::THREADS) {
            int const lx = r % (B + 2) - 1, ly = r / (B + 2) - 1;
            int const gx = tc.ox + lx, gy = tc.oy + ly;
            int const si = (ly + 1) * BW + lx + 4;
            bool const in = gx >= 0 && gy >= 0 && gx < static_cast<int>(I.w) && gy < static_cast<int>(I.h);
            if (!in) {
                sm.time[si] = f_inf();
                sm.cost[si] = f_inf();
            } else if (I.in_is_speed) {
                sm.cost[si] = __fdiv_rn(I.spacing, sm.cost[si]);
            }
        }
    } else {
        for (int r = tid; r < G::RING; r += G::THREADS) {
            int const lx = r % (B + 2) - 1, ly = r / (B + 2) - 1;
            int const gx = tc.ox + lx, gy = tc.oy + ly;
            int const si = (ly + 1) * BW + lx + 4;
            bool const in = gx >= 0 && gy >= 0 && gx < static_cast<int>(I.w) && gy < static_cast<int>(I.h);
            size_t const gi = static_cast<size_t>(gy) * I.w + gx;
            sm.time[si] = in ? __ldcg(&I.time[gi]) : f_inf();
            sm.cost[si] = in ? to_cost(I, __ldg(&I.in[gi])) : f_inf();
        }
    }
    __syncthreads();
    if (s_word[1]) return;  // staging timed out; the grid stops at the next barrier

    float t[G::CPT], c[G::CPT];
    int si[G::CPT], lxs[G::CPT], lys[G::CPT];
    bool v[G::CPT], inside[G::CPT];
#pragma unroll
    for (int k = 0; k < G::CPT; ++k) {
        int const id = tid + k * G::THREADS;
        lxs[k] = id % B;
        lys[k] = id / B;
        inside[k] = lxs[k] < tc.sx && lys[k] < tc.sy;
        si[k] = (lys[k] + 1) * BW + lxs[k] + 4;
        t[k] = sm.time[si[k]];
        c[k] = sm.cost[si[k]];
        v[k] = inside[k] && c[k] < f_inf();
    }
    float const eps = s.eps;
    bool own_changed = false;
    bool capped = false;
    uint32_t sweeps = 0;

    if (!FIM) {
        // Systolic: sweep every cell until no cell moves by more than eps.
        for (;;) {
            bool moved = false;
#pragma unroll
            for (int k = 0; k < G::CPT; ++k) {
                if (!v[k]) continue;
                int const i = si[k];
                float const ax = fminf(sm.time[i - 1], sm.time[i + 1]);
                float const ay = fminf(sm.time[i - BW], sm.time[i + BW]);
                float const nt = godunov(ax, ay, c[k], t[k]);
                if (nt < t[k]) {
                    moved |= time_diff(nt, t[k]) < -eps;
                    t[k] = nt;
                    sm.time[i] = nt;
                    own_changed = true;
                }
            }
            ++sweeps;
            if (!__syncthreads_or(moved)) break;
            if (sweeps >= s.max_sweeps) {
                capped = true;
                break;
            }
        }
    } else {
        // Block-FIM: only open cells are solved; a converged cell asks its
        // in-tile neighbours to re-check, and a neighbour that improves by
        // more than eps opens (data/eikonal_ghcm_fim.cl:166-210, 347-372).
        bool open[G::CPT];
        uint32_t const edges = (flags & kEdgeMask) >> 4;
        bool const full = (flags & kFull) != 0u;
#pragma unroll
        for (int k = 0; k < G::CPT; ++k) {
            int const i = si[k];
            bool const on_edge = ((edges & 1u) && lxs[k] == 0) || ((edges & 2u) && lys[k] == 0) ||
                                 ((edges & 4u) && lxs[k] == tc.sx - 1) || ((edges & 8u) && lys[k] == tc.sy - 1);
            bool const by_seed = sm.time[i - 1] == 0.f || sm.time[i + 1] == 0.f || sm.time[i - BW] == 0.f ||
                                 sm.time[i + BW] == 0.f;
            open[k] = v[k] && (full || on_edge || by_seed);
        }
        bool any_open = false;
#pragma unroll
        for (int k = 0; k < G::CPT; ++k) any_open |= open[k];
        if (__syncthreads_or(any_open)) {
            for (;;) {
#pragma unroll
                for (int k = 0; k < G::CPT; ++k) {
                    if (!open[k]) continue;
                    int const i = si[k];
                    float const ax = fminf(sm.time[i - 1], sm.time[i + 1]);
                    float const ay = fminf(sm.time[i - BW], sm.time[i + BW]);
                    float const nt = godunov(ax, ay, c[k], t[k]);
                    bool moved = false;
                    if (nt < t[k]) {
                        moved = time_diff(nt, t[k]) < -eps;
                        t[k] = nt;
                        sm.time[i] = nt;
                        own_changed = true;
                    }
                    if (moved) continue;
                    open[k] = false;
                    int const lx = lxs[k], ly = lys[k];
                    if (lx > 0 && sm.cost[i - 1] < f_inf()) s_check[ly * B + lx - 1] = 1;
                    if (lx + 1 < tc.sx && sm.cost[i + 1] < f_inf()) s_check[ly * B + lx + 1] = 1;
                    if (ly > 0 && sm.cost[i - BW] < f_inf()) s_check[(ly - 1) * B + lx] = 1;
                    if (ly + 1 < tc.sy && sm.cost[i + BW] < f_inf()) s_check[(ly + 1) * B + lx] = 1;
                }
                __syncthreads();
                bool still_open = false;
#pragma unroll
                for (int k = 0; k < G::CPT; ++k) {
                    if (!v[k]) continue;
                    int const cell = lys[k] * B + lxs[k];
                    if (s_check[cell]) {
                        s_check[cell] = 0;
                        if (!open[k]) {
                            int const i = si[k];
                            float const ax = fminf(sm.time[i - 1], sm.time[i + 1]);
                            float const ay = fminf(sm.time[i - BW], sm.time[i + BW]);
                            float const nt = godunov(ax, ay, c[k], t[k]);
                            if (nt < t[k]) {
                                open[k] = time_diff(nt, t[k]) < -eps;
                                t[k] = nt;
                                sm.time[i] = nt;
                                own_changed = true;
                            }
                        }
                    }
                    still_open |= open[k];
                }
                ++sweeps;
                if (!__syncthreads_or(still_open)) break;
                if (sweeps >= s.max_sweeps) {
                    capped = true;
                    break;
                }
            }
        }
    }

    // Probe the neighbour tiles' edge rows with the converged tile
    // (data/eikonal_ghcm_systolic.cl:8-41): edge e, cell i of that row.
    int const e = tid / B;
    int const ei = tid % B;
    bool e_imp = false;
    float e_key = f_inf();
    int nb = -1;
    if (tid < 4 * B) {
        nb = neighbour_tile(I, tc.tx, tc.ty, e);
        int const len = (e & 1) ? tc.sx : tc.sy;
        if (nb >= 0 && ei < len) {
            int px, py, qx, qy;
            if (e == 0) { px = -1; py = ei; qx = 0; qy = ei; }
            else if (e == 1) { px = ei; py = -1; qx = ei; qy = 0; }
            else if (e == 2) { px = tc.sx; py = ei; qx = tc.sx - 1; qy = ei; }
            else { px = ei; py = tc.sy; qx = ei; qy = tc.sy - 1; }
            int const pi = (py + 1) * BW + px + 4;
            float const cp = sm.cost[pi];
            if (cp < f_inf()) {
                float const told = sm.time[pi];
                // the cell beyond the probed one lies outside the staged halo: +inf
                float const a_norm = sm.time[(qy + 1) * BW + qx + 4];
                float const a_lat = (e & 1) ? fminf(sm.time[pi - 1], sm.time[pi + 1])
                                            : fminf(sm.time[pi - BW], sm.time[pi + BW]);
                float const nt = godunov(a_norm, a_lat, cp, told);
                if (time_diff(nt, told) < -eps) {
                    e_imp = true;
                    e_key = nt;
                }
            }
        }
#pragma unroll
        for (int o = B / 2; o >= 1; o >>= 1) {
            e_imp |= __shfl_xor_sync(0xffffffffu, static_cast<int>(e_imp), o) != 0;
            e_key = fminf(e_key, __shfl_xor_sync(0xffffffffu, e_key, o));
        }
    }

    GHCM_PROF_COUNT(s.ctl, 3, sweeps);
    // Commit the tile and its smallest time.
    bool const tile_changed = __syncthreads_or(own_changed) != 0;
    float lmin = f_inf();
#pragma unroll
    for (int k = 0; k < G::CPT; ++k) {
        if (!inside[k]) continue;
        lmin = fminf(lmin, t[k]);
        if (tile_changed)
            I.time[static_cast<size_t>(tc.oy + lys[k]) * I.w + tc.ox + lxs[k]] = t[k];
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) lmin = fminf(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
    if ((tid & 31) == 0) s_red[tid >> 5] = lmin;
    __threadfence();
    __syncthreads();
    if (tid == 0) {
        float m = s_red[0];
        for (int w = 1; w < G::THREADS / 32; ++w) m = fminf(m, s_red[w]);
        s.tmin[tile] = m;
        if (capped) activate(s, tile, kFull, m, nxt);
    }
    if (tid < 4 * B && ei == 0 && e_imp) activate(s, static_cast<uint32_t>(nb), kEdgeBit0 << ((e + 2) & 3), e_key, nxt);
    __syncthreads();
}

template <int B, bool FIM>
__global__ void __launch_bounds__(TileGeom<B>::THREADS) k_persistent(const __grid_constant__ Sched s) {
    using G = TileGeom<B>;
    __shared__ __align__(128) TileSmem<B> sm;
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ uint32_t s_hist[256];
    __shared__ uint32_t s_sel[8];
    __shared__ uint32_t s_word[4];
    __shared__ float s_red[G::THREADS / 32];
    __shared__ uint8_t s_check[FIM ? B * B : 4];

    Ctl* ctl = s.ctl;
    BarrierWords* bw = reinterpret_cast<BarrierWords*>(ctl);
    int const tid = threadIdx.x;
    if (ld_relaxed(&ctl->error) != 0u) return;  // the init kernels rejected the input

    if (tid == 0) mbar_init(&s_bar, 1);
    if (FIM)
        for (int i = tid; i < B * B; i += G::THREADS) s_check[i] = 0;
    __syncthreads();

    GHCM_PROF_BEGIN(t_kernel);
    uint32_t parity = 0u;
    bool tma_pending = false;
    uint32_t cur = 0u;
    unsigned long long solves = 0ull;
    for (;;) {
        if (blockIdx.x == 0) {
            GHCM_PROF_BEGIN(t_sel);
            select_phase<G::THREADS>(s, cur, s_hist, s_sel);
            GHCM_PROF_END(ctl, 2, t_sel);
        }
        GHCM_PROF_BEGIN(t_b0);
        bool const ok0 = grid_barrier(bw, &ctl->error, s.timeout_ns);
        GHCM_PROF_END(ctl, 0, t_b0);
        if (!ok0) break;
        if (ld_relaxed(&ctl->stop)) break;
        uint32_t const nj = ld_relaxed(&ctl->job_count);
        if (nj == 0u) {
            GHCM_PROF_BEGIN(t_res);
            residual_pass<B>(s, cur ^ 1u);
            GHCM_PROF_END(ctl, 4, t_res);
            if (!grid_barrier(bw, &ctl->error, s.timeout_ns)) break;
            if (ld_relaxed(&ctl->count[cur ^ 1u]) == 0u) break;  // converged
            if (blockIdx.x == 0 && tid == 0) ctl->residual_passes += 1u;
            cur ^= 1u;
            continue;
        }
        const uint32_t* jobs = ld_relaxed(&ctl->jobs_in_list) ? s.list[cur] : s.jobs;
        for (;;) {
            if (tid == 0) s_word[2] = atomicAdd(&ctl->job_next, 1u);
            __syncthreads();
            uint32_t const j = s_word[2];
            __syncthreads();
            if (j >= nj) break;
            GHCM_PROF_BEGIN(t_solve);
            solve_tile<B, FIM>(s, __ldcg(&jobs[j]), cur ^ 1u, sm, &s_bar, parity, tma_pending, s_check, s_word,
                               s_red);
            GHCM_PROF_END(ctl, 1, t_solve);
            ++solves;
        }
        GHCM_PROF_BEGIN(t_b1);
        bool const ok1 = grid_barrier(bw, &ctl->error, s.timeout_ns);
        GHCM_PROF_END(ctl, 0, t_b1);
        if (!ok1) break;
        cur ^= 1u;
    }
    if (tid == 0 && solves) atomicAdd(&ctl->block_solves, solves);
    if (blockIdx.x == 0) {
        GHCM_PROF_END(ctl, 5, t_kernel);
    }
    // A TMA copy still in flight after a timed-out wait: give it a bounded
    // chance to land before the CTA's shared memory is released.
    if (tid == 0 && tma_pending) (void)mbar_wait(&s_bar, parity, s.timeout_ns);
}

// ---------------------------------------------------------------------------
// Initialisation kernels (src/eikonal_hcm.cpp:189-238).
// ---------------------------------------------------------------------------
__global__ void k_init_tiles(Sched s) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < s.num_tiles; t += gridDim.x * blockDim.x) {
        s.flags[t] = 0u;
        s.key[t] = inf_bits();
        s.tmin[t] = f_inf();
    }
}

// time = +inf everywhere; rejects NaN or negative inputs.
__global__ void k_init_field(const Inst* insts, uint32_t inst, Ctl* ctl) {
    Inst const I = insts[inst];
    size_t const n = static_cast<size_t>(I.w) * I.h;
    bool bad = false;
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        float const v = __ldg(&I.in[i]);
        bad |= !(v >= 0.f);
        I.time[i] = f_inf();
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&ctl->error, kErrBadInput);
}

// Seeds: time 0, and the tiles of their 4-neighbours become active with key 0
// (seed_map and the initial heap, src/eikonal_hcm.cpp:198-238).
__global__ void k_init_seeds(Sched s, const uint32_t* seeds, const uint32_t* seed_inst, uint32_t n_seeds,
                             int block) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_seeds; i += gridDim.x * blockDim.x) {
        uint32_t const ii = seed_inst ? seed_inst[i] : 0u;
        const Inst& I = s.insts[ii];
        uint32_t const x = seeds[2 * i], y = seeds[2 * i + 1];
        if (x >= I.w || y >= I.h) {
            atomicOr(&s.ctl->error, kErrBadSeed);
            continue;
        }
        I.time[static_cast<size_t>(y) * I.w + x] = 0.f;
    }
}

__global__ void k_activate_seeds(Sched s, const uint32_t* seeds, const uint32_t* seed_inst, uint32_t n_seeds,
                                 int block) {
    constexpr int dir[4][2] = {{-1, 0}, {0, -1}, {1, 0}, {0, 1}};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_seeds; i += gridDim.x * blockDim.x) {
        uint32_t const ii = seed_inst ? seed_inst[i] : 0u;
        const Inst& I = s.insts[ii];
        int const x = static_cast<int>(seeds[2 * i]), y = static_cast<int>(seeds[2 * i + 1]);
        if (x >= static_cast<int>(I.w) || y >= static_cast<int>(I.h)) continue;
        for (auto const& d : dir) {
            int const px = x + d[0], py = y + d[1];
            if (px < 0 || py < 0 || px >= static_cast<int>(I.w) || py >= static_cast<int>(I.h)) continue;
            uint32_t const tile = I.tile_base + static_cast<uint32_t>(py / block) * I.tiles_x + px / block;
            s.tmin[tile] = 0.f;
            activate(s, tile, 0u, 0.f, 0u);
        }
    }
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

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
template <int B, bool FIM>
static void* kernel_ptr() {
    return reinterpret_cast<void*>(&k_persistent<B, FIM>);
}

static void* select_kernel(int block, int fim) {
    switch (block) {
        case 8: return fim ? kernel_ptr<8, true>() : kernel_ptr<8, false>();
        case 16: return fim ? kernel_ptr<16, true>() : kernel_ptr<16, false>();
        case 32: return fim ? kernel_ptr<32, true>() : kernel_ptr<32, false>();
        default: return nullptr;
    }
}

static int threads_for(int block) {
    switch (block) {
        case 8: return TileGeom<8>::THREADS;
        case 16: return TileGeom<16>::THREADS;
        case 32: return TileGeom<32>::THREADS;
        default: return 0;
    }
}

int query_persistent(int block, int fim, LaunchInfo* info) {
    void* k = select_kernel(block, fim);
    if (!k) return -1;
    int bps = 0;
    int const threads = threads_for(block);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, threads, 0) != cudaSuccess) return -2;
    info->threads = threads;
    info->blocks_per_sm = bps;
    return 0;
}

cudaError_t launch_init(const Sched& s, const Inst* h_insts, uint32_t n_insts, const uint32_t* d_seeds,
                        const uint32_t* d_seed_inst, uint32_t n_seeds, int block, cudaStream_t st) {
    unsigned const tb = 256;
    unsigned const tiles_grid = static_cast<unsigned>(std::min<uint32_t>((s.num_tiles + tb - 1) / tb, 4096u));
    k_init_tiles<<<std::max(1u, tiles_grid), tb, 0, st>>>(s);
    for (uint32_t i = 0; i < n_insts; ++i) {
        size_t const cells = static_cast<size_t>(h_insts[i].w) * h_insts[i].h;
        unsigned const g = static_cast<unsigned>(std::min<size_t>((cells + tb - 1) / tb, 152u * 16u));
        k_init_field<<<std::max(1u, g), tb, 0, st>>>(s.insts, i, s.ctl);
    }
    if (n_seeds) {
        unsigned const sb = 128;
        unsigned const g = static_cast<unsigned>(std::min<uint32_t>((n_seeds + sb - 1) / sb, 1024u));
        k_init_seeds<<<g, sb, 0, st>>>(s, d_seeds, d_seed_inst, n_seeds, block);
        k_activate_seeds<<<g, sb, 0, st>>>(s, d_seeds, d_seed_inst, n_seeds, block);
    }
    return cudaGetLastError();
}

cudaError_t launch_persistent(int block, int fim, const Sched& s, int grid, cudaStream_t st) {
    void* k = select_kernel(block, fim);
    if (!k) return cudaErrorInvalidValue;
    void* args[] = {const_cast<Sched*>(&s)};
    return cudaLaunchCooperativeKernel(k, dim3(grid), dim3(threads_for(block)), args, 0, st);
}

cudaError_t launch_wait_selftest(uint32_t* flag, Ctl* ctl, uint64_t timeout_ns, cudaStream_t st) {
    k_wait_selftest<<<1, 32, 0, st>>>(flag, ctl, timeout_ns);
    return cudaGetLastError();
}

}  // namespace ghcm

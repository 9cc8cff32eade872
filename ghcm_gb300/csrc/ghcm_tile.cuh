// Block-solves, one tile per CTA.
//
// A CTA stages its tile with a two-cell halo (time and speed/cost) into
// shared memory - one 2-D TMA box load each, or plain loads when the field's
// layout does not allow TMA - and every thread owns one (B <= 16) or four
// (B = 32) cells of the tile.
//
//   systolic  every sweep updates the cells in place (each thread its own,
//             reading its four neighbours from shared memory) until a sweep
//             moves no cell by more than eps; the reference sweeps
//             work-group-sized chunks the same way
//             (data/eikonal_ghcm_systolic.cl:130-153).
//   block-FIM only open cells are solved; a converged cell asks its in-tile
//             neighbours to re-check and a neighbour that improves by more
//             than eps opens (data/eikonal_ghcm_fim.cl:166-210, 347-372).
//             The initial open set is the rows of the edges neighbours
//             flagged (fim.cl:306-332), the cells next to seeds and, for tiles
//             re-queued by the residual check, every cell.
//
// Then each neighbour edge row is probed with the converged tile
// (check_border, data/eikonal_ghcm_systolic.cl:8-41) - probe-only, as
// data/eikonal_ghcm_fim.cl:175-194 does, so no tile writes into another.
// The probe recomputes the neighbour's own update exactly: the second halo
// ring supplies the cell beyond the probed one (the reference treats it as
// +inf, data/eikonal_common.cl:199-206). A neighbour is activated only when
// the probe improves it by more than eps AND this solve changed the edge row
// facing it; with rounding the Godunov update is not monotone, and without
// the second condition two converged tiles can keep activating each other.
#pragma once

#include <type_traits>

#include "ghcm_learn.cuh"

namespace ghcm {

template <int B>
struct TileGeom {
    static constexpr int THREADS = (B * B < 64) ? 64 : (B * B > 256 ? 256 : B * B);
    static constexpr int CPT = (B * B) / THREADS;  // cells per thread
    static constexpr int ROWS_PER_PASS = THREADS / B;
    static constexpr int BW = B + 8;               // staged box width: x in [ox-4, ox+B+4), 16-byte aligned start
    static constexpr int BH = B + 4;               // staged box height: y in [oy-2, oy+B+2)
    static constexpr int BOX = BW * BH;
    static constexpr int BOXP = (BOX + 31) / 32 * 32;  // keeps each box 128-byte aligned for TMA
    static constexpr int RING = (B + 4) * (B + 4);      // the tile and its two halo rings
    static_assert(4 * B % 32 == 0, "edge probes need whole warps");
    static_assert(B * B % THREADS == 0, "cells must divide evenly");
    static_assert(B <= 32, "row masks are 32 bits");
};

template <int B>
struct alignas(128) TileSmem {
    float time[TileGeom<B>::BOXP];
    float cost[TileGeom<B>::BOXP];
    uint8_t check[B * B];  // block-FIM: re-check requests
    float feat[kFeatures]; // trace recorder: features of the current solve
    uint32_t queued[4];    // learned score policy: neighbour queued across edge e, or kNone
    uint32_t queued_pos[4];  // and its entry in the next active list
    QueuedState queued_state[4];  // and its state for the scorer
};

constexpr uint32_t kNone = 0xffffffffu;

// index of local cell (x, y), x in [-4, B+4), y in [-2, B+2), in a staged box
template <int B>
__device__ __forceinline__ int si(int x, int y) {
    return (y + 2) * TileGeom<B>::BW + x + 4;
}

// Outcome of a claimed job.
enum : int { kJobFailed = 0, kJobSolved = 1, kJobDeferred = 2 };

// One block-solve of `tile`; activations go to list[nxt]. Returns kJobSolved,
// kJobDeferred (the learned schedule's veto put it back in the active set) or
// kJobFailed if the TMA stage timed out (the grid then stops at the next
// barrier).
// NORMAL: the systolic sweep loop with the update's cases unfolded and a
// short-root copy for tiles of normal costs; the 32-register wide builds,
// where its extra registers spill, keep the plain loop.
template <int B, bool FIM, bool NORMAL = true>
__device__ int solve_tile(const Sched& s, uint32_t tile, uint32_t nxt, TileSmem<B>& sm, uint64_t* bar,
                           uint32_t& parity, bool& tma_pending, uint32_t* s_word, float* s_red, uint32_t* s_krange,
                           uint32_t wave, uint32_t epoch, uint32_t pbit) {
    using G = TileGeom<B>;
    int const tid = threadIdx.x;
    uint32_t const ii = inst_of(s, tile);
    const Inst& I = s.insts[ii];
    TileCoord const tc = tile_coord<B>(I, tile);
    bool const use_tma = I.tma != 0;

#ifdef GHCM_PROFILE
    uint64_t const p_t0 = (tid == 0) ? global_ns() : 0ull;
#endif
    // Claim: clear the tile's activation state (a later activation re-queues
    // it), and stage the tile with its halo.
    if (tid == 0) {
        // checked builds: the tile lies in its instance and the box starts on a
        // 16-byte boundary; otherwise nothing is staged and the job fails
        bool const tile_ok = GHCM_CHECK(s.ctl, ii < s.num_insts && tc.sx > 0 && tc.sy > 0, 1u);
        bool const x_ok = GHCM_CHECK(s.ctl, ((tc.ox - 4) & 3) == 0, 2u);
        bool const tma_go = tile_ok && x_ok && use_tma;
        // The TMA stage goes out before the claim, so that the two round trips
        // overlap. What the tile and its halo held before this phase is
        // visible already: the wave barrier acquired it. Newer data comes only
        // from a neighbour solved in this phase, and a neighbour that changed
        // the halo activates the tile with this phase's bit (pbit) after its
        // stores; if the claim finds that bit, it has acquired those stores and
        // the time box is loaded again below. A neighbour that activates the
        // tile after the claim re-queues it, as before.
        if (tma_go) {
            fence_proxy_async();
            mbar_arrive_expect_tx(bar, static_cast<uint32_t>(2 * G::BOX * sizeof(float)));
            tma_load_2d(sm.time, time_map(s, ii), bar, tc.ox - 4, tc.oy - 2);
            tma_load_2d(sm.cost, in_map(s, ii), bar, tc.ox - 4, tc.oy - 2);
            tma_pending = true;
        }
        // Both atomics in flight at once. The key is reset first: an activation
        // landing between the two leaves a lower key on an idle tile (it is
        // only a priority), while its data reaches this solve: the flag clear
        // acquires it, and its phase bit has the time box loaded again.
        uint32_t const kmx0 = learn_claim_kmax(s, tile);
        uint32_t const kold = atomicExch(&s.key[tile], inf_bits());
        uint32_t const f = atom_and_acquire(&s.flags[tile], ~(kActive | kFull | kEdgeMask | kActPhaseMask));
        uint32_t const kmx = learn_claim(s, tile, f, kold, kmx0, wave, sm.feat);
        s_word[0] = f;
        s_word[1] = 0u;  // abort flag
        s_word[2] = (tma_go && (f & pbit)) ? 1u : 0u;  // load the time box again after the claim
        s_word[4] = 0u;  // edge rows changed by this solve
        s_word[5] = kold;
#pragma unroll
        for (int e = 0; e < 4; ++e) sm.queued[e] = kNone;
        s_word[6] = kmx;
        s_word[3] = (tile_ok && x_ok) ? 0u : 1u;  // 1: nothing staged (written only here)
    }
    __syncthreads();
    uint32_t const flags = s_word[0];
    // learned schedule, veto mode: warp 0 scores the tile while its stage is in flight
    bool const may_veto = s.learn.veto && s.learn.params;
    if (may_veto) {
        if (tid < 32) {
            bool const v = learn_veto_warp(s, tile, flags, s_word[5], s_word[6], wave);
            if (tid == 0) s_word[7] = v ? 1u : 0u;
        }
        __syncthreads();
    }
    bool const vetoed = may_veto && s_word[7] != 0u;
    bool const staged = s_word[3] == 0u;
    if (use_tma && staged) {
        if (!mbar_wait(bar, parity, s.timeout_ns)) {
            atomicOr(&s.ctl->error, kErrTimeout);
            s_word[1] = 1u;  // every thread acts on it after the barrier below
        } else if (tid == 0) {
            tma_pending = false;
        }
        parity ^= 1u;
    }
    if (vetoed) {
        __syncthreads();
        if (s_word[1] || !staged) return kJobFailed;
        if (tid == 0) learn_defer(s, tile, flags, s_word[5], s_word[6], nxt, s_krange);
        __syncthreads();
        return kJobDeferred;
    }
    if (s_word[2]) {
        // a neighbour solved in this phase activated the tile before the claim:
        // its stores, acquired by the claim, may postdate the box loaded above
        __syncthreads();  // every thread has passed the wait above
        if (!s_word[1]) {
            if (tid == 0) {
                fence_proxy_async();
                mbar_arrive_expect_tx(bar, static_cast<uint32_t>(G::BOX * sizeof(float)));
                tma_load_2d(sm.time, time_map(s, ii), bar, tc.ox - 4, tc.oy - 2);
                tma_pending = true;
            }
            if (!mbar_wait(bar, parity, s.timeout_ns)) {
                atomicOr(&s.ctl->error, kErrTimeout);
                s_word[1] = 1u;
            } else if (tid == 0) {
                tma_pending = false;
            }
            parity ^= 1u;
        }
    }
    // fill / fix up the two rings: outside the field is +inf; speed -> cost
    for (int r = tid; r < G::RING; r += G::THREADS) {
        int const lx = r % (B + 4) - 2, ly = r / (B + 4) - 2;
        int const gx = tc.ox + lx, gy = tc.oy + ly;
        int const k = si<B>(lx, ly);
        bool const in = gx >= 0 && gy >= 0 && gx < static_cast<int>(I.w) && gy < static_cast<int>(I.h);
        if (!GHCM_CHECK(s.ctl, k >= 0 && k < G::BOX, 3u)) continue;
        if (!in) {
            sm.time[k] = f_inf();
            sm.cost[k] = f_inf();
        } else if (use_tma) {
            sm.cost[k] = to_cost(I, sm.cost[k]);
        } else {
            size_t const gi = static_cast<size_t>(gy) * I.w + gx;
            sm.time[k] = __ldcg(&I.time[gi]);
            sm.cost[k] = to_cost(I, __ldg(&I.in[gi]));
        }
    }
    __syncthreads();
    if (s_word[1] || !staged) return kJobFailed;
#ifdef GHCM_PROFILE
    uint64_t const p_t1 = (tid == 0) ? global_ns() : 0ull;
#endif

    constexpr int BW = G::BW;
    float t[G::CPT], t0[G::CPT], c[G::CPT], c2[G::CPT];
    int idx[G::CPT], lxs[G::CPT], lys[G::CPT];
    bool v[G::CPT], inside[G::CPT];
#pragma unroll
    for (int k = 0; k < G::CPT; ++k) {
        int const id = tid + k * G::THREADS;
        lxs[k] = id % B;
        lys[k] = id / B;
        inside[k] = lxs[k] < tc.sx && lys[k] < tc.sy;
        idx[k] = si<B>(lxs[k], lys[k]);
        if (!GHCM_CHECK(s.ctl, idx[k] - BW >= 0 && idx[k] + BW < G::BOX, 4u)) idx[k] = si<B>(0, 0);
        t[k] = sm.time[idx[k]];
        t0[k] = t[k];
        c[k] = sm.cost[idx[k]];
        c2[k] = __fmul_rn(__fmul_rn(c[k], c[k]), 2.0f);
        v[k] = inside[k] && c[k] < f_inf() && t[k] != 0.f;  // a time of 0 is a seed: fixed
    }
    float const eps = s.eps;
    // Rounding makes the update slightly non-monotone, so keeping the minimum
    // of every evaluation (the reference's min(T_old, update)) leaves a cell
    // an ulp low wherever one evaluation rounded low, and along a long front
    // those ulps add up; a block-solve evaluates each cell ~B times. So the
    // sweeps recompute each cell from its neighbours, bounded by the cell's
    // value when this solve began (kUpdInSolve: nothing rises above what
    // neighbours saw). Until the tile has had `refresh` quiet block-solves
    // (solves that moved no cell far, falls_far) the bound is dropped
    // (kUpdFresh: a value an earlier solve rounded low rises again and the
    // neighbours are told). Past fresh_sweeps sweeps, and for the reference
    // form, cells only fall (kUpdKeepMin); the limits end the one-ulp
    // oscillations of nearly tied neighbours. The last sweep before the sweep
    // cap is always lower-only, so a solve the cap stops has lowered some cell
    // by more than eps in that sweep: re-queues by the cap make progress and
    // end (an oscillation that only ever returns to its start cannot hold a
    // tile). A capped solve also spends the refresh budget.
    int mode = solve_count(flags) < s.refresh ? kUpdFresh : (s.in_solve ? kUpdInSolve : kUpdKeepMin);
    uint32_t const fresh_sweeps = min(4u * B, s.max_sweeps - 1u);
    if (fresh_sweeps == 0u) mode = kUpdKeepMin;  // a cap of one sweep
    bool own_changed = false;
    bool capped = false;
    uint32_t sweeps = 0;

    if (!FIM && NORMAL) {
        // The sweep loop, with next_time and moves unfolded for the solve: b0
        // is a cell's bound before the lower-only phase (+inf fresh, t0 in
        // solve), keep says the phase has begun. A tile whose updatable costs
        // are all normal_cost runs the update with the short square root.
        float b0[G::CPT];
        bool ok = true;
#pragma unroll
        for (int k = 0; k < G::CPT; ++k) {
            b0[k] = (mode == kUpdFresh) ? f_inf() : t0[k];
            ok &= !v[k] || normal_cost(c[k]);
        }
        bool keep = mode == kUpdKeepMin;
        auto sweep_loop = [&](auto normal) {
            for (;;) {
                bool moved = false;
#pragma unroll
                for (int k = 0; k < G::CPT; ++k) {
                    if (!v[k]) continue;
                    int const i = idx[k];
                    float const ax = fminf(sm.time[i - 1], sm.time[i + 1]);
                    float const ay = fminf(sm.time[i - BW], sm.time[i + BW]);
                    float const raw = decltype(normal)::value ? godunov2_raw_normal(ax, ay, c[k], c2[k])
                                                              : godunov2_raw(ax, ay, c[k], c2[k]);
                    float const nt = fminf(keep ? t[k] : b0[k], raw);
                    if (nt != t[k]) {
                        float const d = __fsub_rn(nt, t[k]);  // nt != t: moves() without its equal case
                        moved |= keep ? d < -eps : fabsf(d) > eps;
                        t[k] = nt;
                        sm.time[i] = nt;
                        own_changed = true;
                    }
                }
                ++sweeps;
                if (!__syncthreads_or(moved)) break;
                if (sweeps >= fresh_sweeps) keep = true;
                if (sweeps >= s.max_sweeps) {
                    capped = true;
                    break;
                }
            }
        };
        if (__syncthreads_and(ok))
            sweep_loop(std::true_type{});
        else
            sweep_loop(std::false_type{});
    } else if (!FIM) {
        for (;;) {
            bool moved = false;
#pragma unroll
            for (int k = 0; k < G::CPT; ++k) {
                if (!v[k]) continue;
                int const i = idx[k];
                float const ax = fminf(sm.time[i - 1], sm.time[i + 1]);
                float const ay = fminf(sm.time[i - BW], sm.time[i + BW]);
                float const nt = next_time(godunov2_raw(ax, ay, c[k], c2[k]), t[k], t0[k], mode);
                if (nt != t[k]) {
                    moved |= moves(nt, t[k], eps, mode != kUpdKeepMin);
                    t[k] = nt;
                    sm.time[i] = nt;
                    own_changed = true;
                }
            }
            ++sweeps;
            if (!__syncthreads_or(moved)) break;
            if (sweeps >= fresh_sweeps) mode = kUpdKeepMin;
            if (sweeps >= s.max_sweeps) {
                capped = true;
                break;
            }
        }
    } else {
        uint8_t* check = sm.check;
        bool open[G::CPT];
        uint32_t const edges = (flags & kEdgeMask) >> 4;
        bool const full = (flags & kFull) != 0u;
#pragma unroll
        for (int k = 0; k < G::CPT; ++k) {
            int const i = idx[k];
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
                    int const i = idx[k];
                    float const ax = fminf(sm.time[i - 1], sm.time[i + 1]);
                    float const ay = fminf(sm.time[i - BW], sm.time[i + BW]);
                    float const nt = next_time(godunov2_raw(ax, ay, c[k], c2[k]), t[k], t0[k], mode);
                    bool moved = false;
                    if (nt != t[k]) {
                        moved = moves(nt, t[k], eps, mode != kUpdKeepMin);
                        t[k] = nt;
                        sm.time[i] = nt;
                        own_changed = true;
                    }
                    if (moved) continue;
                    open[k] = false;  // converged: have the neighbours re-checked
                    int const lx = lxs[k], ly = lys[k];
                    if (lx > 0 && sm.cost[i - 1] < f_inf()) check[ly * B + lx - 1] = 1;
                    if (lx + 1 < tc.sx && sm.cost[i + 1] < f_inf()) check[ly * B + lx + 1] = 1;
                    if (ly > 0 && sm.cost[i - BW] < f_inf()) check[(ly - 1) * B + lx] = 1;
                    if (ly + 1 < tc.sy && sm.cost[i + BW] < f_inf()) check[(ly + 1) * B + lx] = 1;
                }
                __syncthreads();
                bool still_open = false;
#pragma unroll
                for (int k = 0; k < G::CPT; ++k) {
                    if (!v[k]) continue;
                    int const cell = lys[k] * B + lxs[k];
                    if (check[cell]) {
                        check[cell] = 0;
                        if (!open[k]) {
                            int const i = idx[k];
                            float const ax = fminf(sm.time[i - 1], sm.time[i + 1]);
                            float const ay = fminf(sm.time[i - BW], sm.time[i + BW]);
                            float const nt = next_time(godunov2_raw(ax, ay, c[k], c2[k]), t[k], t0[k], mode);
                            if (nt != t[k]) {
                                open[k] = moves(nt, t[k], eps, mode != kUpdKeepMin);
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
                if (sweeps >= fresh_sweeps) mode = kUpdKeepMin;
                if (sweeps >= s.max_sweeps) {
                    capped = true;
                    break;
                }
            }
        }
    }

#ifdef GHCM_PROFILE
    uint64_t const p_t2 = (tid == 0) ? global_ns() : 0ull;
#endif
    // Which edge rows this solve changed (bit e: the row facing neighbour e).
    {
        uint32_t ec = 0u;
#pragma unroll
        for (int k = 0; k < G::CPT; ++k) {
            if (!inside[k] || t[k] == t0[k]) continue;
            if (falls_far(t[k], t0[k])) ec |= 16u;  // not a quiet solve
            if (lxs[k] == 0) ec |= 1u;
            if (lys[k] == 0) ec |= 2u;
            if (lxs[k] == tc.sx - 1) ec |= 4u;
            if (lys[k] == tc.sy - 1) ec |= 8u;
        }
        ec = __reduce_or_sync(0xffffffffu, ec);
        if ((tid & 31) == 0 && ec) atomicOr(&s_word[4], ec);
    }
    // Probe the neighbours' edge rows: edge e, cell ei of that row.
    int const e = tid / B;
    int const ei = tid % B;
    bool e_imp = false;
    float e_key = f_inf();
    int nb = -1;
    if (tid < 4 * B) {
        nb = neighbour_tile(I, tc.tx, tc.ty, e);
        int const len = (e & 1) ? tc.sx : tc.sy;
        if (nb >= 0 && ei < len) {
            int px, py, qx, qy, fx, fy;
            if (e == 0) { px = -1; py = ei; qx = 0; qy = ei; fx = -2; fy = ei; }
            else if (e == 1) { px = ei; py = -1; qx = ei; qy = 0; fx = ei; fy = -2; }
            else if (e == 2) { px = tc.sx; py = ei; qx = tc.sx - 1; qy = ei; fx = tc.sx + 1; fy = ei; }
            else { px = ei; py = tc.sy; qx = ei; qy = tc.sy - 1; fx = ei; fy = tc.sy + 1; }
            int const pi = si<B>(px, py);
            int const fi = si<B>(fx, fy);
            bool const in_box = GHCM_CHECK(s.ctl, pi - BW >= 0 && pi + BW < G::BOX && fi >= 0 && fi < G::BOX, 5u);
            float const cp = in_box ? sm.cost[pi] : f_inf();
            float const told = in_box ? sm.time[pi] : 0.f;
            if (cp < f_inf() && told != 0.f) {  // seeds never change
                float const a_norm = fminf(sm.time[si<B>(qx, qy)], sm.time[fi]);
                float const a_lat = (e & 1) ? fminf(sm.time[pi - 1], sm.time[pi + 1])
                                            : fminf(sm.time[pi - BW], sm.time[pi + BW]);
                bool const track_rise = s.refresh != 0u;
                float const nt = next_time(godunov_raw(a_norm, a_lat, cp), told, told, track_rise ? kUpdFresh : kUpdKeepMin);
                if (moves(nt, told, eps, track_rise)) {
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

    // Commit the tile and its smallest time.
    bool const tile_changed = __syncthreads_or(own_changed) != 0;
    bool useful = false;  // some cell moved by more than eps (the trace label)
    if (s.learn.tstat) {
        bool mv = false;
#pragma unroll
        for (int k = 0; k < G::CPT; ++k) mv |= inside[k] && moves(t[k], t0[k], eps, true);
        useful = __syncthreads_or(mv) != 0;
    }
    float lmin = f_inf();
#pragma unroll
    for (int k = 0; k < G::CPT; ++k) {
        if (!inside[k]) continue;
        lmin = fminf(lmin, t[k]);
        size_t const gi = static_cast<size_t>(tc.oy + lys[k]) * I.w + tc.ox + lxs[k];
        if (tile_changed && GHCM_CHECK(s.ctl, gi < static_cast<size_t>(I.w) * I.h, 6u)) I.time[gi] = t[k];
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) lmin = fminf(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
    if ((tid & 31) == 0) s_red[tid >> 5] = lmin;
    __syncthreads();
    // the barrier above gathers every thread's tile stores; an activation is a
    // release, so the neighbour that consumes it stages them
    if (tid == 0) {
        float m = s_red[0];
        for (int w = 1; w < G::THREADS / 32; ++w) m = fminf(m, s_red[w]);
        s.tmin[tile] = m;
        if (tile_changed) s.epoch[tile] = epoch;  // the next residual pass re-checks it and its neighbours
        if (solve_count(flags) < s.refresh && (capped || !(s_word[4] & 16u))) atomicAdd(&s.flags[tile], kSolveOne);
        learn_commit(s, tile, useful, wave, sweeps, sm.feat);
        if (capped) activate(s, tile, kFull, m, nxt, s_krange, 0u);
    }
    uint32_t const edge_changed = s_word[4];
    bool const scoring = s.learn.params && !s.learn.veto;  // learned score policy
    if (tid < 4 * B && ei == 0 && e_imp && ((edge_changed >> e) & 1u) &&
        GHCM_CHECK(s.ctl, nb >= 0 && static_cast<uint32_t>(nb) < s.num_tiles, 7u)) {
        uint32_t const pos =
            activate(s, static_cast<uint32_t>(nb), kEdgeBit0 << ((e + 2) & 3), e_key, nxt, s_krange, pbit, [&]() {
                if (scoring)
                    sm.queued_state[e].load(s, I, static_cast<uint32_t>(nb), tc.tx + (e == 2) - (e == 0),
                                            tc.ty + (e == 3) - (e == 1));
            });
        if (pos != kNoPos) {  // appended now: score it (a re-activation keeps its entry's score)
            sm.queued[e] = static_cast<uint32_t>(nb);
            sm.queued_pos[e] = pos;
        }
    }
    if (scoring) {  // score what this solve queued, a warp per tile
        __syncthreads();
        for (int q = tid >> 5; q < 4; q += G::THREADS / 32)
            if (sm.queued[q] != kNone) score_queued_warp(s, sm.queued_state[q], nxt, sm.queued_pos[q], wave + 1u);
    }
#ifdef GHCM_PROFILE
    if (tid == 0) {
        uint64_t const p_t3 = global_ns();
        atomicAdd(&s.ctl->prof[10], static_cast<unsigned long long>(p_t1 - p_t0));
        atomicAdd(&s.ctl->prof[11], static_cast<unsigned long long>(p_t2 - p_t1));
        atomicAdd(&s.ctl->prof[12], static_cast<unsigned long long>(p_t3 - p_t2));
        atomicAdd(&s.ctl->prof[13], 1ull);
        atomicMax(&s.ctl->prof[18], static_cast<unsigned long long>(p_t3 - p_t0));  // longest solve of the wave
        atomicAdd(&s.ctl->prof[3], static_cast<unsigned long long>(sweeps));
        atomicMax(&s.ctl->wave_max_sweeps, sweeps);
    }
#endif
    __syncthreads();
    return kJobSolved;
}

// Global residual check, one tile per warp: re-activates every tile holding
// a cell whose Godunov update would still move it by more than eps. Pass
// `pass` (1-based) re-checks only tiles that changed, or have a neighbour that
// changed, since the pass before it (epoch >= pass): a cell's update reads
// only the cell and its four neighbours, so a tile with no change around it
// keeps the residual the previous pass found clean. The reference has no such
// check (src/eikonal_hcm.cpp:343, 486-488).
template <int B>
__device__ void residual_warp(const Sched& s, uint32_t nxt, uint32_t warp_global, uint32_t warps, uint32_t* s_krange,
                              uint32_t pass) {
    int const lane = threadIdx.x & 31;
    for (uint32_t tile = warp_global; tile < s.num_tiles; tile += warps) {
        const Inst& I = s.insts[inst_of(s, tile)];
        TileCoord const tc = tile_coord<B>(I, tile);
        {
            uint32_t ep = 0u;
            if (lane < 4) {
                int const nb = neighbour_tile(I, tc.tx, tc.ty, lane);
                if (nb >= 0) ep = __ldcg(&s.epoch[nb]);
            } else if (lane == 4) {
                ep = __ldcg(&s.epoch[tile]);
            }
            if (!__any_sync(0xffffffffu, ep >= pass)) continue;
        }
        bool const fresh = solve_count(ld_relaxed(&s.flags[tile])) < s.refresh;
        bool bad = false;
        float kmin = f_inf();
        for (int k = lane; k < B * B; k += 32) {
            int const lx = k % B, ly = k / B;
            if (lx >= tc.sx || ly >= tc.sy) continue;
            int const gx = tc.ox + lx, gy = tc.oy + ly;
            size_t const gi = static_cast<size_t>(gy) * I.w + gx;
            if (!GHCM_CHECK(s.ctl, gi < static_cast<size_t>(I.w) * I.h, 8u)) continue;
            float const cst = to_cost(I, __ldg(&I.in[gi]));
            if (!(cst < f_inf())) continue;
            float const t = __ldcg(&I.time[gi]);
            if (t == 0.f) continue;  // seed
            float const xl = gx > 0 ? __ldcg(&I.time[gi - 1]) : f_inf();
            float const xr = gx + 1 < static_cast<int>(I.w) ? __ldcg(&I.time[gi + 1]) : f_inf();
            float const yu = gy > 0 ? __ldcg(&I.time[gi - I.w]) : f_inf();
            float const yd = gy + 1 < static_cast<int>(I.h) ? __ldcg(&I.time[gi + I.w]) : f_inf();
            float const nt = next_time(godunov_raw(fminf(xl, xr), fminf(yu, yd), cst), t, t, fresh ? kUpdFresh : kUpdKeepMin);
            if (moves(nt, t, s.eps, fresh)) {
                bad = true;
                kmin = fminf(kmin, fminf(nt, t));
            }
        }
        if (__any_sync(0xffffffffu, bad)) {
#pragma unroll
            for (int o = 16; o >= 1; o >>= 1) kmin = fminf(kmin, __shfl_xor_sync(0xffffffffu, kmin, o));
            if (lane == 0) activate(s, tile, kFull, kmin, nxt, s_krange, 0u);
        }
    }
}

}  // namespace ghcm

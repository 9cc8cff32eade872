// Block-solves with one warp per tile (systolic kernel; used for B = 8).
//
// Lane l of the warp owns column x = l % B of row band g = l / B of the tile
// (R = B*B/32 rows: 2 for B = 8, 8 for B = 16) and keeps its R cells in
// registers. A sweep updates all of them at once from the values of the
// previous sweep (Jacobi): the neighbours left and right are one warp shuffle
// away, the ones above and below are in the lane's own registers or one
// shuffle across bands, and the tile's halo - fixed during the solve - is
// read from the staged box in shared memory. The R updates of a lane are
// independent, so a sweep is a few hundred instructions with no CTA barrier;
// each warp is an independent worker and a wave's tiles all run at once.
//
// The staging (TMA box with a two-cell halo), the exact edge probe, the edge-
// change gating of activations and the commit are those of the CTA solver
// (ghcm_tile.cuh), done by one warp.
#pragma once

#include "ghcm_tile.cuh"

namespace ghcm {

template <int B>
struct WarpTileGeom {
    static constexpr int G = 32 / B;       // row bands per tile
    static constexpr int R = B / G;        // rows per lane
    static constexpr int NW = 8;           // warps (tile workers) per CTA
    static constexpr int THREADS = NW * 32;
    static_assert(B == 8 || B == 16, "warp tiles cover B = 8 and 16");
};

template <int B>
struct alignas(128) WarpTileSmem {
    float time[TileGeom<B>::BOXP];
    float cost[TileGeom<B>::BOXP];
    float feat[kFeatures];
    uint32_t claim[4];  // flags, key, largest activation key of the claimed tile
    uint64_t bar;
};

// One block-solve of `tile` by the calling warp. Returns kJobSolved,
// kJobDeferred (vetoed by the learned schedule) or kJobFailed (the TMA stage
// timed out).
template <int B>
__device__ int solve_tile_warp(const Sched& s, uint32_t tile, uint32_t nxt, WarpTileSmem<B>& sm, uint32_t& parity,
                                bool& tma_pending, uint32_t* s_krange, uint32_t wave, uint32_t epoch,
                                uint32_t pbit) {
    using G = TileGeom<B>;
    using W = WarpTileGeom<B>;
    constexpr unsigned FULL = 0xffffffffu;
    constexpr int R = W::R;
    int const lane = threadIdx.x & 31;
    int const x = lane % B;
    int const band = lane / B;
    uint32_t const ii = inst_of(s, tile);
    const Inst& I = s.insts[ii];
    TileCoord const tc = tile_coord<B>(I, tile);
    bool const use_tma = I.tma != 0;

    // Claim and stage.
    if (lane == 0) {
        uint32_t const kmx0 = learn_claim_kmax(s, tile);
        uint32_t const kold = atomicExch(&s.key[tile], inf_bits());  // all in flight, as in solve_tile
        uint32_t const f = atom_and_acquire(&s.flags[tile], ~(kActive | kFull | kEdgeMask | kActPhaseMask));
        uint32_t const kmx = learn_claim(s, tile, f, kold, kmx0, wave, sm.feat);
        sm.claim[0] = f;
        sm.claim[1] = kold;
        sm.claim[2] = kmx;
        bool const x_ok = GHCM_CHECK(s.ctl, ((tc.ox - 4) & 3) == 0, 11u);  // x on a 16-byte boundary
        sm.claim[3] = x_ok ? 1u : 0u;  // 0 (checked builds only): nothing staged, the job fails
        if (use_tma && x_ok) {
            fence_proxy_async();
            mbar_arrive_expect_tx(&sm.bar, static_cast<uint32_t>(2 * G::BOX * sizeof(float)));
            tma_load_2d(sm.time, time_map(s, ii), &sm.bar, tc.ox - 4, tc.oy - 2);
            tma_load_2d(sm.cost, in_map(s, ii), &sm.bar, tc.ox - 4, tc.oy - 2);
            tma_pending = true;
        }
    }
    __syncwarp();
    bool const vetoed = learn_veto_warp(s, tile, sm.claim[0], sm.claim[1], sm.claim[2], wave);
    if (sm.claim[3] == 0u) return kJobFailed;
    if (use_tma) {
        bool const landed = mbar_wait(&sm.bar, parity, s.timeout_ns);
        parity ^= 1u;
        if (!__all_sync(FULL, landed)) {
            if (lane == 0) atomicOr(&s.ctl->error, kErrTimeout);
            return kJobFailed;
        }
        if (lane == 0) tma_pending = false;
    }
    if (vetoed) {
        if (lane == 0) learn_defer(s, tile, sm.claim[0], sm.claim[1], sm.claim[2], nxt, s_krange);
        __syncwarp();
        return kJobDeferred;
    }
    for (int r = lane; r < G::RING; r += 32) {
        int const lx = r % (B + 4) - 2, ly = r / (B + 4) - 2;
        int const gx = tc.ox + lx, gy = tc.oy + ly;
        int const k = si<B>(lx, ly);
        bool const in = gx >= 0 && gy >= 0 && gx < static_cast<int>(I.w) && gy < static_cast<int>(I.h);
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
    __syncwarp();

    float t[R], t0[R], c[R], c2[R];
    bool fix[R];  // seeds (time 0) and walls keep their value
#pragma unroll
    for (int k = 0; k < R; ++k) {
        int const i = si<B>(x, band * R + k);
        t[k] = sm.time[i];
        t0[k] = t[k];
        c[k] = sm.cost[i];
        c2[k] = __fmul_rn(__fmul_rn(c[k], c[k]), 2.0f);
        fix[k] = t[k] == 0.f || !(c[k] < f_inf());
    }
    float const h_top = sm.time[si<B>(x, -1)];  // used by band 0
    float const h_bot = sm.time[si<B>(x, B)];   // used by the last band
    float const eps = s.eps;
    // how sweeps bound the update (see solve_tile)
    int mode = solve_count(sm.claim[0]) < s.refresh ? kUpdFresh : (s.in_solve ? kUpdInSolve : kUpdKeepMin);
    uint32_t const fresh_sweeps = min(4u * B, s.max_sweeps - 1u);  // see solve_tile
    if (fresh_sweeps == 0u) mode = kUpdKeepMin;
    bool changed = false;
    bool capped = false;
    uint32_t sweeps = 0;
    for (;;) {
        float nt[R];
        float const up_in = __shfl_up_sync(FULL, t[R - 1], B);    // last row of the band above
        float const down_in = __shfl_down_sync(FULL, t[0], B);    // first row of the band below
        bool moved = false;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            float l = __shfl_up_sync(FULL, t[k], 1, B);
            float r = __shfl_down_sync(FULL, t[k], 1, B);
            if (x == 0) l = sm.time[si<B>(-1, band * R + k)];
            if (x == B - 1) r = sm.time[si<B>(B, band * R + k)];
            float const u = (k > 0) ? t[k > 0 ? k - 1 : 0] : (band > 0 ? up_in : h_top);
            float const d = (k < R - 1) ? t[k < R - 1 ? k + 1 : 0] : (band < W::G - 1 ? down_in : h_bot);
            nt[k] = fix[k] ? t[k] : next_time(godunov2_raw(fminf(l, r), fminf(u, d), c[k], c2[k]), t[k], t0[k], mode);
            moved |= moves(nt[k], t[k], eps, mode != kUpdKeepMin);
        }
#pragma unroll
        for (int k = 0; k < R; ++k) {
            changed |= nt[k] != t[k];
            t[k] = nt[k];
        }
        ++sweeps;
        if (!__any_sync(FULL, moved)) break;
        if (sweeps >= fresh_sweeps) mode = kUpdKeepMin;
        if (sweeps >= s.max_sweeps) {
            capped = true;
            break;
        }
    }

    // The converged tile into the box interior (for the probes), noting the
    // edge rows this solve changed against the staged values it replaces.
    uint32_t ec = 0u;
    bool mv = false;  // some cell moved by more than eps
#pragma unroll
    for (int k = 0; k < R; ++k) {
        int const y = band * R + k;
        float const staged = sm.time[si<B>(x, y)];
        sm.time[si<B>(x, y)] = t[k];
        mv |= x < tc.sx && y < tc.sy && moves(t[k], staged, eps, true);
        if (x < tc.sx && y < tc.sy && t[k] != staged && falls_far(t[k], staged)) ec |= 16u;  // not a quiet solve
        if (x < tc.sx && y < tc.sy && t[k] != staged) {
            if (x == 0) ec |= 1u;
            if (y == 0) ec |= 2u;
            if (x == tc.sx - 1) ec |= 4u;
            if (y == tc.sy - 1) ec |= 8u;
        }
    }
    ec = __reduce_or_sync(FULL, ec);
    __syncwarp();

    // Probes: 4 edges x B cells over the 32 lanes, each edge within B lanes.
    uint32_t imp_mask = 0u;
    float keys[4] = {f_inf(), f_inf(), f_inf(), f_inf()};
#pragma unroll
    for (int it = 0; it < 4 * B / 32; ++it) {
        int const p = it * 32 + lane;
        int const e = p / B;
        int const ei = p % B;
        bool imp = false;
        float key = f_inf();
        int const nb = neighbour_tile(I, tc.tx, tc.ty, e);
        int const len = (e & 1) ? tc.sx : tc.sy;
        if (nb >= 0 && ei < len) {
            int px, py, qx, qy, fx, fy;
            if (e == 0) { px = -1; py = ei; qx = 0; qy = ei; fx = -2; fy = ei; }
            else if (e == 1) { px = ei; py = -1; qx = ei; qy = 0; fx = ei; fy = -2; }
            else if (e == 2) { px = tc.sx; py = ei; qx = tc.sx - 1; qy = ei; fx = tc.sx + 1; fy = ei; }
            else { px = ei; py = tc.sy; qx = ei; qy = tc.sy - 1; fx = ei; fy = tc.sy + 1; }
            int const pi = si<B>(px, py);
            float const cp = sm.cost[pi];
            float const told = sm.time[pi];
            if (cp < f_inf() && told != 0.f) {  // seeds never change
                float const a_norm = fminf(sm.time[si<B>(qx, qy)], sm.time[si<B>(fx, fy)]);
                float const a_lat = (e & 1) ? fminf(sm.time[pi - 1], sm.time[pi + 1])
                                            : fminf(sm.time[pi - G::BW], sm.time[pi + G::BW]);
                bool const track_rise = s.refresh != 0u;
                float const nv = next_time(godunov_raw(a_norm, a_lat, cp), told, told, track_rise ? kUpdFresh : kUpdKeepMin);
                if (moves(nv, told, eps, track_rise)) {
                    imp = true;
                    key = nv;
                }
            }
        }
#pragma unroll
        for (int o = B / 2; o >= 1; o >>= 1) {
            imp |= __shfl_xor_sync(FULL, static_cast<int>(imp), o) != 0;
            key = fminf(key, __shfl_xor_sync(FULL, key, o));
        }
        // lane 0 gathers the edge results of each group of B lanes
#pragma unroll
        for (int q = 0; q < 32 / B; ++q) {
            int const eq = (it * 32 + q * B) / B;
            bool const iq = __shfl_sync(FULL, static_cast<int>(imp), q * B) != 0;
            float const kq = __shfl_sync(FULL, key, q * B);
            if (iq) imp_mask |= 1u << eq;
            keys[eq] = kq;
        }
    }

    // Commit (coalesced along rows) and the smallest time.
    bool const tile_changed = __any_sync(FULL, changed);
    bool const useful = __any_sync(FULL, mv);  // the trace label
    float lmin = f_inf();
#pragma unroll
    for (int k = 0; k < R; ++k) {
        int const y = band * R + k;
        if (x < tc.sx && y < tc.sy) {
            lmin = fminf(lmin, t[k]);
            size_t const gi = static_cast<size_t>(tc.oy + y) * I.w + tc.ox + x;
            if (tile_changed && GHCM_CHECK(s.ctl, gi < static_cast<size_t>(I.w) * I.h, 12u)) I.time[gi] = t[k];
        }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) lmin = fminf(lmin, __shfl_xor_sync(FULL, lmin, o));
    capped = __any_sync(FULL, capped);
    __syncwarp();
    if (lane == 0) {
        s.tmin[tile] = lmin;
        if (tile_changed) s.epoch[tile] = epoch;  // the next residual pass re-checks it and its neighbours
        if (solve_count(sm.claim[0]) < s.refresh && (capped || !(ec & 16u))) atomicAdd(&s.flags[tile], kSolveOne);
        learn_commit(s, tile, useful, wave, sweeps, sm.feat);
#pragma unroll
        for (int e = 0; e < 4; ++e)
            if (((imp_mask & ec) >> e) & 1u)
                activate(s, static_cast<uint32_t>(neighbour_tile(I, tc.tx, tc.ty, e)), kEdgeBit0 << ((e + 2) & 3),
                         keys[e], nxt, s_krange, pbit);
        if (capped) activate(s, tile, kFull, lmin, nxt, s_krange, 0u);
#ifdef GHCM_PROFILE
        atomicAdd(&s.ctl->prof[3], static_cast<unsigned long long>(sweeps));
        atomicMax(&s.ctl->wave_max_sweeps, sweeps);
#endif
    }
    __syncwarp();
    return kJobSolved;
}

}  // namespace ghcm

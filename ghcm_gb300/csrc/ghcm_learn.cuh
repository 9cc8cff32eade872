// Learned block schedule: per-tile features, the warp-cooperative MLP that
// scores a tile as it is queued, and the claim-time veto.
//
// The reference picks the n tiles with the smallest frozen min-time key
// (src/eikonal_hcm.cpp:47-80, 344-358). The learned schedule scores every
// active tile with a 12 -> 64 -> 64 -> 1 FP32 MLP (the CTA that queues a tile
// scores it right after its own solve) and solves those scoring at or above a
// threshold (tiles re-queued by the residual check or a sweep cap always go),
// filled up to fallback_jobs in the plain key order. The global Godunov
// residual check is unchanged, so a wrong score costs work, never accuracy.
//
// The same features are written, with the outcome of each solve, by the
// trace recorder of the plain solver; the model is trained on those traces
// by the kernels of ghcm_mlp.cu.
#pragma once

#include "ghcm_sched.cuh"

namespace ghcm {

// Features of a tile (all roughly in [-1, 1]):
//   0 (key - front) / span       where the tile's key sits in this wave's key range
//   1 (kmax - key) / span        spread of the boundary values that activated it
//   2 never solved
//   3 (smallest time - key)/span how far the tile's current times lie above the new boundary
//   4-6 log2 min / max / mean speed / 8
//   7 active neighbours / 4
//   8 waves since the tile's last useful solve / 64 (1: never)
//   9 log2(1 + solves so far) / 8
//  10 re-queued in full (residual check or sweep cap)
//  11 edges with new boundary values / 4
//
// The features from the loaded tile state. key/kmax: the tile's activation
// keys, flags: its scheduler flags, tm: smallest time, ns: solves so far,
// st: log speed statistics, lc: wave of its last useful solve + 1, act:
// active neighbours, front/span: this wave's key range.
__device__ __forceinline__ void features_from(float key, float kmax, uint32_t flags, float tm, uint32_t ns, float4 st,
                                              uint32_t lc, int act, uint32_t wave, float front, float span,
                                              float (&f)[kFeatures]) {
    float const inv = 1.0f / span;
    float const k = (key < f_inf()) ? key : front + span;
    f[0] = fminf(fmaxf((k - front) * inv, 0.f), 1.f);
    f[1] = fminf(fmaxf((fmaxf(kmax, k) - k) * inv, 0.f), 1.f);
    f[2] = ns ? 0.f : 1.f;
    f[3] = (tm < f_inf()) ? fminf(fmaxf((tm - k) * inv, -1.f), 1.f) : 1.f;
    f[4] = st.x;
    f[5] = st.y;
    f[6] = st.z;
    f[7] = 0.25f * static_cast<float>(act);
    f[8] = lc ? fminf(static_cast<float>(wave + 1u - lc), 64.f) * (1.f / 64.f) : 1.f;
    f[9] = log2f(1.f + static_cast<float>(ns)) * 0.125f;
    f[10] = (flags & kFull) ? 1.f : 0.f;
    f[11] = 0.25f * static_cast<float>(__popc((flags & kEdgeMask) >> 4));
}

// Loads a tile's state and computes its features (claim-time trace and veto).
__device__ __forceinline__ void tile_features(const Sched& s, uint32_t tile, uint32_t flags, float key, float kmax,
                                              uint32_t wave, float front, float span, float (&f)[kFeatures]) {
    const Learn& L = s.learn;
    float const tm = __ldcg(&s.tmin[tile]);
    uint32_t const ns = __ldcg(&L.nsolve[tile]);
    float4 const st = __ldg(&L.tstat[tile]);
    uint32_t const lc = __ldcg(&L.last_change[tile]);
    const Inst& I = s.insts[inst_of(s, tile)];
    uint32_t const local = tile - I.tile_base;
    uint32_t const tx = local % I.tiles_x, ty = local / I.tiles_x;
    int act = 0;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        int const nb = neighbour_tile(I, tx, ty, e);
        if (nb >= 0 && (__ldcg(&s.flags[nb]) & kActive)) ++act;
    }
    features_from(key, kmax, flags, tm, ns, st, lc, act, wave, front, span, f);
}

// The MLP parameters staged in the kernel's dynamic shared memory (kParams
// floats) by every CTA of a learned-schedule launch, so that scoring reads
// them at shared-memory latency.
extern __shared__ __align__(16) float g_mlp_params[];

// Logit of the MLP for features x, computed by the whole warp (every lane
// holds x and gets the result). Lane l owns hidden units l and l + 32. P is
// the flat parameter vector (shared or global memory).
__device__ __forceinline__ float mlp_logit_warp(const float* __restrict__ P, const float (&x)[kFeatures]) {
    constexpr unsigned FULL = 0xffffffffu;
    int const lane = threadIdx.x & 31;
    float h0 = (P[kOffB1 + lane]);
    float h1 = (P[kOffB1 + 32 + lane]);
#pragma unroll
    for (int i = 0; i < kFeatures; ++i) {
        h0 = fmaf((P[kOffW1 + i * kHidden + lane]), x[i], h0);
        h1 = fmaf((P[kOffW1 + i * kHidden + 32 + lane]), x[i], h1);
    }
    h0 = fmaxf(h0, 0.f);
    h1 = fmaxf(h1, 0.f);
    float a0 = (P[kOffB2 + lane]);
    float a1 = (P[kOffB2 + 32 + lane]);
#pragma unroll 8
    for (int k = 0; k < 32; ++k) {
        float const v = __shfl_sync(FULL, h0, k);
        a0 = fmaf((P[kOffW2 + k * kHidden + lane]), v, a0);
        a1 = fmaf((P[kOffW2 + k * kHidden + 32 + lane]), v, a1);
    }
#pragma unroll 8
    for (int k = 0; k < 32; ++k) {
        float const v = __shfl_sync(FULL, h1, k);
        a0 = fmaf((P[kOffW2 + (k + 32) * kHidden + lane]), v, a0);
        a1 = fmaf((P[kOffW2 + (k + 32) * kHidden + 32 + lane]), v, a1);
    }
    a0 = fmaxf(a0, 0.f);
    a1 = fmaxf(a1, 0.f);
    float z = fmaf((P[kOffW3 + lane]), a0, (P[kOffW3 + 32 + lane]) * a1);
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) z += __shfl_xor_sync(FULL, z, o);
    return z + (P[kOffB3]);
}

// Per-tile log2 speed statistics (features 4-6), one warp per tile.
template <int B>
__device__ void tile_speed_stats(const Sched& s, uint32_t tile) {
    int const lane = threadIdx.x & 31;
    const Inst& I = s.insts[inst_of(s, tile)];
    TileCoord const tc = tile_coord<B>(I, tile);
    float lo = f_inf(), hi = 0.f, sum = 0.f;
    int n = 0;
    for (int k = lane; k < B * B; k += 32) {
        int const lx = k % B, ly = k / B;
        if (lx >= tc.sx || ly >= tc.sy) continue;
        float const c = to_cost(I, __ldg(&I.in[static_cast<size_t>(tc.oy + ly) * I.w + tc.ox + lx]));
        float const v = (c < f_inf() && c > 0.f) ? I.spacing / c : 0.f;  // speed; 0 for walls
        lo = fminf(lo, v);
        hi = fmaxf(hi, v);
        sum += v;
        ++n;
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        n += __shfl_xor_sync(0xffffffffu, n, o);
    }
    if (lane == 0) {
        auto lg = [](float v) { return fminf(fmaxf(log2f(fmaxf(v, 1e-30f)) * 0.125f, -2.f), 2.f); };
        s.learn.tstat[tile] = make_float4(lg(lo), lg(hi), lg(sum / static_cast<float>(n > 0 ? n : 1)), 0.f);
    }
}

// Score policy. The state of a tile the calling CTA's solve activates, as
// the scorer needs it: its flags, keys, smallest time, solves, speed
// statistics, wave of its last useful solve, its neighbours' flags and the
// wave's key range. load() is run by the activating thread right after its
// flag atomic, into the shared-memory slot the scoring warp reads: every
// load is issued before the first store, so the round trip overlaps the
// activation's own, and the thread's own key, kmax and flag updates precede
// the loads in program order and are seen.
struct QueuedState {
    float4 st;
    uint32_t flags, key, kmax, ns, lc, act;
    float tm, front, span;
    __device__ __forceinline__ void load(const Sched& s, const Inst& I, uint32_t tile, uint32_t tx, uint32_t ty) {
        const Learn& L = s.learn;
        uint32_t const f = __ldcg(&s.flags[tile]);
        uint32_t const k = __ldcg(&s.key[tile]);
        uint32_t const km = __ldcg(&L.kmax[tile]);
        float const t = __ldcg(&s.tmin[tile]);
        uint32_t const n = __ldcg(&L.nsolve[tile]);
        float4 const sv = __ldg(&L.tstat[tile]);
        uint32_t const l = __ldcg(&L.last_change[tile]);
        float const fr = __ldcg(&s.ctl->wave_front);
        float const sp = __ldcg(&s.ctl->wave_span);
        uint32_t nf[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            int const nb = neighbour_tile(I, tx, ty, e);
            nf[e] = nb >= 0 ? __ldcg(&s.flags[nb]) : 0u;
        }
        uint32_t a = 0u;
#pragma unroll
        for (int e = 0; e < 4; ++e) a += (nf[e] & kActive) ? 1u : 0u;
        flags = f;
        key = k;
        kmax = km;
        tm = t;
        ns = n;
        st = sv;
        lc = l;
        front = fr;
        span = sp;
        act = a;
    }
};

// The model logit of a tile just appended at entry `pos` of list[nxt] by the
// calling CTA's solve, from its loaded state, computed by the calling warp
// and kept in that entry's score for the next decision. Tiles re-queued in
// full need no score (they are always taken).
__device__ void score_queued_warp(const Sched& s, const QueuedState& q, uint32_t nxt, uint32_t pos, uint32_t wave) {
    if (q.flags & kFull) return;
    float x[kFeatures];
    features_from(__uint_as_float(q.key), __uint_as_float(q.kmax), q.flags, q.tm, q.ns, q.st, q.lc,
                  static_cast<int>(q.act), wave, q.front, q.span, x);
    float const z = mlp_logit_warp(g_mlp_params, x);
    if ((threadIdx.x & 31) == 0) __stcg(&s.learn.lscore[nxt][pos], z);
}

}  // namespace ghcm

namespace ghcm {

// Claim-time bookkeeping of a block-solve, by one thread, in two parts.
// learn_claim_kmax resets the tile's largest activation key and returns it;
// it is issued with the claim's other atomics, before the flag clear acquires
// (an activation landing in between leaves its key for the tile's next
// queueing: it is only a feature). learn_claim then, when tracing, writes the
// features the scheduler saw into feat. flags / key_bits / kmx: the tile's
// state as claimed.
__device__ __forceinline__ uint32_t learn_claim_kmax(const Sched& s, uint32_t tile) {
    return s.learn.tstat ? atomicExch(&s.learn.kmax[tile], 0u) : 0u;
}
__device__ __forceinline__ uint32_t learn_claim(const Sched& s, uint32_t tile, uint32_t flags, uint32_t key_bits,
                                                uint32_t kmx, uint32_t wave, float* feat) {
    if (!s.learn.tstat) return 0u;
    if (s.learn.trace) {
        float f[kFeatures];
        tile_features(s, tile, flags, __uint_as_float(key_bits), __uint_as_float(kmx), wave,
                      ld_relaxed_f(&s.ctl->wave_front), ld_relaxed_f(&s.ctl->wave_span), f);
#pragma unroll
        for (int i = 0; i < kFeatures; ++i) feat[i] = f[i];
    }
    return kmx;
}

// Veto mode: decides, by one whole warp, whether the claimed tile is deferred
// instead of solved - its score is below the threshold, it was not
// re-queued in full and it has been deferred fewer than max_vetoes times in a
// row. Every lane gets the decision.
__device__ __forceinline__ bool learn_veto_warp(const Sched& s, uint32_t tile, uint32_t flags, uint32_t key_bits,
                                                uint32_t kmax_bits, uint32_t wave) {
    if (!s.learn.params || !s.learn.veto || (flags & kFull)) return false;
    if (__ldcg(&s.learn.vetoes[tile]) >= s.learn.max_vetoes) return false;
    float x[kFeatures];
    tile_features(s, tile, flags, __uint_as_float(key_bits), __uint_as_float(kmax_bits), wave,
                  ld_relaxed_f(&s.ctl->wave_front), ld_relaxed_f(&s.ctl->wave_span), x);
    float const z = mlp_logit_warp(g_mlp_params, x);
    return z < logf(s.learn.threshold / (1.f - s.learn.threshold));
}

// A vetoed tile goes back to the next active set with its key, edge bits and
// largest activation key, by one thread.
__device__ __forceinline__ void learn_defer(const Sched& s, uint32_t tile, uint32_t flags, uint32_t key_bits,
                                            uint32_t kmax_bits, uint32_t nxt, uint32_t* s_krange) {
    __stcg(&s.learn.vetoes[tile], __ldcg(&s.learn.vetoes[tile]) + 1u);
    atomicMax(&s.learn.kmax[tile], kmax_bits);
    atomicAdd(&s.ctl->vetoes, 1u);
    activate(s, tile, flags & (kFull | kEdgeMask), __uint_as_float(key_bits), nxt, s_krange, 0u);
}

// Commit-time bookkeeping, by one thread: solve count, wave of the last
// useful solve and the trace record.
__device__ __forceinline__ void learn_commit(const Sched& s, uint32_t tile, bool useful, uint32_t wave,
                                             uint32_t sweeps, const float* feat) {
    if (!s.learn.tstat) return;
    __stcg(&s.learn.nsolve[tile], __ldcg(&s.learn.nsolve[tile]) + 1u);
    if (s.learn.veto) __stcg(&s.learn.vetoes[tile], 0u);
    if (useful) __stcg(&s.learn.last_change[tile], wave + 1u);
    if (s.learn.trace) {
        uint32_t const pos = atomicAdd(&s.ctl->trace_count, 1u);
        if (pos < s.learn.trace_cap) {
            TraceRec& r = s.learn.trace[pos];
#pragma unroll
            for (int i = 0; i < kFeatures; ++i) r.f[i] = feat[i];
            r.tile = tile;
            r.wave = wave;
            r.useful = useful ? 1u : 0u;
            r.sweeps = sweeps;
        }
    }
}

}  // namespace ghcm

// Device-side block scheduler: tile addressing, neighbour activation, the
// top-n histogram select and the wave barrier whose last arriving CTA decides the
// next phase. Replaces the host priority queue and activation loop of
// src/eikonal_hcm.cpp:343-469.
#pragma once

#include "ghcm_device.cuh"

namespace ghcm {

// Scheduler phases (Ctl::phase).
enum : uint32_t {
    kPhaseInit = 0,
    kPhaseJobs = 1,      // solve the selected tiles
    kPhaseResidual = 2,  // global fixed-point check
    kPhaseDone = 3,
    kPhaseStop = 4,
};

struct TileCoord {
    uint32_t tx, ty;
    int ox, oy;  // origin
    int sx, sy;  // size clipped at the field edge
};

__device__ __forceinline__ uint32_t inst_of(const Sched& s, uint32_t tile) {
    return s.tile_inst ? __ldg(&s.tile_inst[tile]) : 0u;
}

// TMA tensor maps of instance ii: a batch keeps them in a device table, a
// single solve in the kernel parameters.
__device__ __forceinline__ const CUtensorMap* time_map(const Sched& s, uint32_t ii) {
    return s.maps ? &s.maps[2u * ii] : &s.tmap_time;
}
__device__ __forceinline__ const CUtensorMap* in_map(const Sched& s, uint32_t ii) {
    return s.maps ? &s.maps[2u * ii + 1u] : &s.tmap_in;
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

// cost = h / speed (src/test_runner.cpp:38-42), IEEE-rounded like the host's,
// then capped: min(cost, cap) makes walls permeable as the reference's
// field_cost_as_permeable does (src/test_runner.cpp:70-75); cap = +inf: none.
__device__ __forceinline__ float cap_cost(const Inst& I, float c) { return fminf(c, I.cost_cap); }
__device__ __forceinline__ float to_cost(const Inst& I, float v) {
    return cap_cost(I, I.in_is_speed ? __fdiv_rn(I.spacing, v) : v);
}

constexpr uint32_t kNoPos = 0xffffffffu;

// Puts `tile` into the next active set: lowers its key to `key`, ORs `bits`
// (and `pbit`, act_phase_bit of the phase when a solve of this phase activates
// a neighbour, else 0) into its flags and appends it to list[nxt] unless it
// is already active.
// The device form of the dirty-set test + heap push + border-mask OR of
// src/eikonal_hcm.cpp:451-462. s_krange (the calling CTA's {min, max} key
// bits of what it activated this phase) is widened to `key`. Returns the
// tile's position in list[nxt] when this call appended it (it was idle),
// else kNoPos. `after_flag` runs right after the flag atomic is issued: loads
// it makes are in flight with that atomic and the append (a release orders
// only what comes before it).
struct NoHook {
    __device__ void operator()() const {}
};
template <class Hook = NoHook>
__device__ __forceinline__ uint32_t activate(const Sched& s, uint32_t tile, uint32_t bits, float key, uint32_t nxt,
                                             uint32_t* s_krange, uint32_t pbit, Hook after_flag = Hook{}) {
    uint32_t const kb = __float_as_uint(key);
    atomicMin(&s.key[tile], kb);
    if (s.learn.kmax) atomicMax(&s.learn.kmax[tile], kb);
    if (s_krange) {
        atomicMin(&s_krange[0], kb);
        atomicMax(&s_krange[1], kb);
    }
    uint32_t const old = atom_or_release(&s.flags[tile], kActive | bits | pbit);
    after_flag();
    if (!(old & kActive)) {
        uint32_t const pos = atomicAdd(&s.ctl->count[nxt], 1u);
        if (pos < s.num_tiles) {
            s.list[nxt][pos] = tile;
            // learned score policy: tiles re-queued in full always go; others wait for a score
            if (s.learn.lscore[nxt]) s.learn.lscore[nxt][pos] = (bits & kFull) ? f_inf() : -f_inf();
            return pos;
        }
        atomicOr(&s.ctl->error, kErrInternal);
    }
    return kNoPos;
}

// Priority key of an active tile (smaller = solved first), as float bits.
// Keys stay exact: a tile activated again with a lower key moves up (the
// reference freezes a heap entry's key, src/eikonal_hcm.cpp:74-75, and on the
// 4096^2 rings frozen keys took the device schedule from 766 to 2,338 waves).
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

// Score gate of the learned schedule for select_top_n: tiles whose score (at
// their list entry) reaches `thr` go first, at most `cap` of them; the wave
// is filled up to the select's n in key order.
struct ScoreGate {
    bool on;
    float thr;     // threshold logit
    uint32_t cap;  // most jobs a wave
};

// Selects the n smallest keys among the m tiles of list[L], by the whole CTA:
// a histogram of SELECT_BINS bins over [lo, hi] (the keys' range, or a
// superset of it; with have_range false a first pass finds it), a scan for
// the bin holding the n-th key, then every tile of a lower bin and enough
// tiles of that bin go to s.jobs from jobs_base, the rest to list[L ^ 1].
// The order is exact up to 1/SELECT_BINS of the range. With the
// gate on, bin 0 holds the qualifying tiles and the keys use the others; n
// becomes max(min(qualifying, cap), n). Returns the number carried; the
// jobs are m - carried.
constexpr int SELECT_BINS = 2048;

template <int THREADS, int R>
__device__ uint32_t select_top_n(const Sched& s, uint32_t L, uint32_t m, uint32_t n, uint32_t* s_hist, uint32_t* s_sel,
                                 float lo, float hi, bool have_range, uint32_t jobs_base, ScoreGate gate) {
    __shared__ float s_fmin[THREADS / 32], s_fmax[THREADS / 32];
    int const tid = threadIdx.x;
    int const lane = tid & 31, warp = tid >> 5;
    const uint32_t* list = s.list[L];
    uint32_t* carry = s.list[L ^ 1u];
    const float* score = s.learn.lscore[L];
    float* carry_score = s.learn.lscore[L ^ 1u];
#ifdef GHCM_PROFILE
    uint64_t const p_s0 = global_ns();
#endif
    for (int i = tid; i < SELECT_BINS; i += THREADS) s_hist[i] = 0u;
    if (!have_range) {
        // pass 1: range of the finite keys
        lo = f_inf();
        hi = 0.f;
        for (uint32_t i = tid; i < m; i += THREADS) {
            float const k = __uint_as_float(tile_key(s, __ldcg(&list[i])));
            if (k < f_inf()) {
                lo = fminf(lo, k);
                hi = fmaxf(hi, k);
            }
        }
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if (lane == 0) {
            s_fmin[warp] = lo;
            s_fmax[warp] = hi;
        }
        __syncthreads();
        lo = s_fmin[0];
        hi = s_fmax[0];
        for (int w = 1; w < THREADS / 32; ++w) {
            lo = fminf(lo, s_fmin[w]);
            hi = fmaxf(hi, s_fmax[w]);
        }
    } else {
        __syncthreads();
    }
    int const first = gate.on ? 1 : 0;  // bins of the keys: [first, SELECT_BINS)
    float const span = hi - lo;
    float const scale = (span > 0.f) ? static_cast<float>(SELECT_BINS - 1 - first) / span : 0.f;
    // Entries i0 + tid + u * THREADS (u < R): ids and, with the gate on,
    // scores in one round trip, then the keys in a second; b = -1 past m.
    auto load = [&](uint32_t i0, uint32_t (&t)[R], int (&b)[R]) {
        bool q[R];
#pragma unroll
        for (int u = 0; u < R; ++u) {
            uint32_t const i = i0 + tid + u * THREADS;
            t[u] = (i < m) ? __ldcg(&list[i]) : 0u;
            q[u] = gate.on && i < m && __ldcg(&score[i]) >= gate.thr;  // +inf: re-queued in full
        }
        uint32_t kb[R];
#pragma unroll
        for (int u = 0; u < R; ++u) kb[u] = (i0 + tid + u * THREADS < m) ? tile_key(s, t[u]) : inf_bits();
#pragma unroll
        for (int u = 0; u < R; ++u) {
            float const k = __uint_as_float(kb[u]);
            int bb = SELECT_BINS - 1;
            if (q[u]) {
                bb = 0;
            } else if (k < f_inf()) {
                bb = first + static_cast<int>((k - lo) * scale);
                bb = bb < first ? first : (bb >= SELECT_BINS ? SELECT_BINS - 1 : bb);
            }
            b[u] = (i0 + tid + u * THREADS < m) ? bb : -1;
        }
    };
    // pass 2: histogram. The first R * THREADS entries keep their ids and
    // bins in registers for the gather; longer lists find them again there.
    bool const held = m <= static_cast<uint32_t>(R * THREADS);
    uint32_t t[R];
    int b[R];
    load(0u, t, b);
#pragma unroll
    for (int u = 0; u < R; ++u)
        if (b[u] >= 0) atomicAdd(&s_hist[b[u]], 1u);
    if (!held) {
        for (uint32_t i0 = R * THREADS; i0 < m; i0 += R * THREADS) {
            uint32_t t2[R];
            int b2[R];
            load(i0, t2, b2);
#pragma unroll
            for (int u = 0; u < R; ++u)
                if (b2[u] >= 0) atomicAdd(&s_hist[b2[u]], 1u);
        }
    }
    if (tid == 0) {
        s_sel[0] = SELECT_BINS;  // n >= m: every bin lies below the boundary
        s_sel[1] = 0u;
        s_sel[2] = 0u;
        s_sel[3] = 0u;
        s_sel[4] = 0u;
    }
    __syncthreads();
#ifdef GHCM_PROFILE
    uint64_t const p_s1 = global_ns();
#endif
    if (gate.on) n = max(min(s_hist[0], gate.cap), n);  // qualifying tiles first, up to the cap
    if (n < m) {
        // the bin holding the n-th smallest entry: thread t scans bins [t*PER, (t+1)*PER)
        constexpr int PER = SELECT_BINS / THREADS;
        uint32_t hv[PER];  // scalar reads: s_hist is only 4-byte aligned
#pragma unroll
        for (int j = 0; j < PER; ++j) hv[j] = s_hist[tid * PER + j];
        uint32_t part = 0u;
#pragma unroll
        for (int j = 0; j < PER; ++j) part += hv[j];
        uint32_t incl = part;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t const v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        __shared__ uint32_t s_wsum[THREADS / 32];
        if (lane == 31) s_wsum[warp] = incl;
        __syncthreads();
        uint32_t wbase = 0u;
        for (int w = 0; w < warp; ++w) wbase += s_wsum[w];
        uint32_t below = wbase + incl - part;
        if (below < n && n <= below + part) {
#pragma unroll
            for (int j = 0; j < PER; ++j) {
                uint32_t const h = hv[j];
                if (below + h >= n) {
                    s_sel[0] = static_cast<uint32_t>(tid * PER + j);
                    s_sel[1] = n - below;  // how many of the boundary bin to take
                    break;
                }
                below += h;
            }
        }
        __syncthreads();
    }
    int const bnd = static_cast<int>(s_sel[0]);
    uint32_t const take_eq = s_sel[1];
#ifdef GHCM_PROFILE
    uint64_t const p_s2 = global_ns();
#endif
    // pass 3: gather. An entry of the boundary bin takes its turn with its own
    // shared atomic (the first take_eq go); a warp then takes its job and
    // carry positions for all R entries of each lane with one atomic each. A
    // carried entry keeps whether it qualified (+inf / -inf): the gate only
    // compares scores with its fixed threshold.
    auto gather = [&](const uint32_t (&tt)[R], const int (&bb)[R]) {
        uint32_t const lt = (1u << lane) - 1u;
        bool tk[R];
        uint32_t ntake = 0u, ncarry = 0u;
#pragma unroll
        for (int u = 0; u < R; ++u) {
            bool const valid = bb[u] >= 0;
            bool take = valid && bb[u] < bnd;
            if (valid && bb[u] == bnd) take = atomicAdd(&s_sel[2], 1u) < take_eq;
            tk[u] = take;
            ntake += __popc(__ballot_sync(0xffffffffu, take));
            ncarry += __popc(__ballot_sync(0xffffffffu, valid && !take));
        }
        uint32_t jb = 0u, cb = 0u;
        if (lane == 0) {
            if (ntake) jb = atomicAdd(&s_sel[3], ntake);
            if (ncarry) cb = atomicAdd(&s_sel[4], ncarry);
        }
        jb = jobs_base + __shfl_sync(0xffffffffu, jb, 0);
        cb = __shfl_sync(0xffffffffu, cb, 0);
#pragma unroll
        for (int u = 0; u < R; ++u) {
            bool const valid = bb[u] >= 0;
            uint32_t const tm = __ballot_sync(0xffffffffu, tk[u]);
            uint32_t const cm = __ballot_sync(0xffffffffu, valid && !tk[u]);
            if (tk[u]) {
                uint32_t const pos = jb + __popc(tm & lt);
                if (GHCM_CHECK(s.ctl, pos < s.max_jobs, 9u)) s.jobs[pos] = tt[u];
            } else if (valid) {
                uint32_t const pos = cb + __popc(cm & lt);
                if (GHCM_CHECK(s.ctl, pos < s.num_tiles, 10u)) {
                    carry[pos] = tt[u];
                    if (gate.on) carry_score[pos] = (bb[u] == 0) ? f_inf() : -f_inf();
                }
            }
            jb += __popc(tm);
            cb += __popc(cm);
        }
    };
    gather(t, b);
    if (!held) {
        for (uint32_t i0 = R * THREADS; i0 < m; i0 += R * THREADS) {
            uint32_t t2[R];
            int b2[R];
            load(i0, t2, b2);
            gather(t2, b2);
        }
    }
    if (gate.on && tid == 0) s_sel[5] = s_hist[0];  // qualifying tiles, for the counters
    __syncthreads();
#ifdef GHCM_PROFILE
    if (tid == 0) {  // [24] histogram, [25] scan, [26] gather
        uint64_t const p_s3 = global_ns();
        s.ctl->prof[24] += p_s1 - p_s0;
        s.ctl->prof[25] += p_s2 - p_s1;
        s.ctl->prof[26] += p_s3 - p_s2;
    }
#endif
    return s_sel[4];
}

// The scheduler state each CTA keeps in shared memory (s_state[]), refreshed
// from the release word at every wave barrier.
enum : int {
    kStPhase = 0, kStCur = 1, kStJobs = 2, kStInList = 3, kStError = 4, kStWaves = 5, kStGen = 6,
    kStResid = 7,  // residual passes begun
};

// Release word: the decision of the last CTA, published with the release.
//   bits 0-31 job count, 32-35 phase, 36 cur, 37 jobs-in-list, 38 error,
//   40-63 barrier generation.
__device__ __forceinline__ unsigned long long pack_release(uint32_t gen, uint32_t phase, uint32_t cur, uint32_t jobs,
                                                           uint32_t in_list, uint32_t err) {
    return static_cast<unsigned long long>(jobs) | (static_cast<unsigned long long>(phase & 15u) << 32) |
           (static_cast<unsigned long long>(cur & 1u) << 36) | (static_cast<unsigned long long>(in_list & 1u) << 37) |
           (static_cast<unsigned long long>(err ? 1u : 0u) << 38) |
           (static_cast<unsigned long long>(gen & 0xffffffu) << 40);
}

__device__ __forceinline__ void unpack_release(unsigned long long w, uint32_t* st) {
    uint32_t const phase = static_cast<uint32_t>(w >> 32) & 15u;
    st[kStJobs] = static_cast<uint32_t>(w);
    st[kStPhase] = phase;
    st[kStCur] = static_cast<uint32_t>(w >> 36) & 1u;
    st[kStInList] = static_cast<uint32_t>(w >> 37) & 1u;
    st[kStError] = static_cast<uint32_t>(w >> 38) & 1u;
    st[kStGen] = static_cast<uint32_t>(w >> 40) & 0xffffffu;
    if (phase == kPhaseJobs) st[kStWaves] += 1u;
    if (phase == kPhaseResidual) st[kStResid] += 1u;
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ float ld_relaxed_f(const float* p) { return __uint_as_float(ld_relaxed(reinterpret_cast<const uint32_t*>(p))); }

// Runs the top-n on list[L] (m tiles): its n lowest keys (with the gate on,
// the qualifying tiles first, see ScoreGate) become jobs base.. of the next
// JOBS phase (or, with no jobs before them and m <= n, the list itself), the
// rest is carried to list[L ^ 1], where the activations of that phase also
// go. Returns {in_list, job count} in s_sel[8], [11].
template <int THREADS, int R>
__device__ void plan_jobs(const Sched& s, uint32_t L, uint32_t m, uint32_t n, uint32_t base, float lo, float hi,
                          uint32_t* s_hist, uint32_t* s_sel, ScoreGate gate) {
    Ctl* ctl = s.ctl;
    bool const all = m <= n;
    uint32_t carried = 0u;
    uint32_t qualifying = 0u;  // learned schedule: tiles scoring at or above the threshold
    if (!all) {
        carried = select_top_n<THREADS, R>(s, L, m, n, s_hist, s_sel, lo, hi, s.key_mode == 0u, base, gate);
        if (gate.on) qualifying = s_sel[5];
    } else {
        if (base)
            for (uint32_t i = threadIdx.x; i < m; i += THREADS) s.jobs[base + i] = __ldcg(&s.list[L][i]);
        if (gate.on) {
            bool q = false;
            for (uint32_t i = threadIdx.x; i < m; i += THREADS) q |= __ldcg(&s.learn.lscore[L][i]) >= gate.thr;
            qualifying = __syncthreads_or(q) ? 1u : 0u;
        }
    }
    if (threadIdx.x == 0) {
        ctl->count[L ^ 1u] = carried;
        // the carried keys lie in [lo, hi]: a superset range for list[L ^ 1]
        ctl->krange[L ^ 1u][0] = carried ? __float_as_uint(lo) : inf_bits();
        ctl->krange[L ^ 1u][1] = carried ? __float_as_uint(hi) : 0u;
        s_sel[8] = (all && base == 0u) ? 1u : 0u;
        s_sel[11] = base + (all ? m : m - carried);
        // learned schedule: a wave that took tiles by score, or one that went by key alone
        if (gate.on) atomicAdd(qualifying ? &ctl->score_waves : &ctl->fallback_waves, 1u);
    }
}

// Decides the next phase; run by the whole of the last CTA to reach the wave
// barrier while every other CTA waits. `st` is this CTA's view of the state
// the previous barrier published. Returns the new
// {jobs-in-list, phase, cur, job count} in s_sel[8..11].
//   after INIT / JOBS / RESIDUAL, the set to process is list[act]:
//     non-empty, plain        -> JOBS on its n lowest keys (the rest carried over)
//     non-empty, learned      -> JOBS on the tiles whose score qualifies,
//                                filled up to fallback_jobs in plain key order
//     empty after JOBS        -> RESIDUAL: the global fixed-point check
//     empty after RESIDUAL    -> DONE
// The key range of list[act] comes from the activations (ctl->krange); its
// min and span are published as this wave's front for the features.
template <int THREADS, int R>
__device__ void decide_phase(const Sched& s, const uint32_t* st, uint32_t* s_hist, uint32_t* s_sel) {
    Ctl* ctl = s.ctl;
    int const tid = threadIdx.x;
    uint32_t const prev = st[kStPhase];
    uint32_t const cur = st[kStCur];
    uint32_t phase = kPhaseJobs, ncur = cur;
    {
        uint32_t const act = (prev == kPhaseInit) ? 0u : (cur ^ 1u);
#ifdef GHCM_PROFILE
        if (tid == 0) ctl->prof[23] = global_ns();  // decision start
#endif
        // every control word the decision reads, in one round trip
        // a list holds each tile at most once; an overflow (an internal error,
        // already flagged by activate) never makes the select read past it
        uint32_t const m = min(ld_relaxed(&ctl->count[act]), s.num_tiles);
        uint32_t const klo = ld_relaxed(&ctl->krange[act][0]);
        uint32_t const khi = ld_relaxed(&ctl->krange[act][1]);
        if (tid == 0) s_sel[12] = ld_relaxed(&ctl->error);
        if (m == 0u) {
            if (prev == kPhaseResidual) {
                phase = kPhaseDone;
            } else {
                phase = kPhaseResidual;
                ncur = act ^ 1u;  // residual activations go to list[act], now empty
                if (tid == 0) {
                    ctl->count[act] = 0u;
                    ctl->krange[act][0] = inf_bits();
                    ctl->krange[act][1] = 0u;
                    atomicAdd(&ctl->residual_passes, 1u);
                }
            }
            if (tid == 0) {
                s_sel[8] = 0u;
                s_sel[11] = 0u;
            }
        } else if (s.max_waves != 0u && st[kStWaves] >= s.max_waves) {
            phase = kPhaseStop;
            if (tid == 0) {
                atomicOr(&ctl->error, kErrNotConverged);
                s_sel[8] = 0u;
                s_sel[11] = 0u;
            }
        } else {
            float const lo = __uint_as_float(klo);
            float const hi = __uint_as_float(khi);
            if (tid == 0) {
                ctl->wave_front = (lo < f_inf()) ? lo : 0.f;
                ctl->wave_span = (hi > lo && lo < f_inf()) ? hi - lo : 1.f;
                atomicMax(&ctl->max_active, m);
            }
            ncur = act;
#ifdef GHCM_PROFILE
            uint64_t const p_sel0 = global_ns();
#endif
            // learned schedule, score policy: the tiles scoring at or above the
            // threshold (at list entries, written when they were queued) first,
            // up to max_jobs, filled to fallback_jobs in plain key order
            bool const scored = s.learn.params && !s.learn.veto;
            ScoreGate gate{scored, 0.f, s.max_jobs};
            if (scored) gate.thr = logf(s.learn.threshold / (1.f - s.learn.threshold));
            uint32_t const n = scored ? min(s.learn.fallback_jobs, s.max_jobs) : s.max_jobs;
            plan_jobs<THREADS, R>(s, act, m, n, 0u, lo, hi, s_hist, s_sel, gate);
            if (tid == 0) atomicAdd(&ctl->waves, 1u);
#ifdef GHCM_PROFILE
            if (tid == 0) {  // [20] decision loads, [21] job planning, [22] waves that ran the top-n select
                ctl->prof[20] += p_sel0 - ctl->prof[23];
                ctl->prof[21] += global_ns() - p_sel0;
                if (m > n) ctl->prof[22] += 1u;
            }
#endif
        }
    }
    if (tid == 0) {
        s_sel[9] = phase;
        s_sel[10] = ncur;
    }
}

// Job order of the persistent grid. Consecutive block indices share SMs
// (a 608-block launch put blocks 0-15 four to an SM), so a wave with fewer
// jobs than CTAs would crowd its tiles onto a few SMs. Each CTA instead takes
// a slot on its SM when it starts (sm_enter) and, once every CTA has entered,
// ranks itself (sm_rank): first slot 0 of every SM in SM order, then slot 1,
// and so on - a permutation of 0..gridDim.x-1. Jobs j, j + grid, ... go to
// rank j.
__device__ __forceinline__ void sm_enter(Ctl* ctl, uint32_t* s_slot) {
    uint32_t smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    s_slot[0] = smid;
    if (smid < kMaxSms)
        s_slot[1] = atomicAdd(&ctl->sm_ctas[smid], 1u);
    else
        atomicOr(&ctl->sm_far, 1u);
}

// Every thread returns this CTA's rank; call after a grid barrier that
// follows every CTA's sm_enter.
template <int THREADS>
__device__ uint32_t sm_rank(const Ctl* ctl, const uint32_t* s_slot, uint32_t* s_tmp) {
    static_assert(THREADS >= 32 && THREADS % 32 == 0, "whole warps");
    int const tid = threadIdx.x;
    if (ld_relaxed(&ctl->sm_far) != 0u) return blockIdx.x;
    uint32_t const smid = s_slot[0], slot = s_slot[1];
    uint32_t part = 0u;
    for (uint32_t m = tid; m < kMaxSms; m += THREADS) {
        uint32_t const c = ld_relaxed(&ctl->sm_ctas[m]);
        part += min(c, slot) + ((m < smid && c > slot) ? 1u : 0u);
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((tid & 31) == 0) s_tmp[tid >> 5] = part;
    __syncthreads();
    uint32_t r = 0u;
#pragma unroll
    for (int w = 0; w < THREADS / 32; ++w) r += s_tmp[w];
    __syncthreads();
    return r;
}

// Grid-wide wave barrier. Every CTA arrives; the last one to arrive decides
// the next phase (decide_phase) and releases the others with one 64-bit word
// that carries the decision, so a released CTA needs no further load. The
// waits are bounded. On return s_state holds the new state; returns false
// when the grid must stop (timeout or error).
template <int THREADS, int R>
__device__ bool wave_barrier(const Sched& s, uint32_t* s_hist, uint32_t* s_sel, uint32_t* s_state,
                             uint32_t* s_krange) {
    __shared__ uint32_t s_last;
    Ctl* ctl = s.ctl;
    __syncthreads();
    if (threadIdx.x == 0) {
        // the keys this CTA activated or carried in the phase just run went
        // to list[cur ^ 1]: fold their range into that list's
        if (s_krange[0] <= s_krange[1]) {
            uint32_t const nxt = s_state[kStCur] ^ 1u;
            atomicMin(&ctl->krange[nxt][0], s_krange[0]);
            atomicMax(&ctl->krange[nxt][1], s_krange[1]);
        }
        s_krange[0] = inf_bits();
        s_krange[1] = 0u;
        // publish this CTA's work (gathered by the barrier above) and, for the
        // last to arrive, acquire everyone's
        uint32_t const arrived = atom_add_acq_rel(&ctl->bar_count, 1u) + 1u;
        s_last = (arrived == gridDim.x) ? 1u : 0u;
        if (s_last) ctl->bar_count = 0u;
    }
    __syncthreads();
    if (s_last) {
#ifdef GHCM_PROFILE
        uint64_t const t_last = global_ns();
        if (threadIdx.x == 0) {
            if (ctl->release_ns) ctl->prof[6] += t_last - ctl->release_ns;  // release -> last arrival
            ctl->prof[8] += ctl->wave_max_sweeps;
            ctl->wave_max_sweeps = 0u;
            ctl->prof[15] += ctl->prof[14];  // per-wave maxima: job end, first-job start, longest solve
            ctl->prof[17] += ctl->prof[16];
            ctl->prof[19] += ctl->prof[18];
            ctl->prof[14] = ctl->prof[16] = ctl->prof[18] = 0ull;
        }
#endif
        decide_phase<THREADS, R>(s, s_state, s_hist, s_sel);
#ifdef GHCM_PROFILE
        uint64_t const t_dec = global_ns();
#endif
        __syncthreads();
        if (threadIdx.x == 0) {
            // errors raised before the arrivals, or the wave cap just hit
            uint32_t const err = s_sel[12] | (s_sel[9] == kPhaseStop ? 1u : 0u);
            unsigned long long const w =
                pack_release(s_state[kStGen] + 1u, s_sel[9], s_sel[10], s_sel[11], s_sel[8], err);
#ifdef GHCM_PROFILE
            uint64_t const t_rel = global_ns();
            ctl->prof[2] += t_rel - t_last;  // decide
            ctl->prof[27] += t_rel - t_dec;  // end of the decision -> release store issued
            ctl->prof[9] += 1u;
            ctl->release_ns = t_rel;
#endif
            st_release_u64(&ctl->release, w);  // the decision's stores, gathered by the barrier above
            unpack_release(w, s_state);
        }
    } else if (threadIdx.x == 0) {
        uint32_t const gen = s_state[kStGen];
        uint64_t const t0 = global_ns();
        uint32_t spins = 0;
        unsigned long long w;
        for (;;) {
            w = ld_acquire_u64(&ctl->release);
            if ((static_cast<uint32_t>(w >> 40) & 0xffffffu) != gen) break;
            if (++spins > 32) {
                __nanosleep(32);
                if (global_ns() - t0 > s.timeout_ns) {
                    atomicOr(&ctl->error, kErrTimeout);
                    w = pack_release(gen, kPhaseStop, 0u, 0u, 0u, 1u);
                    break;
                }
            }
        }
#ifdef GHCM_PROFILE
        atomicAdd(&ctl->prof[7], static_cast<unsigned long long>(global_ns() - ld_relaxed_u64(&ctl->release_ns)));
#endif
        unpack_release(w, s_state);
    }
    __syncthreads();
    return s_state[kStError] == 0u;
}

}  // namespace ghcm

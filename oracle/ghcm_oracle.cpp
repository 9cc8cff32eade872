// ghcm oracle: a CPU restatement of the reference's eikonal solvers.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker for the CUDA solver in
// ghcm_gb300/ and the timed CPU baseline of bench.py. The product library
// (libghcm.so) never links it, and the product path never calls it.
//
// Parity of this restatement is pinned against the reference itself: the
// reference's src/eikonal_fim.cpp and src/eikonal_fmm.cpp are compiled from
// their own sources into oracle/_ref/libghcm_ref.so (oracle/Makefile) and the
// tests in tests/test_oracle.py require bit-identical fields on seeded inputs;
// tests/golden/ holds fields produced by that reference build.
//
// Conventions (all from the reference):
//   * fields are row-major, x fastest: idx = x + y * W   (src/util_dim.h:17-21)
//   * the solver input is COST = h / speed               (src/test_runner.cpp:38-42)
//   * cells outside the field read as +inf               (src/util_field.h:40-41)
//   * seeds are (x, y) pairs with time 0
// Build with -ffp-contract=off so that no multiply-add is fused: the Godunov
// update must round exactly like the reference build on every host.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <limits>
#include <queue>
#include <thread>
#include <vector>

namespace {

constexpr float kInf = std::numeric_limits<float>::infinity();

struct Grid {
    std::int64_t w, h;
    bool inside(std::int64_t x, std::int64_t y) const { return x >= 0 && y >= 0 && x < w && y < h; }
    std::int64_t idx(std::int64_t x, std::int64_t y) const { return x + y * w; }
};

// Offsets in the order the reference visits a cell's 4-neighbourhood when it
// seeds the open list (k_border_directions, src/eikonal_fim.cpp:7, also
// src/eikonal_hcm.cpp:18): -x, -y, +x, +y.
constexpr int kSeedDirs[4][2] = {{-1, 0}, {0, -1}, {1, 0}, {0, 1}};
// Order in which a converged cell tries its neighbours
// (add_neighbour_axis(x) then (y), each -axis before +axis:
// src/eikonal_fim.cpp:70-75): -x, +x, -y, +y.
constexpr int kNbrDirs[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};

// The reference CPU 2-D Godunov update, eikonal_solve<2> (src/eikonal.h:121-137).
// `a <= b` are the sorted per-axis neighbour minima. Note the one-finite-axis
// branches return cost + axis WITHOUT the min against the current time; the
// device twin (data/eikonal_common.cl:288-308) keeps that min everywhere.
template <typename F>
inline F godunov_cpu(F a, F b, F cost, F t_cur) {
    if (std::isinf(a)) return cost + b;
    if (std::isinf(b)) return cost + a;
    F const d = a - b;
    if (cost < std::fabs(d)) return std::min(t_cur, std::min(a, b) + cost);
    F const q = cost * cost * 2 - d * d;
    F const p = (a + b + std::sqrt(q)) / 2;
    return std::min(t_cur, p);
}

// The device form (data/eikonal_common.cl:288-308): min(t_cur, update) in all
// branches. Used for the fixed-point residual only.
inline float godunov_dev(float a, float b, float cost, float t_cur) {
    float r;
    if (std::isinf(a)) r = cost + b;
    else if (std::isinf(b)) r = cost + a;
    else {
        float const d = a - b;
        if (cost < std::fabs(d)) r = std::min(a, b) + cost;
        else {
            float const q = cost * cost * 2 - d * d;
            r = (a + b + std::sqrt(q)) / 2;
        }
    }
    return std::min(t_cur, r);
}

template <typename F>
struct FieldView {
    Grid g;
    std::vector<F>& t;
    F at(std::int64_t x, std::int64_t y) const {
        return g.inside(x, y) ? t[g.idx(x, y)] : std::numeric_limits<F>::infinity();
    }
    // sorted per-axis minima of the 4-neighbourhood (src/eikonal_fim.cpp:31-34)
    void axes(std::int64_t x, std::int64_t y, F& lo, F& hi) const {
        F const ax = std::min(at(x + 1, y), at(x - 1, y));
        F const ay = std::min(at(x, y + 1), at(x, y - 1));
        lo = std::min(ax, ay);
        hi = std::max(ax, ay);
    }
};

// ---------------------------------------------------------------------------
// Sequential FIM, restating eikonal_fim_sequential (src/eikonal_fim.cpp:13-107).
// ---------------------------------------------------------------------------
std::int64_t fim_sequential(float eps, const float* cost, Grid g, const std::uint32_t* seeds,
                            std::uint32_t n_seeds, float* out) {
    std::vector<float> t(static_cast<size_t>(g.w * g.h), kInf);
    std::vector<std::uint8_t> open(t.size(), 0);
    std::deque<std::int64_t> fifo;  // packed x + y * W
    FieldView<float> fv{g, t};
    auto cost_at = [&](std::int64_t x, std::int64_t y) { return g.inside(x, y) ? cost[g.idx(x, y)] : kInf; };

    struct Solved { float old_t, new_t, diff; };
    auto solve_at = [&](std::int64_t x, std::int64_t y) {
        float lo, hi;
        fv.axes(x, y, lo, hi);
        Solved s;
        s.old_t = t[g.idx(x, y)];
        s.new_t = godunov_cpu<float>(lo, hi, cost[g.idx(x, y)], s.old_t);
        s.diff = (s.new_t == s.old_t) ? 0.f : s.new_t - s.old_t;  // src/eikonal.h:142-143
        return s;
    };

    auto const t0 = std::chrono::high_resolution_clock::now();
    for (std::uint32_t i = 0; i < n_seeds; ++i) {
        std::int64_t const sx = seeds[2 * i], sy = seeds[2 * i + 1];
        t[g.idx(sx, sy)] = 0.f;
        for (auto const& d : kSeedDirs) {
            std::int64_t const x = sx + d[0], y = sy + d[1];
            if (!g.inside(x, y)) continue;
            open[g.idx(x, y)] = 1;
            fifo.push_back(g.idx(x, y));
        }
    }
    while (!fifo.empty()) {
        std::int64_t const p = fifo.front();
        fifo.pop_front();
        std::int64_t const px = p % g.w, py = p / g.w;
        Solved const s = solve_at(px, py);
        t[p] = s.new_t;
        if (eps < std::fabs(s.diff)) {  // not converged: revisit later
            fifo.push_back(p);
            continue;
        }
        for (auto const& d : kNbrDirs) {
            std::int64_t const x = px + d[0], y = py + d[1];
            if (cost_at(x, y) == kInf) continue;  // also rejects cells outside the field
            std::int64_t const q = g.idx(x, y);
            if (open[q]) continue;
            Solved const sn = solve_at(x, y);
            if (sn.diff < 0) {
                t[q] = sn.new_t;
                open[q] = 1;
                fifo.push_back(q);
            }
        }
        open[p] = 0;
    }
    auto const t1 = std::chrono::high_resolution_clock::now();
    std::memcpy(out, t.data(), t.size() * sizeof(float));
    return std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count();
}

// ---------------------------------------------------------------------------
// Sequential FMM, restating eikonal_fmm_sequential (src/eikonal_fmm.cpp:13-71),
// in F = float (the reference's precision) or F = double (the FP64 oracle).
// ---------------------------------------------------------------------------
template <typename F>
struct HeapItem {
    std::int64_t x, y;
    F t;
    // std::priority_queue is a max-heap on operator<: invert for a min-heap,
    // exactly as CellRef::operator< (src/eikonal_fmm.cpp:18-19).
    bool operator<(HeapItem const& o) const { return t > o.t; }
};

template <typename F>
std::int64_t fmm_sequential(const float* cost, Grid g, const std::uint32_t* seeds, std::uint32_t n_seeds,
                            F* out) {
    F const inf = std::numeric_limits<F>::infinity();
    std::vector<F> t(static_cast<size_t>(g.w * g.h), inf);
    FieldView<F> fv{g, t};
    auto cost_at = [&](std::int64_t x, std::int64_t y) -> F {
        return g.inside(x, y) ? static_cast<F>(cost[g.idx(x, y)]) : inf;
    };
    std::priority_queue<HeapItem<F>> heap;

    auto const t0 = std::chrono::high_resolution_clock::now();
    for (std::uint32_t i = 0; i < n_seeds; ++i)
        heap.push({static_cast<std::int64_t>(seeds[2 * i]), static_cast<std::int64_t>(seeds[2 * i + 1]), F(0)});
    while (!heap.empty()) {
        HeapItem<F> const c = heap.top();
        heap.pop();
        F& tc = t[g.idx(c.x, c.y)];
        if (tc <= c.t) continue;  // lazy deletion: already accepted with a smaller time
        tc = c.t;
        for (auto const& d : kNbrDirs) {
            std::int64_t const x = c.x + d[0], y = c.y + d[1];
            if (!(cost_at(x, y) < inf) || fv.at(x, y) != inf) continue;
            F lo, hi;
            fv.axes(x, y, lo, hi);
            heap.push({x, y, godunov_cpu<F>(lo, hi, cost_at(x, y), inf)});
        }
    }
    auto const t1 = std::chrono::high_resolution_clock::now();
    std::memcpy(out, t.data(), t.size() * sizeof(F));
    return std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count();
}

// ---------------------------------------------------------------------------
// The reference gHCM solve with the systolic kernel, restated on the CPU:
// host scheduler src/eikonal_hcm.cpp:186-482 and device kernel
// data/eikonal_ghcm_systolic.cl:8-175 (+ data/eikonal_common.cl:46-359).
// It reproduces the reference's schedule - stale priority keys, the dirty
// set cleared after a wave's statuses are read (so a block dirtied while in
// flight is not re-queued), check_border writing into the neighbour block -
// to count block-solves and waves. Jobs of one wave, which the reference runs
// concurrently, run here one after another; inside a job, every work-group
// chunk is updated Jacobi-style (all lanes read, then all write), as the
// lock-step wavefront does.
// ---------------------------------------------------------------------------
struct HcmCount {
    std::uint64_t block_solves = 0;
    std::uint64_t waves = 0;
};

HcmCount hcm_systolic(float eps, const float* cost, Grid g, const std::uint32_t* seeds, std::uint32_t n_seeds,
                      std::uint32_t block, std::uint32_t max_jobs, std::uint32_t wg, float* out) {
    std::vector<float> t(static_cast<size_t>(g.w * g.h), kInf);
    for (std::uint32_t i = 0; i < n_seeds; ++i) t[g.idx(seeds[2 * i], seeds[2 * i + 1])] = 0.f;
    std::int64_t const bx = (g.w + block - 1) / block, by = (g.h + block - 1) / block;
    std::int64_t const nb = bx * by;
    std::vector<float> smallest(static_cast<size_t>(nb), kInf);
    std::vector<std::uint32_t> border_mask(static_cast<size_t>(nb), 0);
    std::vector<std::uint8_t> dirty(static_cast<size_t>(nb), 0);

    auto calc_min = [&](std::int64_t id) {  // BlockWrapper::calc_min_time
        std::int64_t const cx = id % bx, cy = id / bx;
        float m = smallest[id];
        for (auto const& d : kSeedDirs) {
            std::int64_t const x = cx + d[0], y = cy + d[1];
            if (x >= 0 && y >= 0 && x < bx && y < by) m = std::min(m, smallest[x + y * bx]);
        }
        return m;
    };
    struct Wrapped {
        std::int64_t id;
        float recorded;
        bool operator<(Wrapped const& o) const { return recorded > o.recorded; }
    };
    std::priority_queue<Wrapped> queue;
    {  // seed_map: blocks of the seeds' 4-neighbours, in block-id order
        std::vector<std::int64_t> seed_blocks;
        for (std::uint32_t i = 0; i < n_seeds; ++i)
            for (auto const& d : kSeedDirs) {
                std::int64_t const x = static_cast<std::int64_t>(seeds[2 * i]) + d[0];
                std::int64_t const y = static_cast<std::int64_t>(seeds[2 * i + 1]) + d[1];
                if (g.inside(x, y)) seed_blocks.push_back((x / block) + (y / block) * bx);
            }
        std::stable_sort(seed_blocks.begin(), seed_blocks.end());
        for (std::int64_t id : seed_blocks) {
            if (dirty[id]) continue;
            dirty[id] = 1;
            smallest[id] = 0.f;
            queue.push({id, calc_min(id)});
        }
    }

    HcmCount cnt;
    // one block-solve of the systolic kernel; returns border flags
    auto run_job = [&](std::int64_t id, float& smin, bool flags[4]) {
        std::int64_t const cx = id % bx, cy = id / bx;
        std::int64_t const ox = cx * block, oy = cy * block;
        std::int64_t const sx = std::min<std::int64_t>(block, g.w - ox), sy = std::min<std::int64_t>(block, g.h - oy);
        std::vector<float> cache(static_cast<size_t>(sx * sy));
        for (std::int64_t y = 0; y < sy; ++y)
            for (std::int64_t x = 0; x < sx; ++x) cache[x + y * sx] = t[g.idx(ox + x, oy + y)];
        // local read: tile from the cache, the one-cell ring from the global
        // field, beyond it +inf (in_bounds_padded, data/eikonal_common.cl:199-206)
        auto rd = [&](std::int64_t lx, std::int64_t ly) -> float {
            if (lx < -1 || ly < -1 || lx > sx || ly > sy) return kInf;
            if (lx >= 0 && ly >= 0 && lx < sx && ly < sy) return cache[lx + ly * sx];
            std::int64_t const x = ox + lx, y = oy + ly;
            return g.inside(x, y) ? t[g.idx(x, y)] : kInf;
        };
        auto cost_at = [&](std::int64_t lx, std::int64_t ly) {
            std::int64_t const x = ox + lx, y = oy + ly;
            return g.inside(x, y) ? cost[g.idx(x, y)] : 0.f;  // field_get_cost(info, 0.f, ...)
        };
        auto update = [&](std::int64_t lx, std::int64_t ly) {
            float const ax = std::min(rd(lx - 1, ly), rd(lx + 1, ly));
            float const ay = std::min(rd(lx, ly - 1), rd(lx, ly + 1));
            return godunov_dev(std::min(ax, ay), std::max(ax, ay), cost_at(lx, ly), rd(lx, ly));
        };
        smin = kInf;
        std::int64_t const len = sx * sy;
        std::vector<float> nw(static_cast<size_t>(wg));
        for (;;) {
            bool converged = true;
            for (std::int64_t base = 0; base < len; base += wg) {
                std::int64_t const end = std::min<std::int64_t>(len, base + wg);
                for (std::int64_t i = base; i < end; ++i) nw[i - base] = update(i % sx, i / sx);
                for (std::int64_t i = base; i < end; ++i) {
                    float const old = cache[i];
                    float const v = nw[i - base];
                    cache[i] = v;
                    smin = std::min(smin, v);
                    float const diff = (v == old) ? 0.f : v - old;
                    converged &= -eps < diff;
                }
            }
            if (converged) break;
        }
        // check_border: solve the neighbour's edge row and store if better
        for (int e = 0; e < 4; ++e) {
            flags[e] = false;
            std::int64_t const nx = cx + (e == 0 ? -1 : e == 2 ? 1 : 0), ny = cy + (e == 1 ? -1 : e == 3 ? 1 : 0);
            if (nx < 0 || ny < 0 || nx >= bx || ny >= by) continue;
            std::int64_t const blen = (e == 0 || e == 2) ? sy : sx;
            std::vector<float> vals(static_cast<size_t>(blen));
            std::vector<std::int64_t> px(static_cast<size_t>(blen)), py(static_cast<size_t>(blen));
            for (std::int64_t i = 0; i < blen; ++i) {
                px[i] = e == 0 ? -1 : e == 2 ? sx : i;
                py[i] = e == 1 ? -1 : e == 3 ? sy : i;
                vals[i] = update(px[i], py[i]);
            }
            for (std::int64_t i = 0; i < blen; ++i) {
                float const old = rd(px[i], py[i]);
                t[g.idx(ox + px[i], oy + py[i])] = vals[i];
                smin = std::min(smin, vals[i]);
                float const diff = (vals[i] == old) ? 0.f : vals[i] - old;
                flags[e] = flags[e] || diff <= -eps;
            }
        }
        for (std::int64_t y = 0; y < sy; ++y)
            for (std::int64_t x = 0; x < sx; ++x) t[g.idx(ox + x, oy + y)] = cache[x + y * sx];
    };

    std::vector<std::int64_t> jobs;
    while (!queue.empty()) {
        jobs.clear();
        while (jobs.size() < max_jobs && !queue.empty()) {
            jobs.push_back(queue.top().id);
            border_mask[queue.top().id] = 0;
            queue.pop();
        }
        cnt.waves += 1;
        std::vector<std::pair<float, std::array<bool, 4>>> status(jobs.size());
        for (size_t j = 0; j < jobs.size(); ++j) {
            bool f[4];
            run_job(jobs[j], status[j].first, f);
            for (int e = 0; e < 4; ++e) status[j].second[e] = f[e];
        }
        cnt.block_solves += jobs.size();
        for (size_t j = 0; j < jobs.size(); ++j) {
            std::int64_t const id = jobs[j];
            smallest[id] = status[j].first;
            std::int64_t const cx = id % bx, cy = id / bx;
            for (int e = 0; e < 4; ++e) {
                // k_border_directions order: -x, -y, +x, +y
                std::int64_t const x = cx + kSeedDirs[e][0], y = cy + kSeedDirs[e][1];
                if (!status[j].second[e] || x < 0 || y < 0 || x >= bx || y >= by) continue;
                std::int64_t const nid = x + y * bx;
                if (!dirty[nid]) {
                    dirty[nid] = 1;
                    queue.push({nid, calc_min(nid)});
                }
                border_mask[nid] |= 1u << (8 * ((e + 2) & 3));
            }
        }
        for (std::int64_t id : jobs) dirty[id] = 0;
    }
    std::memcpy(out, t.data(), t.size() * sizeof(float));
    return cnt;
}

bool valid_seeds(Grid g, const std::uint32_t* seeds, std::uint32_t n) {
    if (n && !seeds) return false;
    for (std::uint32_t i = 0; i < n; ++i)
        if (!g.inside(seeds[2 * i], seeds[2 * i + 1])) return false;
    return true;
}

}  // namespace

extern "C" {

// Sequential FIM (FP32). Returns 0, or -1 on a bad argument.
int ghcm_oracle_fim(float eps, const float* cost, std::uint32_t w, std::uint32_t h, const std::uint32_t* seeds_xy,
                    std::uint32_t n_seeds, float* time_out, std::int64_t* elapsed_us) {
    Grid const g{w, h};
    if (!cost || !time_out || w == 0 || h == 0 || !valid_seeds(g, seeds_xy, n_seeds)) return -1;
    std::int64_t const us = fim_sequential(eps, cost, g, seeds_xy, n_seeds, time_out);
    if (elapsed_us) *elapsed_us = us;
    return 0;
}

// Sequential FMM in FP32, as the reference computes it.
int ghcm_oracle_fmm(const float* cost, std::uint32_t w, std::uint32_t h, const std::uint32_t* seeds_xy,
                    std::uint32_t n_seeds, float* time_out, std::int64_t* elapsed_us) {
    Grid const g{w, h};
    if (!cost || !time_out || w == 0 || h == 0 || !valid_seeds(g, seeds_xy, n_seeds)) return -1;
    std::int64_t const us = fmm_sequential<float>(cost, g, seeds_xy, n_seeds, time_out);
    if (elapsed_us) *elapsed_us = us;
    return 0;
}

// The same FMM carried out in FP64 on the FP32 cost field: the accuracy oracle.
int ghcm_oracle_fmm64(const float* cost, std::uint32_t w, std::uint32_t h, const std::uint32_t* seeds_xy,
                      std::uint32_t n_seeds, double* time_out, std::int64_t* elapsed_us) {
    Grid const g{w, h};
    if (!cost || !time_out || w == 0 || h == 0 || !valid_seeds(g, seeds_xy, n_seeds)) return -1;
    std::int64_t const us = fmm_sequential<double>(cost, g, seeds_xy, n_seeds, time_out);
    if (elapsed_us) *elapsed_us = us;
    return 0;
}

// Largest fixed-point residual T - G(T) over cells with finite cost, where G
// is the device-form Godunov update (data/eikonal_common.cl:288-308). A field
// converged to eps has a residual of at most about eps.
double ghcm_oracle_residual(const float* cost, const float* time, std::uint32_t w, std::uint32_t h) {
    Grid const g{w, h};
    std::vector<float> t(time, time + static_cast<size_t>(w) * h);
    FieldView<float> fv{g, t};
    double worst = 0.0;
    for (std::int64_t y = 0; y < g.h; ++y)
        for (std::int64_t x = 0; x < g.w; ++x) {
            float const c = cost[g.idx(x, y)];
            if (!(c < kInf)) continue;
            float lo, hi;
            fv.axes(x, y, lo, hi);
            float const cur = t[g.idx(x, y)];
            float const nxt = godunov_dev(lo, hi, c, cur);
            if (cur == nxt) continue;
            double const r = std::isinf(cur) ? std::numeric_limits<double>::infinity() : double(cur) - double(nxt);
            worst = std::max(worst, r);
        }
    return worst;
}

// The reference's gHCM schedule with the systolic kernel (see hcm_systolic):
// arrival times into time_out, block-solve and wave counts into counts[0..1].
int ghcm_oracle_hcm(float eps, const float* cost, std::uint32_t w, std::uint32_t h, const std::uint32_t* seeds_xy,
                    std::uint32_t n_seeds, std::uint32_t block, std::uint32_t max_jobs, std::uint32_t wg,
                    float* time_out, std::uint64_t* counts) {
    Grid const g{w, h};
    if (!cost || !time_out || !counts || w == 0 || h == 0 || block == 0 || max_jobs == 0 || wg == 0 ||
        !valid_seeds(g, seeds_xy, n_seeds))
        return -1;
    HcmCount const c = hcm_systolic(eps, cost, g, seeds_xy, n_seeds, block, max_jobs, wg, time_out);
    counts[0] = c.block_solves;
    counts[1] = c.waves;
    return 0;
}

// Runs `count` independent FMM (kind 0) or FIM (kind 1) solves of the same
// field on `threads` host threads and returns the wall time in microseconds:
// the all-cores CPU throughput baseline. Each solve writes its own copy of the
// output; the copy of solve 0 is returned in time_out.
std::int64_t ghcm_oracle_throughput(int kind, float eps, const float* cost, std::uint32_t w, std::uint32_t h,
                                    const std::uint32_t* seeds_xy, std::uint32_t n_seeds, std::uint32_t count,
                                    std::uint32_t threads, float* time_out) {
    Grid const g{w, h};
    if (!cost || !time_out || w == 0 || h == 0 || !valid_seeds(g, seeds_xy, n_seeds) || count == 0) return -1;
    threads = std::max<std::uint32_t>(1, std::min(threads, count));
    std::vector<std::vector<float>> outs(threads, std::vector<float>(static_cast<size_t>(w) * h));
    auto const t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    for (std::uint32_t k = 0; k < threads; ++k) {
        pool.emplace_back([&, k] {
            for (std::uint32_t j = k; j < count; j += threads) {
                if (kind == 0) fmm_sequential<float>(cost, g, seeds_xy, n_seeds, outs[k].data());
                else fim_sequential(eps, cost, g, seeds_xy, n_seeds, outs[k].data());
            }
        });
    }
    for (auto& th : pool) th.join();
    auto const t1 = std::chrono::steady_clock::now();
    std::memcpy(time_out, outs[0].data(), outs[0].size() * sizeof(float));
    return std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count();
}

}  // extern "C"

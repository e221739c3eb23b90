// Per-level autotuner (see autotune.hpp).
//
// 1. Launch shapes, level by level: the level's Jacobi sweep is timed with one and with two
//    tiles per thread (and, on the fine level, the vector update with one and four), with
//    CUDA events on the solve's stream; the faster shape is kept. Levels with fewer than
//    two waves of tiles keep one tile per thread: there every block counts.
// 2. Sweeps: whole solves of the batch's system are timed for a list of candidates
//    (uniform pre/post sweeps and damping; then, around the best, the coarse levels'
//    sweeps, the fine level's sweeps, the damping); a candidate counts only if every
//    planet meets its tolerance. Each candidate runs once untimed first (CUDA graph
//    recording), then once timed.
#include "autotune.hpp"

#include "kernels.hpp"
#include "profile.hpp"

#include <algorithm>
#include <chrono>
#include <stdexcept>

namespace psgb {

namespace {

constexpr std::uint32_t kMinTunedTiles = 2 * 152;   // below: one tile per thread
constexpr int kTimedLaunches = 10;

struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    EventPair() {
        PSGB_CUDA(cudaEventCreate(&a));
        PSGB_CUDA(cudaEventCreate(&b));
    }
    ~EventPair() {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
};

template <typename T>
LevelView<T> view_of(const Batch& b, std::size_t l);
template <>
LevelView<float> view_of<float>(const Batch& b, std::size_t l) { return view32(b, l); }
template <>
LevelView<double> view_of<double>(const Batch& b, std::size_t l) { return view64(b, l); }

template <typename T>
struct Vecs {
    T *x, *y, *rhs;
};
template <typename T>
Vecs<T> vecs_of(BatchLevel& L);
template <>
Vecs<float> vecs_of<float>(BatchLevel& L) { return {L.x32, L.y32, L.b32}; }
template <>
Vecs<double> vecs_of<double>(BatchLevel& L) { return {L.x64, L.y64, L.b64}; }

// Mean device time of `launch` over kTimedLaunches launches (after warm-up).
template <typename F>
double time_launches(cudaStream_t st, F&& launch) {
    EventPair ev;
    for (int k = 0; k < 3; ++k) launch();
    PSGB_CUDA(cudaEventRecord(ev.a, st));
    for (int k = 0; k < kTimedLaunches; ++k) launch();
    PSGB_CUDA(cudaEventRecord(ev.b, st));
    PSGB_CUDA(cudaEventSynchronize(ev.b));
    float ms = 0.0F;
    PSGB_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
    return static_cast<double>(ms) / kTimedLaunches;
}

template <typename T>
void tune_shapes(Batch& b, cudaStream_t st) {
    const T omega = static_cast<T>(b.smoother.omega);
    for (std::size_t l = 0; l < b.levels.size(); ++l) {
        BatchLevel& L = b.levels[l];
        if (L.tiles < kMinTunedTiles) {
            L.sets_stencil = 1;
            L.sets_vector = 1;
            continue;
        }
        const Vecs<T> v = vecs_of<T>(L);
        double best = 0.0;
        std::uint8_t pick = 1;
        for (std::uint8_t sets : {std::uint8_t(1), std::uint8_t(2)}) {
            L.sets_stencil = sets;
            const LevelView<T> lv = view_of<T>(b, l);
            const double ms = time_launches(st, [&] { launch_smooth<T>(lv, v.rhs, v.x, v.y, omega, b.scalars, kGateAlways, st); });
            if (sets == 1 || ms < best) { best = ms; pick = sets; }
        }
        L.sets_stencil = pick;
        if (l != 0) continue;
        pick = 1;
        for (std::uint8_t sets : {std::uint8_t(1), std::uint8_t(4)}) {
            L.sets_vector = sets;
            const LevelView<T> lv = view_of<T>(b, l);
            const double ms = time_launches(st, [&] { launch_smooth_zero<T>(lv, v.rhs, v.x, omega, b.scalars, kGateAlways, st); });
            if (sets == 1 || ms < best) { best = ms; pick = sets; }
        }
        L.sets_vector = pick;
    }
    // Where the coarse tail starts (or none): time whole V-cycles over every planet.
    T* rhs = vecs_of<T>(b.levels[0]).rhs;
    T* x = vecs_of<T>(b.levels[0]).x;
    double best = -1.0;
    int pick = b.tail_level;
    for (int tail = 0; tail < static_cast<int>(b.levels.size()); ++tail) {
        b.tail_level = tail;
        const double ms = time_launches(st, [&] { vcycle<T>(b, rhs, x, kGateAlways, false, st); });
        if (best < 0.0 || ms < best) { best = ms; pick = tail; }
    }
    b.tail_level = pick;
    PSGB_CUDA(cudaGetLastError());
}

struct Sweeps {
    std::vector<int> pre, post;
    double omega;
    std::vector<int> inner;    // empty: one sweep per launch everywhere
    double correction = 1.0;   // coarse-grid correction scale
};

void set_sweeps(Batch& b, const Sweeps& s) {
    b.smoother.level_pre = s.pre;
    b.smoother.level_post = s.post;
    b.smoother.level_inner = s.inner;
    b.smoother.omega = s.omega;
    b.smoother.correction = s.correction;
}

bool all_ok(const Batch& b) {
    for (const InstanceScalars& s : b.host_scalars)
        if (s.outer_status != kConverged) return false;
    return true;
}

// Wall time of one solve (ms) from the initial guess x0 (null: zero); negative if some
// planet missed its tolerance.
double trial(Batch& b, const SolveOptions& opt, const double* rhs, const double* x0, double* x, std::size_t rows,
             cudaStream_t st, int& count) {
    ++count;
    if (x0 != nullptr) {
        PSGB_CUDA(cudaMemcpyAsync(x, x0, rows * sizeof(double), cudaMemcpyDeviceToDevice, st));
    } else {
        PSGB_CUDA(cudaMemsetAsync(x, 0, rows * sizeof(double), st));
    }
    PSGB_CUDA(cudaStreamSynchronize(st));
    const auto t0 = std::chrono::steady_clock::now();
    solve(b, opt, rhs, x, st);
    PSGB_CUDA(cudaStreamSynchronize(st));
    const auto t1 = std::chrono::steady_clock::now();
    if (!all_ok(b)) return -1.0;
    return std::chrono::duration<double, std::milli>(t1 - t0).count();
}

}  // namespace

Tuning current_tuning(const Batch& b) {
    Tuning t;
    for (std::size_t l = 0; l < b.levels.size(); ++l) {
        t.pre.push_back(b.smoother.pre_at(l));
        t.post.push_back(b.smoother.post_at(l));
        t.inner.push_back(b.smoother.inner_at(l));
        t.sets_stencil.push_back(b.levels[l].sets_stencil);
        t.sets_vector.push_back(b.levels[l].sets_vector);
    }
    t.omega = b.smoother.omega;
    t.correction = b.smoother.correction;
    t.tail_level = b.tail_level;
    t.tail_spread = b.tail_spread;
    t.tail_shared = b.tail_shared;
    t.tail_cluster = b.tail_cluster;
    // the tail launch last built, else the one the settings ask for
    t.tail_blocks = b.tail_level == 0             ? 0u
                    : b.tail_launch_blocks != 0   ? b.tail_launch_blocks
                    : b.tail_cluster != 0         ? b.instances * b.tail_cluster
                    : b.tail_shared               ? b.instances
                    : (b.tail_spread && b.tail_cta_at[b.tail_level] != nullptr) ? b.tail_ctas_at[b.tail_level]
                                                                                 : b.instances;
    return t;
}

void apply_tuning(Batch& b, const Tuning& t) {
    const std::size_t depth = b.levels.size();
    if (t.pre.size() != depth || t.post.size() != depth || t.sets_stencil.size() != depth || t.sets_vector.size() != depth ||
        (!t.inner.empty() && t.inner.size() != depth))
        throw std::invalid_argument("tuning levels do not match the batch");
    for (int k : t.inner)
        if (k < 1 || k > 8) throw std::invalid_argument("block-local sweeps must be 1..8");
    for (std::size_t l = 0; l < depth; ++l) {
        if (t.pre[l] < 1 || t.pre[l] > 8 || t.post[l] < 0 || t.post[l] > 8)
            throw std::invalid_argument("tuned sweeps must be 1..8 (pre) and 0..8 (post)");
        if ((t.sets_stencil[l] != 1 && t.sets_stencil[l] != 2) || (t.sets_vector[l] != 1 && t.sets_vector[l] != 4))
            throw std::invalid_argument("tuned tile sets must be 1 or 2 (stencil) and 1 or 4 (vector)");
    }
    if (!(t.omega > 0.0 && t.omega < 2.0)) throw std::invalid_argument("tuned damping must be in (0, 2)");
    if (!(t.correction > 0.0 && t.correction <= 4.0))
        throw std::invalid_argument("the coarse-grid correction scale must be in (0, 4]");
    if (t.tail_level < 0 || static_cast<std::size_t>(t.tail_level) >= depth)
        throw std::invalid_argument("the coarse tail level must be 0 (none) or a level below the fine one");
    if (t.tail_cluster != 0 && t.tail_cluster != 2 && t.tail_cluster != 4 && t.tail_cluster != 8)
        throw std::invalid_argument("the coarse tail's cluster must be 0 (none), 2, 4 or 8 blocks");
    for (std::size_t l = 0; l < depth; ++l) {
        b.levels[l].sets_stencil = t.sets_stencil[l];
        b.levels[l].sets_vector = t.sets_vector[l];
    }
    b.smoother.level_pre = t.pre;
    b.smoother.level_post = t.post;
    b.smoother.level_inner = t.inner;
    b.smoother.omega = t.omega;
    b.smoother.correction = t.correction;
    b.tail_level = t.tail_level;
    b.tail_spread = t.tail_spread;
    b.tail_shared = t.tail_shared;
    b.tail_cluster = t.tail_cluster;
    b.tail_launch_blocks = 0;
    b.tuned = true;
}

void clear_tuning(Batch& b) {
    b.smoother.level_pre.clear();
    b.smoother.level_post.clear();
    b.smoother.level_inner.clear();
    b.smoother.correction = 1.0;
    default_launch_shapes(b);
    b.tuned = false;
}

Tuning autotune(Batch& b, const SolveOptions& opt, const double* rhs, const double* x0, double* x, cudaStream_t st) {
    if (!b.matrix_ready) throw std::logic_error("autotune before the matrix was set");
    if (profile_active()) throw std::logic_error("autotune while a profile records");
    const std::size_t depth = b.levels.size(), rows = b.levels[0].rows;
    Tuning result;
    // Settings before tuning: the reference point.
    const Sweeps before{std::vector<int>(depth, b.smoother.pre_at(0)), std::vector<int>(depth, b.smoother.post_at(0)),
                        b.smoother.omega, {}};
    set_sweeps(b, before);
    default_launch_shapes(b);
    trial(b, opt, rhs, x0, x, rows, st, result.trials);
    result.default_ms = trial(b, opt, rhs, x0, x, rows, st, result.trials);

    // 1. launch shapes (result-neutral)
    if (opt.precision == kMixed) tune_shapes<float>(b, st);
    else tune_shapes<double>(b, st);

    // 2. sweeps: uniform candidates, then coarse-level variants of the best
    // a candidate's time: the faster of two solves after one that records its graphs (one
    // timing alone lets noise of a few percent flip close choices)
    auto run = [&](const Sweeps& s) {
        set_sweeps(b, s);
        if (trial(b, opt, rhs, x0, x, rows, st, result.trials) < 0.0) return -1.0;
        const double first = trial(b, opt, rhs, x0, x, rows, st, result.trials);
        if (first < 0.0) return -1.0;
        const double second = trial(b, opt, rhs, x0, x, rows, st, result.trials);
        return second < 0.0 ? -1.0 : std::min(first, second);
    };
    Sweeps best = before;
    double best_ms = run(before);
    const struct { int pre, post; double omega; } uniform[] = {
        {1, 1, 1.0}, {1, 1, 0.8}, {2, 2, 1.0}, {2, 1, 0.9}, {1, 2, 0.9}, {3, 3, 0.8}};
    for (const auto& u : uniform) {
        const Sweeps s{std::vector<int>(depth, u.pre), std::vector<int>(depth, u.post), u.omega, {}};
        const double ms = run(s);
        if (ms > 0.0 && (best_ms < 0.0 || ms < best_ms)) { best = s; best_ms = ms; }
    }

    auto consider = [&](const Sweeps& s) {
        const double ms = run(s);
        if (ms > 0.0 && (best_ms < 0.0 || ms < best_ms)) { best = s; best_ms = ms; }
    };
    if (depth > 1) {
        // coarse levels (cheap, latency-bound sweeps) around the best uniform setting
        const int coarse[][2] = {{1, 1}, {2, 2}, {3, 3}, {4, 4}, {6, 6}};
        const Sweeps base = best;
        for (const auto& c : coarse) {
            Sweeps s = base;
            for (std::size_t l = 1; l < depth; ++l) { s.pre[l] = c[0]; s.post[l] = c[1]; }
            if (s.pre == base.pre && s.post == base.post) continue;
            consider(s);
        }
        // then the fine level with the best coarse setting
        const int fine[][2] = {{1, 1}, {2, 2}, {1, 2}, {2, 1}};
        const Sweeps with_coarse = best;
        for (const auto& f : fine) {
            Sweeps s = with_coarse;
            s.pre[0] = f[0];
            s.post[0] = f[1];
            if (s.pre == with_coarse.pre && s.post == with_coarse.post) continue;
            consider(s);
        }
    }
    // block-local sweeps on the coarse levels: several Jacobi sweeps per launch
    // (pre launches + 1, post launches + 1, sweeps per launch): fewer, longer launches trade
    // the latency of a launch against tile-local coupling
    const int block[][3] = {{2, 2, 2}, {2, 2, 3}, {2, 2, 4}, {3, 3, 2}, {3, 3, 3},
                            {2, 2, 6}, {2, 2, 8}, {2, 1, 6}, {2, 1, 8}};
    const auto try_block_sweeps = [&] {
        const Sweeps base = best;
        for (const auto& c : block) {
            Sweeps s = base;
            s.inner.assign(depth, 1);
            for (std::size_t l = 1; l < depth; ++l) { s.pre[l] = c[0]; s.post[l] = c[1]; s.inner[l] = c[2]; }
            if (s.pre == base.pre && s.post == base.post && s.inner == base.inner) continue;
            consider(s);
        }
    };
    if (depth > 1) {
        try_block_sweeps();
        // then the levels below the first coarse one on their own: the smallest levels
        // are pure latency, fewer launches may beat more smoothing there
        if (depth > 2 && !best.inner.empty()) {
            const int deep[][3] = {{1, 1, 1}, {2, 1, 8}, {2, 2, 8}};
            const Sweeps with_first = best;
            for (const auto& c : deep) {
                Sweeps s = with_first;
                for (std::size_t l = 2; l < depth; ++l) { s.pre[l] = c[0]; s.post[l] = c[1]; s.inner[l] = c[2]; }
                if (s.pre == with_first.pre && s.post == with_first.post && s.inner == with_first.inner) continue;
                consider(s);
            }
        }
    }
    // damping around the best
    for (double omega : {0.9, 1.0}) {
        if (omega == best.omega) continue;
        Sweeps s = best;
        s.omega = omega;
        consider(s);
    }
    // over-correction of the coarse-grid correction, then the coarse sweeps again under the
    // chosen scale (a stronger correction may do with fewer or shorter sweeps)
    if (depth > 1) {
        const Sweeps base = best;
        for (double c : {1.5, 2.0}) {
            Sweeps s = base;
            s.correction = c;
            consider(s);
        }
        if (best.correction != base.correction) try_block_sweeps();
    }
    // where the coarse tail starts, with the chosen sweeps (whole solves: the tail's cost
    // depends on how many sweeps its levels run)
    set_sweeps(b, best);
    {
        // modes: 0 spread over co-resident blocks, 1 one block per planet, 2 one block per
        // planet with the levels' vectors in shared memory, 3/4/5 a cluster of 2/4/8 blocks
        // per planet with the vectors in its distributed shared memory
        const auto mode_of = [&] {
            if (b.tail_cluster != 0) return b.tail_cluster == 2 ? 3 : (b.tail_cluster == 4 ? 4 : 5);
            return b.tail_shared ? 2 : (b.tail_spread ? 0 : 1);
        };
        const auto set_mode = [&](int mode) {
            b.tail_shared = mode == 2;
            b.tail_spread = mode == 0;
            b.tail_cluster = mode >= 3 ? 1u << (mode - 2) : 0u;
            b.tail_launch_blocks = 0;
        };
        const int chosen = b.tail_level;
        const int chosen_mode = mode_of();
        int pick = chosen, pick_mode = chosen_mode;
        const bool mixed = opt.precision == kMixed;
        for (int tail = 0; tail < static_cast<int>(depth); ++tail) {
            for (int mode : {0, 1, 2, 3, 4, 5}) {
                if ((tail == chosen && mode == chosen_mode) || (tail == 0 && mode != 0)) continue;
                if (mode == 2 && !(mixed ? tail_fits_shared<float>(b, tail) : tail_fits_shared<double>(b, tail))) continue;
                const unsigned cluster = mode >= 3 ? 1u << (mode - 2) : 0u;
                if (mode >= 3 && !(mixed ? tail_fits_cluster<float>(b, tail, cluster)
                                         : tail_fits_cluster<double>(b, tail, cluster)))
                    continue;
                b.tail_level = tail;
                set_mode(mode);
                const double ms = run(best);
                if (ms > 0.0 && ms < best_ms) { best_ms = ms; pick = tail; pick_mode = mode; }
            }
        }
        b.tail_level = pick;
        set_mode(pick_mode);
    }
    // the fine level's tile-set sizes again, by whole solves with everything else chosen: a
    // sweep launch timed alone favours two tiles a thread, while whole solves (many short
    // launches overlapping, lanes beside each other) measured faster with one on the
    // 64-planet mix and on one L8 planet
    if (best_ms > 0.0 && b.levels[0].tiles >= kMinTunedTiles) {
        BatchLevel& F = b.levels[0];
        const std::uint8_t s0 = F.sets_stencil, v0 = F.sets_vector;
        std::uint8_t ps = s0, pv = v0;
        for (std::uint8_t s : {std::uint8_t(1), std::uint8_t(2)}) {
            for (std::uint8_t v : {std::uint8_t(1), std::uint8_t(4)}) {
                if (s == s0 && v == v0) continue;
                F.sets_stencil = s;
                F.sets_vector = v;
                const double ms = run(best);
                if (ms > 0.0 && ms < best_ms) { best_ms = ms; ps = s; pv = v; }
            }
        }
        F.sets_stencil = ps;
        F.sets_vector = pv;
    }
    if (best_ms < 0.0) {
        set_sweeps(b, before);
        throw std::runtime_error("autotune: no candidate met the tolerance on every planet");
    }
    set_sweeps(b, best);
    b.tuned = true;
    result.pre = best.pre;
    result.post = best.post;
    result.inner = best.inner.empty() ? std::vector<int>(depth, 1) : best.inner;
    result.omega = best.omega;
    result.correction = best.correction;
    for (std::size_t l = 0; l < depth; ++l) {
        result.sets_stencil.push_back(b.levels[l].sets_stencil);
        result.sets_vector.push_back(b.levels[l].sets_vector);
    }
    result.tail_level = b.tail_level;
    result.tail_spread = b.tail_spread;
    result.tail_shared = b.tail_shared;
    result.tail_cluster = b.tail_cluster;
    result.tuned_ms = best_ms;
    return result;
}

}  // namespace psgb

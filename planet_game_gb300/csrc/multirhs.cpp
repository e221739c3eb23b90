// Host driver of the multi-right-hand-side block solve (multirhs.hpp). It runs, for all
// right-hand sides at once, exactly the sequence of phases the single solve of a
// one-planet batch runs (solver.cpp: the FP64 refinement loop, BiCGSTAB, the V-cycle with
// its zero-start sweeps fused into the Krylov updates), so each right-hand side follows its
// own single solve.
#include "multirhs.hpp"

#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <type_traits>

namespace psgb {
namespace mr {

Space::~Space() {
    if (pinned != nullptr) cudaFreeHost(pinned);
}

namespace {

template <typename T>
struct Sel;
template <>
struct Sel<double> {
    static std::vector<double*>& x(Space& s) { return s.x64; }
    static std::vector<double*>& y(Space& s) { return s.y64; }
    static std::vector<double*>& b(Space& s) { return s.b64; }
    static std::vector<double*>& r(Space& s) { return s.r64; }
    static double** k(Space& s) { return s.k64; }
    static LevelView<double> view(const Batch& bt, std::size_t l) { return view64(bt, l); }
    static const double* dense_inv(const Batch& bt) { return bt.dense.inv64; }
};
template <>
struct Sel<float> {
    static std::vector<float*>& x(Space& s) { return s.x32; }
    static std::vector<float*>& y(Space& s) { return s.y32; }
    static std::vector<float*>& b(Space& s) { return s.b32; }
    static std::vector<float*>& r(Space& s) { return s.r32; }
    static float** k(Space& s) { return s.k32; }
    static LevelView<float> view(const Batch& bt, std::size_t l) { return view32(bt, l); }
    static const float* dense_inv(const Batch& bt) { return bt.dense.inv32; }
};

template <typename T>
T* zeroed(DeviceStore& store, std::size_t count) {
    T* p = store.alloc<T>(count);
    PSGB_CUDA(cudaMemset(p, 0, count * sizeof(T)));
    return p;
}

template <typename T>
void lay_out(Batch& b, Space& s) {
    const std::size_t P0 = b.levels[0].rows;
    for (std::size_t l = 0; l < b.levels.size(); ++l) {
        const std::size_t n = std::size_t(b.levels[l].rows) * kRhs;
        Sel<T>::x(s).push_back(zeroed<T>(s.store, n));
        Sel<T>::y(s).push_back(zeroed<T>(s.store, n));
        Sel<T>::b(s).push_back(zeroed<T>(s.store, n));
        Sel<T>::r(s).push_back(zeroed<T>(s.store, n));
    }
    for (int v = 0; v < Batch::kVectors; ++v) Sel<T>::k(s)[v] = zeroed<T>(s.store, P0 * kRhs);
}

// Every right-hand side's refinement (outer) or inner solve finished?
bool all_done(Space& s, cudaStream_t st, bool outer) {
    PSGB_CUDA(cudaMemcpyAsync(s.pinned, s.sc, kRhs * sizeof(InstanceScalars), cudaMemcpyDeviceToHost, st));
    PSGB_CUDA(cudaStreamSynchronize(st));
    for (int j = 0; j < kRhs; ++j) {
        const InstanceScalars& c = s.pinned[j];
        if (outer ? c.outer_status == kRunning : (c.outer_status == kRunning && c.status == kRunning)) return false;
    }
    return true;
}

template <typename T>
T* first_target(Batch& b, Space& s, T* x) {
    return b.smoother.starts_in_x(0) ? x : Sel<T>::y(s)[0];
}

// The single solve's V-cycle (solver.cpp vcycle) for every right-hand side, the zero-start
// sweep of the fine level done by the Krylov update before it.
template <typename T>
void vcycle(Batch& b, Space& s, const T* rhs, T* x, int gate, cudaStream_t st) {
    using L = Launch<T>;
    const std::size_t depth = b.levels.size();
    const SmootherConfig& sm = b.smoother;
    const T omega = static_cast<T>(sm.omega);
    std::vector<T*> cur(depth), other(depth);
    std::vector<const T*> rhs_of(depth);
    for (std::size_t l = 0; l < depth; ++l) {
        T* X = l == 0 ? x : Sel<T>::x(s)[l];
        T* Y = Sel<T>::y(s)[l];
        cur[l] = sm.starts_in_x(l) ? X : Y;
        other[l] = sm.starts_in_x(l) ? Y : X;
        rhs_of[l] = l == 0 ? rhs : Sel<T>::b(s)[l];
    }
    const int dense_rows = static_cast<int>(b.dense.size[0]);
    const T* dense_inv = Sel<T>::dense_inv(b);
    if (depth == 1) {   // the planet's only level is its coarsest
        L::dense(dense_rows, dense_inv, rhs, x, s.sc, gate, st);
        return;
    }
    for (std::size_t l = 0; l + 1 < depth; ++l) {
        const LevelView<T> lv = Sel<T>::view(b, l);
        for (int k = 1; k < sm.pre_at(l); ++k) {
            L::smooth(lv, rhs_of[l], cur[l], other[l], omega, s.sc, gate, st, sm.inner_at(l));
            std::swap(cur[l], other[l]);
        }
        L::residual(lv, rhs_of[l], cur[l], Sel<T>::r(s)[l], s.sc, gate, st);
        L::restrict_zero(Sel<T>::view(b, l + 1), b.levels[l].member_offset, b.levels[l].member, Sel<T>::r(s)[l],
                         Sel<T>::b(s)[l + 1], cur[l + 1], omega, s.sc, gate, st);
        if (l + 2 == depth) L::dense(dense_rows, dense_inv, Sel<T>::b(s)[l + 1], Sel<T>::x(s)[l + 1], s.sc, gate, st);
    }
    for (std::size_t l = depth - 1; l-- > 0;) {
        const LevelView<T> lv = Sel<T>::view(b, l);
        const T* e = Sel<T>::x(s)[l + 1];
        const bool split = std::is_same<T, double>::value && l == 0;
        if (sm.post_at(l) == 0 || split) {
            L::prolong(lv, b.levels[l].agg, e, cur[l], s.sc, gate, st);
            for (int k = 0; k < sm.post_at(l); ++k) {
                L::smooth(lv, rhs_of[l], cur[l], other[l], omega, s.sc, gate, st, sm.inner_at(l));
                std::swap(cur[l], other[l]);
            }
            continue;
        }
        L::prolong_smooth(lv, b.levels[l].agg, e, rhs_of[l], cur[l], other[l], omega, s.sc, gate, st);
        std::swap(cur[l], other[l]);
        for (int k = 1; k < sm.post_at(l); ++k) {
            L::smooth(lv, rhs_of[l], cur[l], other[l], omega, s.sc, gate, st, sm.inner_at(l));
            std::swap(cur[l], other[l]);
        }
    }
}

// Inner BiCGSTAB, x0 = 0, the single solve's krylov() and krylov_chunk().
template <typename T>
void krylov(Batch& b, Space& s, const SolveOptions& opt, const T* rhs, T* x, double tol, cudaStream_t st) {
    using L = Launch<T>;
    const LevelView<T> lv = Sel<T>::view(b, 0);
    const Ctx ctx{s.part, s.sc};
    T** v = Sel<T>::k(s);
    const T omega_j = static_cast<T>(b.smoother.omega);
    L::bicg_init(lv, rhs, x, v[0], v[1], v[2], v[3], ctx, tol, opt.max_iterations, st);
    T *r = v[0], *shadow = v[1], *p = v[2], *vv = v[3], *phat = v[4], *sv = v[5], *shat = v[6], *t = v[7];
    int it = 0;
    while (it < opt.max_iterations) {
        const int count = std::min(opt.poll, opt.max_iterations - it);
        for (int k = 0; k < count; ++k) {
            L::bicg_p(lv, r, vv, p, first_target<T>(b, s, phat), omega_j, s.sc, st);
            vcycle<T>(b, s, p, phat, kGateRunning, st);
            L::bicg_v(lv, phat, vv, shadow, ctx, st);
            L::bicg_s(lv, r, vv, sv, first_target<T>(b, s, shat), omega_j, ctx, st);
            vcycle<T>(b, s, sv, shat, kGateSecondHalf, st);
            L::bicg_t(lv, shat, t, sv, ctx, st);
            L::bicg_x(lv, phat, shat, sv, t, x, r, shadow, ctx, st);
        }
        it += count;
        PSGB_CUDA(cudaGetLastError());
        if (all_done(s, st, false)) break;
    }
}

template <typename TI>
void refine(Batch& b, Space& s, const SolveOptions& opt, double inner_tol, cudaStream_t st) {
    const LevelView<double> lv64 = view64(b, 0);
    const Ctx ctx{s.part, s.sc};
    TI** v = Sel<TI>::k(s);
    for (int round = 0; round <= opt.max_refinements; ++round) {
        outer_residual<TI>(lv64, s.bb, s.xr, s.rr, v[8], ctx, opt.max_refinements, st);
        if (all_done(s, st, true)) break;
        krylov<TI>(b, s, opt, v[8], v[9], inner_tol, st);
        outer_update<TI>(lv64, v[9], s.xr, s.sc, st);
    }
}

}  // namespace

void prepare(Batch& b, Space& s, const SolveOptions& opt) {
    if (b.instances != 1) throw std::logic_error("the block solve runs on a one-planet batch");
    if (s.xr == nullptr) {
        const std::size_t P0 = b.levels[0].rows;
        s.xr = zeroed<double>(s.store, P0 * kRhs);
        s.rr = zeroed<double>(s.store, P0 * kRhs);
        s.bb = zeroed<double>(s.store, P0 * kRhs);
        s.part = zeroed<double>(s.store, 2 * std::size_t(b.levels[0].tiles) * kRhs);
        s.sc = zeroed<InstanceScalars>(s.store, kRhs);
        s.pointers = s.store.alloc<const double*>(2 * kRhs);
        PSGB_CUDA(cudaMallocHost(&s.pinned, kRhs * sizeof(InstanceScalars)));
        s.host.assign(kRhs, InstanceScalars{});
    }
    if (opt.precision == kFP64 && !s.has64) {
        lay_out<double>(b, s);
        s.has64 = true;
    }
    if (opt.precision == kMixed && !s.has32) {
        lay_out<float>(b, s);
        s.has32 = true;
    }
}

void solve(Batch& b, Space& s, const SolveOptions& opt, cudaStream_t st) {
    if (!b.matrix_ready) throw std::logic_error("block solve before the matrix was set");
    if (opt.method != kBiCGSTAB) throw std::invalid_argument("the multi-right-hand-side block solve runs BiCGSTAB");
    prepare(b, s, opt);
    const LevelView<double> lv64 = view64(b, 0);
    const Ctx ctx{s.part, s.sc};
    const double inner_tol = opt.precision == kMixed ? opt.inner_tolerance : 1e-3 * opt.tolerance;
    outer_init(lv64, s.bb, ctx, opt.tolerance, opt.max_refinements, st);
    if (opt.precision == kMixed) {
        refine<float>(b, s, opt, inner_tol, st);
    } else {
        refine<double>(b, s, opt, inner_tol, st);
    }
    PSGB_CUDA(cudaMemcpyAsync(s.pinned, s.sc, kRhs * sizeof(InstanceScalars), cudaMemcpyDeviceToHost, st));
    PSGB_CUDA(cudaStreamSynchronize(st));
    std::memcpy(s.host.data(), s.pinned, kRhs * sizeof(InstanceScalars));
}

}  // namespace mr
}  // namespace psgb

// Multi-right-hand-side block solve of one planet (multirhs.cu: kernels; multirhs.cpp:
// the host driver). Up to kRhs sub-steps of one planet with one matrix, vectors
// interleaved (row * kRhs + rhs), every right-hand side following the single solve of its
// sub-step bit for bit.
#pragma once

#include "kernels.hpp"
#include "planet.hpp"
#include "solver.hpp"

#include <cstdint>
#include <vector>

namespace psgb {
namespace mr {

constexpr int kRhs = 32;

// Reduction context of the block: FP64 tile partials [quantity][tile][kRhs] and the
// right-hand sides' scalars [kRhs].
struct Ctx {
    double* part;
    InstanceScalars* sc;
};

template <typename T>
struct Launch {
    static void smooth_zero(const LevelView<T>& L, const T* b, T* x, T omega, const InstanceScalars* sc, int gate,
                            cudaStream_t st);
    // inner > 1: that many block-local sweeps of each tile in the launch (the single solve's
    // block sweep)
    static void smooth(const LevelView<T>& L, const T* b, const T* x, T* y, T omega, const InstanceScalars* sc,
                       int gate, cudaStream_t st, int inner = 1);
    static void residual(const LevelView<T>& L, const T* b, const T* x, T* r, const InstanceScalars* sc, int gate,
                         cudaStream_t st);
    static void restrict_zero(const LevelView<T>& C, const std::uint32_t* moff, const std::uint32_t* member,
                              const T* r, T* bc, T* xc, T omega, const InstanceScalars* sc, int gate,
                              cudaStream_t st);
    static void prolong_smooth(const LevelView<T>& L, const std::int32_t* agg, const T* e, const T* b, const T* x,
                               T* y, T omega, const InstanceScalars* sc, int gate, cudaStream_t st);
    static void prolong(const LevelView<T>& L, const std::int32_t* agg, const T* xc, T* x, const InstanceScalars* sc,
                        int gate, cudaStream_t st);
    static void dense(int n, const T* inv, const T* b, T* x, const InstanceScalars* sc, int gate, cudaStream_t st);
    static void bicg_init(const LevelView<T>& L, const T* b, T* x, T* r, T* shadow, T* p, T* v, const Ctx& ctx,
                          double tol, int max_it, cudaStream_t st);
    static void bicg_p(const LevelView<T>& L, const T* r, const T* v, T* p, T* xv, T omega_j,
                       const InstanceScalars* sc, cudaStream_t st);
    static void bicg_v(const LevelView<T>& L, const T* in, T* out, const T* shadow, const Ctx& ctx, cudaStream_t st);
    static void bicg_s(const LevelView<T>& L, const T* r, const T* v, T* s, T* xv, T omega_j, const Ctx& ctx,
                       cudaStream_t st);
    static void bicg_t(const LevelView<T>& L, const T* shat, T* t, const T* s, const Ctx& ctx, cudaStream_t st);
    static void bicg_x(const LevelView<T>& L, const T* phat, const T* shat, const T* s, const T* t, T* x, T* r,
                       const T* shadow, const Ctx& ctx, cudaStream_t st);
};

void outer_init(const LevelView<double>& L, const double* b, const Ctx& ctx, double tol, int max_refine,
                cudaStream_t st);
template <typename TI>
void outer_residual(const LevelView<double>& L, const double* b, const double* x, double* r64, TI* rin, const Ctx& ctx,
                    int max_refine, cudaStream_t st);
template <typename TI>
void outer_update(const LevelView<double>& L, const TI* delta, double* x, InstanceScalars* sc, cudaStream_t st);
// Right-hand sides (A / s) T0_j + A S_j and initial guesses T0_j of `count` sub-steps
// (device pointer arrays t0[count], src[count] of n entries each) into the interleaved
// rhs and x0; the unused right-hand sides and padding rows zero.
void load(std::uint32_t n, std::uint32_t P, int count, const double* const* t0, const double* const* src,
          const double* area, double slope, double* rhs, double* x0, cudaStream_t st);
// Right-hand side j of an interleaved vector into a vector of P entries.
void take(std::uint32_t P, int j, const double* x, double* out, cudaStream_t st);

// Device workspace of a planet's block solves, allocated on first use (per precision).
struct Space {
    DeviceStore store;
    std::vector<double*> x64, y64, b64, r64;   // per level, [rows][kRhs]
    std::vector<float*> x32, y32, b32, r32;
    double* k64[Batch::kVectors] = {};
    float* k32[Batch::kVectors] = {};
    double* xr = nullptr;     // solution, FP64
    double* rr = nullptr;     // residual, FP64
    double* bb = nullptr;     // right-hand sides, FP64
    double* part = nullptr;   // [2][tiles of the fine level][kRhs]
    InstanceScalars* sc = nullptr;
    InstanceScalars* pinned = nullptr;
    const double** pointers = nullptr;   // device [2][kRhs]: the sub-steps' T0 and S
    std::vector<InstanceScalars> host;   // [kRhs] after a solve
    bool has64 = false, has32 = false;
    Space() = default;
    Space(const Space&) = delete;
    Space& operator=(const Space&) = delete;
    ~Space();
};

// The block solve of the interleaved system in space.bb (x0 in space.xr) with the batch's
// matrix and hierarchy (a one-planet batch); the right-hand sides' scalars land in
// space.host. BiCGSTAB only, plain Jacobi sweeps per the batch's smoother (block-local
// sweeps of a tuning are not applied).
void solve(Batch& b, Space& space, const SolveOptions& opt, cudaStream_t st);
// Lays out the workspace for `b` and the precision of `opt`.
void prepare(Batch& b, Space& space, const SolveOptions& opt);

}  // namespace mr
}  // namespace psgb

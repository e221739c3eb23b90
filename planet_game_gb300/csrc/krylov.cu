// Krylov kernels: BiCGSTAB and PCG vector updates with fused dot products, and the
// FP64 iterative-refinement residual/update.
//
// BiCGSTAB follows the reference's right-preconditioned variant
// (sim/planet/surface/heat_transport.cpp:823-897): x0 = 0, shadow = r0, breakdown on
// rho = 0, omega = 0 or shadow.v = 0, stop on ||s|| or ||r|| <= tol ||b||. PCG follows
// solve_newton_system (:394-429). Every scalar stays on the device: a kernel that
// produces dot products writes one partial per 256-row tile; the last tile of a planet
// to finish (integer ticket, so the order of arrival never matters) sums that planet's
// partials in tile order and performs the scalar step. Results are therefore
// bit-identical run to run and the same for a planet alone or inside a batch.
#include "common.cuh"
#include "kernels.hpp"
#include "krylov.hpp"
#include "phases.cuh"
#include "profile.hpp"

#include <cmath>
#include <stdexcept>

namespace psgb {
namespace {

// One 256-thread block per tile: the shared phases of phases.cuh.
//
// Reductions complete in a per-planet finish launch after each reducing phase (kDeferred).
// Completing them by ticket instead (the last tile set of a planet to write its partials
// sums them and performs the scalar step in the reducing launch) gives the same bits and
// one launch fewer per reduction, but measured on GB300 it nearly doubled the reducing
// kernels' time (BiCGSTAB products 10 -> 20 us on the 64-planet workload, 20 -> 32 us at
// L8): the fences and tickets of every tile set and the last tile set's sum sit on the
// kernel's critical path, where a separate small launch overlaps its start with the
// previous kernel's drain.
constexpr int kCompletion = ph::kDeferred;

template <typename T, int R>
__global__ void k_bicg_init(LevelView<T> lv, const T* __restrict__ b, T* x, T* r, T* shadow, T* p, T* v,
                            ReduceCtx ctx, double tol, int max_it) {
    ph::prefetch_meta(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    ph::bicg_init<T, R, kCompletion>(lv, blockIdx.x * R, 0, threadIdx.x, b, x, r, shadow, p, v, ctx, tol, max_it);
}

template <typename T, int R>
__global__ void k_bicg_p(LevelView<T> lv, const T* __restrict__ r, const T* __restrict__ v, T* p, T* xv, T omega_j,
                         const InstanceScalars* sc) {
    ph::prefetch_meta(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    ph::bicg_p<T, R>(lv, blockIdx.x * R, threadIdx.x, r, v, p, xv, omega_j, sc);
}

template <typename T, int W, int R>
__global__ void k_bicg_v(LevelView<T> lv, const T* __restrict__ in, T* __restrict__ out, const T* __restrict__ shadow,
                         ReduceCtx ctx) {
    ph::prefetch_static<T, W, R>(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    ph::bicg_v<T, W, R, kCompletion>(lv, blockIdx.x * R, 0, threadIdx.x, in, out, shadow, ctx);
}

template <typename T, int R>
__global__ void k_bicg_s(LevelView<T> lv, const T* __restrict__ r, const T* __restrict__ v, T* __restrict__ s_out,
                         T* xv, T omega_j, ReduceCtx ctx) {
    ph::prefetch_meta(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    ph::bicg_s<T, R, kCompletion>(lv, blockIdx.x * R, 0, threadIdx.x, r, v, s_out, xv, omega_j, ctx);
}

template <typename T, int W, int R>
__global__ void k_bicg_t(LevelView<T> lv, const T* __restrict__ shat, T* __restrict__ t, const T* __restrict__ s_vec,
                         ReduceCtx ctx) {
    ph::prefetch_static<T, W, R>(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    ph::bicg_t<T, W, R, kCompletion>(lv, blockIdx.x * R, 0, threadIdx.x, shat, t, s_vec, ctx);
}

template <typename T, int R>
__global__ void k_bicg_x(LevelView<T> lv, const T* __restrict__ phat, const T* __restrict__ shat,
                         const T* __restrict__ s_vec, const T* __restrict__ t, T* x, T* r,
                         const T* __restrict__ shadow, ReduceCtx ctx) {
    ph::prefetch_meta(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    ph::bicg_x<T, R, kCompletion>(lv, blockIdx.x * R, 0, threadIdx.x, phat, shat, s_vec, t, x, r, shadow, ctx);
}

template <typename T, int R>
__global__ void k_pcg_init(LevelView<T> lv, const T* __restrict__ b, T* x, T* r, T* p, T* xv, T omega_j,
                           ReduceCtx ctx, double tol, int max_it) {
    ph::prefetch_meta(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    ph::pcg_init<T, R, kCompletion>(lv, blockIdx.x * R, 0, threadIdx.x, b, x, r, p, xv, omega_j, ctx, tol, max_it);
}

template <typename T, int R>
__global__ void k_pcg_rz(LevelView<T> lv, const T* __restrict__ r, const T* __restrict__ z, ReduceCtx ctx) {
    ph::prefetch_meta(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    ph::pcg_rz<T, R, kCompletion>(lv, blockIdx.x * R, 0, threadIdx.x, r, z, ctx);
}

template <typename T, int R>
__global__ void k_pcg_p(LevelView<T> lv, const T* __restrict__ z, T* p, const InstanceScalars* sc) {
    ph::prefetch_meta(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    ph::pcg_p<T, R>(lv, blockIdx.x * R, threadIdx.x, z, p, sc);
}

template <typename T, int W, int R>
__global__ void k_pcg_q(LevelView<T> lv, const T* __restrict__ p, T* __restrict__ q_out, ReduceCtx ctx) {
    ph::prefetch_static<T, W, R>(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    ph::pcg_q<T, W, R, kCompletion>(lv, blockIdx.x * R, 0, threadIdx.x, p, q_out, ctx);
}

template <typename T, int R>
__global__ void k_pcg_xr(LevelView<T> lv, const T* __restrict__ p, const T* __restrict__ q_in, T* x, T* r, T* xv,
                         T omega_j, ReduceCtx ctx) {
    ph::prefetch_meta(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    ph::pcg_xr<T, R, kCompletion>(lv, blockIdx.x * R, 0, threadIdx.x, p, q_in, x, r, xv, omega_j, ctx);
}

template <int R>
__global__ void k_outer_init(LevelView<double> lv, const double* __restrict__ b, ReduceCtx ctx, double tol,
                             int max_refine, const std::uint8_t* __restrict__ active) {
    ph::prefetch_meta(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    static_cast<void>(max_refine);
    ph::outer_init<R, kCompletion>(lv, blockIdx.x * R, 0, threadIdx.x, b, ctx, tol, active);
}

template <typename TI, int W, int R>
__global__ void k_outer_residual(LevelView<double> lv, const double* __restrict__ b, const double* __restrict__ x,
                                 double* __restrict__ r64, TI* __restrict__ rin, ReduceCtx ctx, int max_refine) {
    ph::prefetch_static<double, W, R>(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    ph::outer_residual<TI, W, R, kCompletion>(lv, blockIdx.x * R, 0, threadIdx.x, b, x, r64, rin, ctx, max_refine);
}

template <typename TI, int R>
__global__ void k_outer_update(LevelView<double> lv, const TI* __restrict__ delta, double* x, InstanceScalars* sc) {
    ph::prefetch_meta(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    ph::outer_update<TI, R>(lv, blockIdx.x * R, threadIdx.x, delta, x, sc);
}

// The scalar step of a reduction phase, one planet per block (after the phase's launch).
template <int K>
__global__ void k_finish(ReduceCtx ctx, ph::FinishParams p) {
    const int inst = static_cast<int>(blockIdx.x);
    const unsigned begin = ctx.tile_begin[inst], end = ctx.tile_begin[inst + 1];   // fixed at build
    pdl_begin();
    ph::finish_planet<K>(ctx, inst, static_cast<int>(threadIdx.x), p, begin, end);
}

template <int K>
void launch_finish(int family, const ReduceCtx& ctx, cudaStream_t st, ph::FinishParams p = {}) {
    PSGB_LAUNCH(family, st, launch_pdl(k_finish<K>, ctx.instances, kTile, st, ctx, p));
}

__global__ void k_outer_account(InstanceScalars* sc, std::uint32_t instances) {
    pdl_begin();
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < instances) ph::outer_account(sc[i]);
}

}  // namespace

// ---- launchers -----------------------------------------------------------------------


template <typename T>
void KrylovLaunch<T>::bicg_init(const LevelView<T>& lv, const T* b, T* x, T* r, T* shadow, T* p, T* v,
                                const ReduceCtx& ctx, double tol, int max_it, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, PSGB_VECTOR_SETS(lv.sets_vector, launch_pdl(k_bicg_init<T, R>, ph::tile_sets(lv.tiles, R), kTile, st, counted(lv, kFamKrylovVector), b, x, r, shadow, p, v, ctx, tol, max_it)));
    if constexpr (kCompletion == ph::kDeferred) launch_finish<ph::kFinBicgInit>(kFamKrylovVector, ctx, st, ph::FinishParams{tol, max_it, 0, nullptr});
}
template <typename T>
void KrylovLaunch<T>::bicg_p(const LevelView<T>& lv, const T* r, const T* v, T* p, T* xv, T omega_j,
                             const InstanceScalars* sc, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, PSGB_VECTOR_SETS(lv.sets_vector, launch_pdl(k_bicg_p<T, R>, ph::tile_sets(lv.tiles, R), kTile, st, counted(lv, kFamKrylovVector), r, v, p, xv, omega_j, sc)));
}
template <typename T>
void KrylovLaunch<T>::bicg_v(const LevelView<T>& lv, const T* in, T* out, const T* shadow,
                             const ReduceCtx& ctx, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovSpmv, st, PSGB_WIDTHS(lv.width, PSGB_STENCIL_SETS(lv.sets_stencil, launch_pdl(k_bicg_v<T, W, R>, ph::tile_sets(lv.tiles, R), kTile, st, counted(lv, kFamKrylovSpmv), in, out, shadow, ctx))));
    if constexpr (kCompletion == ph::kDeferred) launch_finish<ph::kFinBicgV>(kFamKrylovSpmv, ctx, st);
}
template <typename T>
void KrylovLaunch<T>::bicg_s(const LevelView<T>& lv, const T* r, const T* v, T* s, T* xv, T omega_j,
                             const ReduceCtx& ctx, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, PSGB_VECTOR_SETS(lv.sets_vector, launch_pdl(k_bicg_s<T, R>, ph::tile_sets(lv.tiles, R), kTile, st, counted(lv, kFamKrylovVector), r, v, s, xv, omega_j, ctx)));
    if constexpr (kCompletion == ph::kDeferred) launch_finish<ph::kFinBicgS>(kFamKrylovVector, ctx, st);
}
template <typename T>
void KrylovLaunch<T>::bicg_t(const LevelView<T>& lv, const T* shat, T* t, const T* s,
                             const ReduceCtx& ctx, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovSpmv, st, PSGB_WIDTHS(lv.width, PSGB_STENCIL_SETS(lv.sets_stencil, launch_pdl(k_bicg_t<T, W, R>, ph::tile_sets(lv.tiles, R), kTile, st, counted(lv, kFamKrylovSpmv), shat, t, s, ctx))));
    if constexpr (kCompletion == ph::kDeferred) launch_finish<ph::kFinBicgT>(kFamKrylovSpmv, ctx, st);
}
template <typename T>
void KrylovLaunch<T>::bicg_x(const LevelView<T>& lv, const T* phat, const T* shat, const T* s,
                             const T* t, T* x, T* r, const T* shadow, const ReduceCtx& ctx,
                             cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, PSGB_VECTOR_SETS(lv.sets_vector, launch_pdl(k_bicg_x<T, R>, ph::tile_sets(lv.tiles, R), kTile, st, counted(lv, kFamKrylovVector), phat, shat, s, t, x, r, shadow, ctx)));
    if constexpr (kCompletion == ph::kDeferred) launch_finish<ph::kFinBicgX>(kFamKrylovVector, ctx, st);
}
template <typename T>
void KrylovLaunch<T>::pcg_init(const LevelView<T>& lv, const T* b, T* x, T* r, T* p, T* xv, T omega_j,
                               const ReduceCtx& ctx, double tol, int max_it, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, PSGB_VECTOR_SETS(lv.sets_vector, launch_pdl(k_pcg_init<T, R>, ph::tile_sets(lv.tiles, R), kTile, st, counted(lv, kFamKrylovVector), b, x, r, p, xv, omega_j, ctx, tol, max_it)));
    if constexpr (kCompletion == ph::kDeferred) launch_finish<ph::kFinPcgInit>(kFamKrylovVector, ctx, st, ph::FinishParams{tol, max_it, 0, nullptr});
}
template <typename T>
void KrylovLaunch<T>::pcg_rz(const LevelView<T>& lv, const T* r, const T* z, const ReduceCtx& ctx,
                             cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, PSGB_VECTOR_SETS(lv.sets_vector, launch_pdl(k_pcg_rz<T, R>, ph::tile_sets(lv.tiles, R), kTile, st, counted(lv, kFamKrylovVector), r, z, ctx)));
    if constexpr (kCompletion == ph::kDeferred) launch_finish<ph::kFinPcgRz>(kFamKrylovVector, ctx, st);
}
template <typename T>
void KrylovLaunch<T>::pcg_p(const LevelView<T>& lv, const T* z, T* p, const InstanceScalars* sc,
                            cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, PSGB_VECTOR_SETS(lv.sets_vector, launch_pdl(k_pcg_p<T, R>, ph::tile_sets(lv.tiles, R), kTile, st, counted(lv, kFamKrylovVector), z, p, sc)));
}
template <typename T>
void KrylovLaunch<T>::pcg_q(const LevelView<T>& lv, const T* p, T* q, const ReduceCtx& ctx,
                            cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovSpmv, st, PSGB_WIDTHS(lv.width, PSGB_STENCIL_SETS(lv.sets_stencil, launch_pdl(k_pcg_q<T, W, R>, ph::tile_sets(lv.tiles, R), kTile, st, counted(lv, kFamKrylovSpmv), p, q, ctx))));
    if constexpr (kCompletion == ph::kDeferred) launch_finish<ph::kFinPcgQ>(kFamKrylovSpmv, ctx, st);
}
template <typename T>
void KrylovLaunch<T>::pcg_xr(const LevelView<T>& lv, const T* p, const T* q, T* x, T* r, T* xv,
                             T omega_j, const ReduceCtx& ctx, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, PSGB_VECTOR_SETS(lv.sets_vector, launch_pdl(k_pcg_xr<T, R>, ph::tile_sets(lv.tiles, R), kTile, st, counted(lv, kFamKrylovVector), p, q, x, r, xv, omega_j, ctx)));
    if constexpr (kCompletion == ph::kDeferred) launch_finish<ph::kFinPcgXr>(kFamKrylovVector, ctx, st);
}

template struct KrylovLaunch<float>;
template struct KrylovLaunch<double>;

void launch_outer_init(const LevelView<double>& lv, const double* b, const ReduceCtx& ctx, double tol,
                       int max_refine, const std::uint8_t* active, cudaStream_t st) {
    PSGB_LAUNCH(kFamRefine, st, PSGB_VECTOR_SETS(lv.sets_vector, launch_pdl(k_outer_init<R>, ph::tile_sets(lv.tiles, R), kTile, st, counted(lv, kFamRefine), b, ctx, tol, max_refine, active)));
    if constexpr (kCompletion == ph::kDeferred) launch_finish<ph::kFinOuterInit>(kFamRefine, ctx, st, ph::FinishParams{tol, 0, max_refine, active});
}

template <typename TI>
void launch_outer_residual(const LevelView<double>& lv, const double* b, const double* x, double* r64,
                           TI* rin, const ReduceCtx& ctx, int max_refine, cudaStream_t st) {
    PSGB_LAUNCH(kFamRefine, st, PSGB_WIDTHS(lv.width, PSGB_STENCIL_SETS(lv.sets_stencil, launch_pdl(k_outer_residual<TI, W, R>, ph::tile_sets(lv.tiles, R), kTile, st, counted(lv, kFamRefine), b, x, r64, rin, ctx, max_refine))));
    if constexpr (kCompletion == ph::kDeferred) launch_finish<ph::kFinOuterResidual>(kFamRefine, ctx, st, ph::FinishParams{0.0, 0, max_refine, nullptr});
}

template <typename TI>
void launch_outer_update(const LevelView<double>& lv, const TI* delta, double* x, InstanceScalars* sc,
                         std::uint32_t instances, cudaStream_t st) {
    PSGB_LAUNCH(kFamRefine, st, launch_pdl(k_outer_account, (instances + 127) / 128, 128, st, sc, instances));
    PSGB_LAUNCH(kFamRefine, st, PSGB_VECTOR_SETS(lv.sets_vector, launch_pdl(k_outer_update<TI, R>, ph::tile_sets(lv.tiles, R), kTile, st, counted(lv, kFamRefine), delta, x, sc)));
}

template void launch_outer_residual<float>(const LevelView<double>&, const double*, const double*, double*,
                                           float*, const ReduceCtx&, int, cudaStream_t);
template void launch_outer_residual<double>(const LevelView<double>&, const double*, const double*, double*,
                                            double*, const ReduceCtx&, int, cudaStream_t);
template void launch_outer_update<float>(const LevelView<double>&, const float*, double*, InstanceScalars*,
                                         std::uint32_t, cudaStream_t);
template void launch_outer_update<double>(const LevelView<double>&, const double*, double*,
                                          InstanceScalars*, std::uint32_t, cudaStream_t);

}  // namespace psgb

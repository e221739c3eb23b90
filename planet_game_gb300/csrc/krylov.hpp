// Host launchers of the Krylov and FP64-refinement kernels (krylov.cu).
#pragma once

#include "kernels.hpp"

namespace psgb {

template <typename T>
struct KrylovLaunch {
    static void bicg_init(const LevelView<T>& lv, const T* b, T* x, T* r, T* shadow, T* p, T* v,
                          const ReduceCtx& ctx, double tol, int max_it, cudaStream_t st);
    static void bicg_p(const LevelView<T>& lv, const T* r, const T* v, T* p, T* xv, T omega_j,
                       const InstanceScalars* sc, cudaStream_t st);
    static void bicg_v(const LevelView<T>& lv, const T* in, T* out, const T* shadow,
                       const ReduceCtx& ctx, cudaStream_t st);
    static void bicg_s(const LevelView<T>& lv, const T* r, const T* v, T* s, T* xv, T omega_j,
                       const ReduceCtx& ctx, cudaStream_t st);
    static void bicg_t(const LevelView<T>& lv, const T* shat, T* t, const T* s, const ReduceCtx& ctx,
                       cudaStream_t st);
    static void bicg_x(const LevelView<T>& lv, const T* phat, const T* shat, const T* s, const T* t,
                       T* x, T* r, const T* shadow, const ReduceCtx& ctx, cudaStream_t st);
    static void pcg_init(const LevelView<T>& lv, const T* b, T* x, T* r, T* p, T* xv, T omega_j,
                         const ReduceCtx& ctx, double tol, int max_it, cudaStream_t st);
    static void pcg_rz(const LevelView<T>& lv, const T* r, const T* z, const ReduceCtx& ctx,
                       cudaStream_t st);
    static void pcg_p(const LevelView<T>& lv, const T* z, T* p, const InstanceScalars* sc,
                      cudaStream_t st);
    static void pcg_q(const LevelView<T>& lv, const T* p, T* q, const ReduceCtx& ctx, cudaStream_t st);
    static void pcg_xr(const LevelView<T>& lv, const T* p, const T* q, T* x, T* r, T* xv, T omega_j,
                       const ReduceCtx& ctx, cudaStream_t st);
};

// `active` (device, per planet, may be null): planets with 0 are skipped by the solve.
void launch_outer_init(const LevelView<double>& lv, const double* b, const ReduceCtx& ctx, double tol,
                       int max_refine, const std::uint8_t* active, cudaStream_t st);
template <typename TI>
void launch_outer_residual(const LevelView<double>& lv, const double* b, const double* x, double* r64,
                           TI* rin, const ReduceCtx& ctx, int max_refine, cudaStream_t st);
template <typename TI>
void launch_outer_update(const LevelView<double>& lv, const TI* delta, double* x, InstanceScalars* sc,
                         std::uint32_t instances, cudaStream_t st);

}  // namespace psgb

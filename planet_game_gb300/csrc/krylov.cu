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
#include "profile.hpp"
#include "kernels.hpp"
#include "krylov.hpp"

#include <cmath>
#include <stdexcept>

namespace psgb {
namespace {

template <typename T>
struct Fine {
    LevelView<T> lv;
};

__device__ __forceinline__ bool running(const InstanceScalars& s) { return s.status == kRunning; }

// Tile-level sum of NQ quantities, per-planet finalisation by the last tile.
// Inside a tile the sum runs in the kernel's precision A (FP32 kernels keep FP64 off the
// narrow FP64 pipe of GB300); tile partials and the per-planet sum are FP64.
// Returns true in thread 0 of the last tile, with `out` holding the planet's sums.
template <typename A, int NQ>
__device__ bool reduce_tiles(A (&v)[NQ], const ReduceCtx& ctx, int inst, double (&out)[NQ]) {
    __shared__ A tile_scratch[NQ][8];
    __shared__ double scratch[NQ][8];
    __shared__ bool last;
    const int tile = blockIdx.x;
    block_sum256<A, NQ>(v, tile_scratch);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) ctx.partial[tile * 8 + q] = static_cast<double>(v[q]);
        __threadfence();
        const unsigned begin = ctx.tile_begin[inst], end = ctx.tile_begin[inst + 1];
        const unsigned ticket = atomicAdd(&ctx.ticket[inst], 1u);
        last = (ticket == end - begin - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    const unsigned begin = ctx.tile_begin[inst], end = ctx.tile_begin[inst + 1];
    double acc[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] = 0.0;
    for (unsigned t = begin + threadIdx.x; t < end; t += kTile) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) acc[q] += __ldcg(&ctx.partial[t * 8 + q]);
    }
    __syncthreads();
    block_sum256<double, NQ>(acc, scratch);
    if (threadIdx.x == 0) {
        ctx.ticket[inst] = 0;
#pragma unroll
        for (int q = 0; q < NQ; ++q) out[q] = acc[q];
        return true;
    }
    return false;
}

// Common prologue: the row of this thread (or -1), the planet, and whether the
// planet takes part (uniform over the tile).
template <typename T>
__device__ __forceinline__ int tile_row(const LevelView<T>& lv, int& inst) {
    inst = lv.tile_inst[blockIdx.x];
    return threadIdx.x < lv.tile_rows[blockIdx.x] ? int(blockIdx.x) * kTile + int(threadIdx.x) : -1;
}

__device__ __forceinline__ bool finite(double v) { return isfinite(v); }

// ---- BiCGSTAB -------------------------------------------------------------------

template <typename T>
__global__ void k_bicg_init(LevelView<T> lv, const T* __restrict__ b, T* x, T* r, T* shadow, T* p,
                            T* v, ReduceCtx ctx, double tol, int max_it) {
    int inst;
    const int row = tile_row(lv, inst);
    if (ctx.sc[inst].outer_status != kRunning) return;
    T q[1] = {T(0)};
    if (row >= 0) {
        const T bv = b[row];
        x[row] = T(0); r[row] = bv; shadow[row] = bv; p[row] = T(0); v[row] = T(0);
        q[0] = bv * bv;
    }
    double out[1];
    if (reduce_tiles(q, ctx, inst, out)) {
        InstanceScalars& s = ctx.sc[inst];
        s.b_norm = sqrt(out[0]);
        s.target = fmax(tol * s.b_norm, 0.5 * s.outer_target);
        s.rho = out[0]; s.alpha = 1.0; s.omega = 1.0; s.beta = 0.0;
        s.iterations = 0; s.half_done = 0; s.max_iterations = max_it; s.first = 1;
        s.r_norm = s.b_norm;
        s.status = !finite(s.b_norm) ? kNonFinite : (s.b_norm > 0.0 ? kRunning : kConverged);
    }
}

// p = r + beta (p - omega v); first smoothing sweep of M p from zero.
template <typename T>
__global__ void k_bicg_p(LevelView<T> lv, const T* __restrict__ r, const T* __restrict__ v, T* p,
                         T* xv, T omega_j, const InstanceScalars* sc) {
    int inst;
    const int row = tile_row(lv, inst);
    if (row < 0 || !running(sc[inst])) return;
    const T beta = T(sc[inst].beta), omega = T(sc[inst].omega);
    const T pv = r[row] + beta * (p[row] - omega * v[row]);
    p[row] = pv;
    if (lv.tile_sweep[blockIdx.x]) xv[row] = omega_j * lv.inv[row] * pv;
}

// out = A in; dot(shadow, out) -> alpha = rho / (shadow . v)
template <typename T, int W>
__global__ void k_bicg_v(LevelView<T> lv, const T* __restrict__ in, T* __restrict__ out,
                         const T* __restrict__ shadow, ReduceCtx ctx) {
    int inst;
    const int row = tile_row(lv, inst);
    if (!running(ctx.sc[inst])) return;
    T q[1] = {T(0)};
    if (row >= 0) {
        const std::uint32_t P = lv.rows;
        T s = lv.vd[W * P + row] * in[row];
#pragma unroll
        for (int j = 0; j < W; ++j) s += lv.vd[j * P + row] * in[lv.col[j * P + row]];
        out[row] = s;
        q[0] = shadow[row] * s;
    }
    double sum[1];
    if (reduce_tiles(q, ctx, inst, sum)) {
        InstanceScalars& s = ctx.sc[inst];
        if (!finite(sum[0])) { s.status = kNonFinite; return; }
        if (sum[0] == 0.0) { s.status = kBreakdown; return; }
        s.alpha = s.rho / sum[0];
    }
}

// s = r - alpha v; ||s||: converged at s -> finish with x += alpha p_hat.
template <typename T>
__global__ void k_bicg_s(LevelView<T> lv, const T* __restrict__ r, const T* __restrict__ v,
                         T* __restrict__ s_out, T* xv, T omega_j, ReduceCtx ctx) {
    int inst;
    const int row = tile_row(lv, inst);
    if (!running(ctx.sc[inst])) return;
    T q[1] = {T(0)};
    const T alpha = T(ctx.sc[inst].alpha);
    if (row >= 0) {
        const T sv = r[row] - alpha * v[row];
        s_out[row] = sv;
        q[0] = sv * sv;
        if (lv.tile_sweep[blockIdx.x]) xv[row] = omega_j * lv.inv[row] * sv;
    }
    double sum[1];
    if (reduce_tiles(q, ctx, inst, sum)) {
        InstanceScalars& s = ctx.sc[inst];
        s.s_norm = sqrt(sum[0]);
        s.iterations += 1;
        if (!finite(s.s_norm)) { s.status = kNonFinite; return; }
        if (s.s_norm <= s.target) s.half_done = 1;
    }
}

// t = A s_hat; (t.t, t.s) -> omega
template <typename T, int W>
__global__ void k_bicg_t(LevelView<T> lv, const T* __restrict__ shat, T* __restrict__ t,
                         const T* __restrict__ s_vec, ReduceCtx ctx) {
    int inst;
    const int row = tile_row(lv, inst);
    const InstanceScalars& sc = ctx.sc[inst];
    if (!running(sc) || sc.half_done) return;
    T q[2] = {T(0), T(0)};
    if (row >= 0) {
        const std::uint32_t P = lv.rows;
        T s = lv.vd[W * P + row] * shat[row];
#pragma unroll
        for (int j = 0; j < W; ++j) s += lv.vd[j * P + row] * shat[lv.col[j * P + row]];
        t[row] = s;
        q[0] = s * s;
        q[1] = s * s_vec[row];
    }
    double sum[2];
    if (reduce_tiles(q, ctx, inst, sum)) {
        InstanceScalars& s = ctx.sc[inst];
        s.omega = sum[0] > 0.0 ? sum[1] / sum[0] : 0.0;
        if (!finite(s.omega)) s.status = kNonFinite;
    }
}

// x += alpha p_hat + omega s_hat; r = s - omega t; (r.r, shadow.r) -> next rho/beta.
template <typename T>
__global__ void k_bicg_x(LevelView<T> lv, const T* __restrict__ phat, const T* __restrict__ shat,
                         const T* __restrict__ s_vec, const T* __restrict__ t, T* x, T* r,
                         const T* __restrict__ shadow, ReduceCtx ctx) {
    int inst;
    const int row = tile_row(lv, inst);
    const InstanceScalars& sc = ctx.sc[inst];
    if (!running(sc)) return;
    const T alpha = T(sc.alpha), omega = T(sc.omega);
    if (sc.half_done) {
        // uniform over the planet: finish at s without a reduction
        if (row >= 0) x[row] += alpha * phat[row];
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            const unsigned begin = ctx.tile_begin[inst], end = ctx.tile_begin[inst + 1];
            const unsigned ticket = atomicAdd(&ctx.ticket[inst], 1u);
            if (ticket == end - begin - 1) {
                ctx.ticket[inst] = 0;
                InstanceScalars& s = ctx.sc[inst];
                s.r_norm = s.s_norm;
                s.half_done = 0;
                s.status = kConverged;
            }
        }
        return;
    }
    T q[2] = {T(0), T(0)};
    if (row >= 0) {
        x[row] += alpha * phat[row] + omega * shat[row];
        const T rv = s_vec[row] - omega * t[row];
        r[row] = rv;
        q[0] = rv * rv;
        q[1] = shadow[row] * rv;
    }
    double sum[2];
    if (reduce_tiles(q, ctx, inst, sum)) {
        InstanceScalars& s = ctx.sc[inst];
        s.r_norm = sqrt(sum[0]);
        if (!finite(s.r_norm)) { s.status = kNonFinite; return; }
        if (s.r_norm <= s.target) { s.status = kConverged; return; }
        const double rho_next = sum[1];
        if (rho_next == 0.0 || s.omega == 0.0) { s.status = kBreakdown; return; }
        s.beta = rho_next / s.rho * (s.alpha / s.omega);
        s.rho = rho_next;
        if (s.iterations >= s.max_iterations) s.status = kCap;
    }
}

// ---- PCG ---------------------------------------------------------------------------

template <typename T>
__global__ void k_pcg_init(LevelView<T> lv, const T* __restrict__ b, T* x, T* r, T* p, T* xv,
                           T omega_j, ReduceCtx ctx, double tol, int max_it) {
    int inst;
    const int row = tile_row(lv, inst);
    if (ctx.sc[inst].outer_status != kRunning) return;
    T q[1] = {T(0)};
    if (row >= 0) {
        const T bv = b[row];
        x[row] = T(0); r[row] = bv; p[row] = T(0);
        if (lv.tile_sweep[blockIdx.x]) xv[row] = omega_j * lv.inv[row] * bv;
        q[0] = bv * bv;
    }
    double out[1];
    if (reduce_tiles(q, ctx, inst, out)) {
        InstanceScalars& s = ctx.sc[inst];
        s.b_norm = sqrt(out[0]);
        s.target = fmax(tol * s.b_norm, 0.5 * s.outer_target);
        s.r_norm = s.b_norm;
        s.iterations = 0; s.half_done = 0; s.max_iterations = max_it; s.first = 1;
        s.rho = 0.0; s.beta = 0.0; s.alpha = 0.0;
        s.status = !finite(s.b_norm) ? kNonFinite : (s.b_norm > 0.0 ? kRunning : kConverged);
    }
}

// rho = r.z, beta = rho / rho_old; p = z + beta p happens in k_pcg_pq.
template <typename T>
__global__ void k_pcg_rz(LevelView<T> lv, const T* __restrict__ r, const T* __restrict__ z,
                         ReduceCtx ctx) {
    int inst;
    const int row = tile_row(lv, inst);
    if (!running(ctx.sc[inst])) return;
    T q[1] = {T(0)};
    if (row >= 0) q[0] = r[row] * z[row];
    double sum[1];
    if (reduce_tiles(q, ctx, inst, sum)) {
        InstanceScalars& s = ctx.sc[inst];
        if (!finite(sum[0])) { s.status = kNonFinite; return; }
        if (!(sum[0] > 0.0)) { s.status = s.first ? kConverged : kBreakdown; return; }
        s.beta = s.first ? 0.0 : sum[0] / s.rho;
        s.rho = sum[0];
        s.first = 0;
    }
}

// p = z + beta p (written by the tile before the product reads it: separate kernel)
template <typename T>
__global__ void k_pcg_p(LevelView<T> lv, const T* __restrict__ z, T* p, const InstanceScalars* sc) {
    int inst;
    const int row = tile_row(lv, inst);
    if (row < 0 || !running(sc[inst])) return;
    p[row] = z[row] + T(sc[inst].beta) * p[row];
}

// q = A p; alpha = rho / p.q
template <typename T, int W>
__global__ void k_pcg_q(LevelView<T> lv, const T* __restrict__ p, T* __restrict__ q_out, ReduceCtx ctx) {
    int inst;
    const int row = tile_row(lv, inst);
    if (!running(ctx.sc[inst])) return;
    T q[1] = {T(0)};
    if (row >= 0) {
        const std::uint32_t P = lv.rows;
        T s = lv.vd[W * P + row] * p[row];
#pragma unroll
        for (int j = 0; j < W; ++j) s += lv.vd[j * P + row] * p[lv.col[j * P + row]];
        q_out[row] = s;
        q[0] = p[row] * s;
    }
    double sum[1];
    if (reduce_tiles(q, ctx, inst, sum)) {
        InstanceScalars& s = ctx.sc[inst];
        if (!finite(sum[0])) { s.status = kNonFinite; return; }
        if (!(sum[0] > 0.0)) { s.status = kBreakdown; return; }
        s.alpha = s.rho / sum[0];
    }
}

// x += alpha p; r -= alpha q; ||r|| -> converged?; first sweep of M r.
template <typename T>
__global__ void k_pcg_xr(LevelView<T> lv, const T* __restrict__ p, const T* __restrict__ q_in, T* x,
                         T* r, T* xv, T omega_j, ReduceCtx ctx) {
    int inst;
    const int row = tile_row(lv, inst);
    if (!running(ctx.sc[inst])) return;
    const T alpha = T(ctx.sc[inst].alpha);
    T q[1] = {T(0)};
    if (row >= 0) {
        x[row] += alpha * p[row];
        const T rv = r[row] - alpha * q_in[row];
        r[row] = rv;
        q[0] = rv * rv;
        if (lv.tile_sweep[blockIdx.x]) xv[row] = omega_j * lv.inv[row] * rv;
    }
    double sum[1];
    if (reduce_tiles(q, ctx, inst, sum)) {
        InstanceScalars& s = ctx.sc[inst];
        s.r_norm = sqrt(sum[0]);
        s.iterations += 1;
        if (!finite(s.r_norm)) { s.status = kNonFinite; return; }
        if (s.r_norm <= s.target) { s.status = kConverged; return; }
        if (s.iterations >= s.max_iterations) s.status = kCap;
    }
}

// ---- FP64 refinement -------------------------------------------------------------

// ||b|| of the outer problem, and the outer state reset.
__global__ void k_outer_init(LevelView<double> lv, const double* __restrict__ b, ReduceCtx ctx,
                             double tol, int max_refine, const std::uint8_t* __restrict__ active) {
    int inst;
    const int row = tile_row(lv, inst);
    if (active != nullptr && !active[inst]) {
        // a planet left out of this step: nothing runs for it
        if (threadIdx.x == 0 && blockIdx.x == ctx.tile_begin[inst]) {
            InstanceScalars& s = ctx.sc[inst];
            s.outer_status = kConverged;
            s.status = kConverged;
            s.refinements = 0;
            s.inner_total = 0;
            s.outer_r_norm = 0.0;
            s.outer_b_norm = 0.0;
        }
        return;
    }
    double q[1] = {0.0};
    if (row >= 0) q[0] = dmul(b[row], b[row]);
    double sum[1];
    if (reduce_tiles(q, ctx, inst, sum)) {
        InstanceScalars& s = ctx.sc[inst];
        s.outer_b_norm = sqrt(sum[0]);
        s.outer_target = tol * s.outer_b_norm;
        s.tolerance = tol;
        s.refinements = 0;
        s.inner_total = 0;
        s.outer_status = !finite(s.outer_b_norm) ? kNonFinite : kRunning;
        s.status = kConverged;   // no inner solve runs until an inner init starts one
    }
}

// r = b - A x in FP64 (FP64 matrix), cast to the inner precision; ||r|| decides.
template <typename TI, int W>
__global__ void k_outer_residual(LevelView<double> lv, const double* __restrict__ b,
                                 const double* __restrict__ x, double* __restrict__ r64,
                                 TI* __restrict__ rin, ReduceCtx ctx, int max_refine) {
    int inst;
    const int row = tile_row(lv, inst);
    if (ctx.sc[inst].outer_status != kRunning) return;
    double q[1] = {0.0};
    if (row >= 0) {
        const std::uint32_t P = lv.rows;
        double s = b[row] - lv.vd[W * P + row] * x[row];
#pragma unroll
        for (int j = 0; j < W; ++j) s -= lv.vd[j * P + row] * x[lv.col[j * P + row]];
        r64[row] = s;
        rin[row] = static_cast<TI>(s);
        q[0] = s * s;
    }
    double sum[1];
    if (reduce_tiles(q, ctx, inst, sum)) {
        InstanceScalars& s = ctx.sc[inst];
        s.outer_r_norm = sqrt(sum[0]);
        if (!finite(s.outer_r_norm)) { s.outer_status = kNonFinite; return; }
        if (s.outer_r_norm <= s.outer_target || s.outer_b_norm == 0.0) {
            s.outer_status = kConverged;
            s.status = kConverged;
            return;
        }
        if (s.refinements >= max_refine) { s.outer_status = kCap; s.status = kConverged; return; }
        s.refinements += 1;
    }
}

// x += delta (inner solution), for planets still refining.
template <typename TI>
__global__ void k_outer_update(LevelView<double> lv, const TI* __restrict__ delta, double* x,
                               InstanceScalars* sc) {
    int inst;
    const int row = tile_row(lv, inst);
    if (sc[inst].outer_status != kRunning) return;
    if (row >= 0) x[row] += static_cast<double>(delta[row]);
}

__global__ void k_outer_account(InstanceScalars* sc, std::uint32_t instances) {
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= instances) return;
    InstanceScalars& s = sc[i];
    if (s.outer_status != kRunning) return;
    s.inner_total += s.iterations;
    if (s.status == kNonFinite) s.outer_status = kNonFinite;
}

}  // namespace

// ---- launchers -----------------------------------------------------------------------

#define PSGB_W(width, ...)                                            \
    switch (width) {                                                  \
        case 6: { constexpr int W = 6; __VA_ARGS__; } break;           \
        case 8: { constexpr int W = 8; __VA_ARGS__; } break;           \
        case 12: { constexpr int W = 12; __VA_ARGS__; } break;         \
        case 16: { constexpr int W = 16; __VA_ARGS__; } break;         \
        default: throw std::logic_error("unsupported ELL width");     \
    }

template <typename T>
void KrylovLaunch<T>::bicg_init(const LevelView<T>& lv, const T* b, T* x, T* r, T* shadow, T* p, T* v,
                                const ReduceCtx& ctx, double tol, int max_it, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, k_bicg_init<T><<<lv.tiles, kTile, 0, st>>>(lv, b, x, r, shadow, p, v, ctx, tol, max_it));
}
template <typename T>
void KrylovLaunch<T>::bicg_p(const LevelView<T>& lv, const T* r, const T* v, T* p, T* xv, T omega_j,
                             const InstanceScalars* sc, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, k_bicg_p<T><<<lv.tiles, kTile, 0, st>>>(lv, r, v, p, xv, omega_j, sc));
}
template <typename T>
void KrylovLaunch<T>::bicg_v(const LevelView<T>& lv, const T* in, T* out, const T* shadow,
                             const ReduceCtx& ctx, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovSpmv, st, PSGB_W(lv.width, (k_bicg_v<T, W><<<lv.tiles, kTile, 0, st>>>(lv, in, out, shadow, ctx))));
}
template <typename T>
void KrylovLaunch<T>::bicg_s(const LevelView<T>& lv, const T* r, const T* v, T* s, T* xv, T omega_j,
                             const ReduceCtx& ctx, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, k_bicg_s<T><<<lv.tiles, kTile, 0, st>>>(lv, r, v, s, xv, omega_j, ctx));
}
template <typename T>
void KrylovLaunch<T>::bicg_t(const LevelView<T>& lv, const T* shat, T* t, const T* s,
                             const ReduceCtx& ctx, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovSpmv, st, PSGB_W(lv.width, (k_bicg_t<T, W><<<lv.tiles, kTile, 0, st>>>(lv, shat, t, s, ctx))));
}
template <typename T>
void KrylovLaunch<T>::bicg_x(const LevelView<T>& lv, const T* phat, const T* shat, const T* s,
                             const T* t, T* x, T* r, const T* shadow, const ReduceCtx& ctx,
                             cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, k_bicg_x<T><<<lv.tiles, kTile, 0, st>>>(lv, phat, shat, s, t, x, r, shadow, ctx));
}
template <typename T>
void KrylovLaunch<T>::pcg_init(const LevelView<T>& lv, const T* b, T* x, T* r, T* p, T* xv, T omega_j,
                               const ReduceCtx& ctx, double tol, int max_it, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, k_pcg_init<T><<<lv.tiles, kTile, 0, st>>>(lv, b, x, r, p, xv, omega_j, ctx, tol, max_it));
}
template <typename T>
void KrylovLaunch<T>::pcg_rz(const LevelView<T>& lv, const T* r, const T* z, const ReduceCtx& ctx,
                             cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, k_pcg_rz<T><<<lv.tiles, kTile, 0, st>>>(lv, r, z, ctx));
}
template <typename T>
void KrylovLaunch<T>::pcg_p(const LevelView<T>& lv, const T* z, T* p, const InstanceScalars* sc,
                            cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, k_pcg_p<T><<<lv.tiles, kTile, 0, st>>>(lv, z, p, sc));
}
template <typename T>
void KrylovLaunch<T>::pcg_q(const LevelView<T>& lv, const T* p, T* q, const ReduceCtx& ctx,
                            cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovSpmv, st, PSGB_W(lv.width, (k_pcg_q<T, W><<<lv.tiles, kTile, 0, st>>>(lv, p, q, ctx))));
}
template <typename T>
void KrylovLaunch<T>::pcg_xr(const LevelView<T>& lv, const T* p, const T* q, T* x, T* r, T* xv,
                             T omega_j, const ReduceCtx& ctx, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, k_pcg_xr<T><<<lv.tiles, kTile, 0, st>>>(lv, p, q, x, r, xv, omega_j, ctx));
}

template struct KrylovLaunch<float>;
template struct KrylovLaunch<double>;

void launch_outer_init(const LevelView<double>& lv, const double* b, const ReduceCtx& ctx, double tol,
                       int max_refine, const std::uint8_t* active, cudaStream_t st) {
    PSGB_LAUNCH(kFamRefine, st, k_outer_init<<<lv.tiles, kTile, 0, st>>>(lv, b, ctx, tol, max_refine, active));
}

template <typename TI>
void launch_outer_residual(const LevelView<double>& lv, const double* b, const double* x, double* r64,
                           TI* rin, const ReduceCtx& ctx, int max_refine, cudaStream_t st) {
    PSGB_LAUNCH(kFamRefine, st, PSGB_W(lv.width, (k_outer_residual<TI, W><<<lv.tiles, kTile, 0, st>>>(lv, b, x, r64, rin, ctx, max_refine))));
}

template <typename TI>
void launch_outer_update(const LevelView<double>& lv, const TI* delta, double* x, InstanceScalars* sc,
                         std::uint32_t instances, cudaStream_t st) {
    PSGB_LAUNCH(kFamRefine, st, k_outer_account<<<(instances + 127) / 128, 128, 0, st>>>(sc, instances));
    PSGB_LAUNCH(kFamRefine, st, k_outer_update<TI><<<lv.tiles, kTile, 0, st>>>(lv, delta, x, sc));
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

// Per-tile phases of the solve, shared by the one-kernel-per-phase path (multigrid.cu,
// krylov.cu) and the persistent solver (persistent.cu), so both compute every row and
// every reduction with the same arithmetic in the same order.
//
// A "group" is 256 consecutive threads of a block working on one 256-row tile (a block
// of 256 threads is one group; the persistent kernel runs 1024-thread blocks = 4 groups).
// Groups synchronise with named barriers (id 1 + group), never with __syncthreads, so the
// groups of a block can work on different tiles independently.
#pragma once

#include "common.cuh"
#include "kernels.hpp"

// Vectors a phase reads were written by an earlier phase. A kernel per phase may read
// them through the read-only (non-coherent) path; the persistent solver, where earlier
// phases ran in the same kernel, must not: it defines PSGB_PHASE_RESTRICT empty.
#ifndef PSGB_PHASE_RESTRICT
#define PSGB_PHASE_RESTRICT __restrict__
#endif

namespace psgb {
namespace ph {

constexpr int kGroups = 4;   // groups per block at most (1024 threads)

__device__ __forceinline__ void group_sync(int gid) {
    asm volatile("bar.sync %0, 256;" ::"r"(gid + 1) : "memory");
}

__device__ __forceinline__ void count_bytes(unsigned long long* counter, int lane, unsigned long long bytes) {
    if (counter != nullptr && lane == 0 && bytes != 0) atomicAdd(counter, bytes);
}

// Sum of NQ values over the 256 threads of a group, in a fixed tree; result in lane 0.
template <typename A, int NQ>
__device__ __forceinline__ void group_sum(A (&v)[NQ], int gid, int lane) {
    __shared__ A scratch[kGroups][NQ][8];
    const int w = lane >> 5;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        const A s = warp_sum(v[q]);
        if ((lane & 31) == 0) scratch[gid][q][w] = s;
    }
    group_sync(gid);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            A s = scratch[gid][q][0];
#pragma unroll
            for (int k = 1; k < 8; ++k) s += scratch[gid][q][k];
            v[q] = s;
        }
    }
    group_sync(gid);
}

// Tile partial sums (in the tile's precision A) to FP64 partials; the last tile of a
// planet to arrive (integer ticket) sums that planet's partials in tile order. Returns
// true in lane 0 of the group that finalises, with the planet's sums in `out`.
template <typename A, int NQ>
__device__ bool tile_reduce(A (&v)[NQ], const ReduceCtx& ctx, int inst, int tile, double (&out)[NQ], int gid,
                            int lane) {
    __shared__ int last[kGroups];
    group_sum<A, NQ>(v, gid, lane);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) ctx.partial[tile * 8 + q] = static_cast<double>(v[q]);
        __threadfence();
        const unsigned begin = ctx.tile_begin[inst], end = ctx.tile_begin[inst + 1];
        const unsigned ticket = atomicAdd(&ctx.ticket[inst], 1u);
        last[gid] = (ticket == end - begin - 1) ? 1 : 0;
    }
    group_sync(gid);
    if (!last[gid]) return false;
    __threadfence();
    const unsigned begin = ctx.tile_begin[inst], end = ctx.tile_begin[inst + 1];
    double acc[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] = 0.0;
    for (unsigned t = begin + lane; t < end; t += kTile) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) acc[q] += __ldcg(&ctx.partial[t * 8 + q]);
    }
    group_sum<double, NQ>(acc, gid, lane);
    if (lane == 0) {
        ctx.ticket[inst] = 0;
#pragma unroll
        for (int q = 0; q < NQ; ++q) out[q] = acc[q];
        return true;
    }
    return false;
}

__device__ __forceinline__ bool gate_open(const InstanceScalars* sc, int inst, int gate) {
    if (gate == kGateAlways) return true;
    const InstanceScalars& s = sc[inst];
    if (gate == kGateOuter) return s.outer_status == kRunning;
    if (s.status != kRunning) return false;
    if (gate == kGateSecondHalf && s.half_done) return false;
    return true;
}

__device__ __forceinline__ bool finite(double v) { return isfinite(v); }

// ---- V-cycle phases ---------------------------------------------------------------------

// Sum of r over an aggregate's members, in ascending member order (the reference's
// order). The gathers are issued eight at a time so that they are in flight together;
// the additions stay sequential, so the sum is the same as the plain loop's.
template <typename T>
__device__ __forceinline__ T member_sum(const std::uint32_t* PSGB_PHASE_RESTRICT member, std::uint32_t k0,
                                        std::uint32_t k1, const T* PSGB_PHASE_RESTRICT r) {
    T s = T(0);
    for (std::uint32_t k = k0; k < k1; k += 8) {
        T v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = (k + j < k1) ? r[member[k + j]] : T(0);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (k + j < k1) s += v[j];
        }
    }
    return s;
}

template <typename T>
__device__ void smooth_zero(const LevelView<T>& lv, int tile, int lane, const T* PSGB_PHASE_RESTRICT b, T* PSGB_PHASE_RESTRICT x,
                            T omega, const InstanceScalars* sc, int gate) {
    const int rows = lv.tile_rows[tile];
    if (!lv.tile_sweep[tile] || !gate_open(sc, lv.tile_inst[tile], gate)) return;
    count_bytes(lv.bytes, lane, static_cast<unsigned long long>(rows) * 3ull * sizeof(T));
    if (lane >= rows) return;
    const int row = tile * kTile + lane;
    x[row] = omega * lv.inv[row] * b[row];
}

template <typename T, int W>
__device__ void smooth(const LevelView<T>& lv, int tile, int lane, const T* PSGB_PHASE_RESTRICT b, const T* PSGB_PHASE_RESTRICT x,
                       T* PSGB_PHASE_RESTRICT y, T omega, const InstanceScalars* sc, int gate) {
    const int rows = lv.tile_rows[tile];
    if (!lv.tile_sweep[tile] || !gate_open(sc, lv.tile_inst[tile], gate)) return;
    count_bytes(lv.bytes, lane, static_cast<unsigned long long>(rows) * (4ull * W + sizeof(T) * (W + 4ull)));
    if (lane >= rows) return;
    const int row = tile * kTile + lane;
    const std::uint32_t P = lv.rows;
    T s = b[row];
#pragma unroll
    for (int j = 0; j < W; ++j) s -= lv.vd[j * P + row] * x[lv.col[j * P + row]];
    const T xo = x[row];
    y[row] = xo + omega * (lv.inv[row] * s - xo);
}

template <typename T, int W>
__device__ void residual(const LevelView<T>& lv, int tile, int lane, const T* PSGB_PHASE_RESTRICT b, const T* PSGB_PHASE_RESTRICT x,
                         T* PSGB_PHASE_RESTRICT r, const InstanceScalars* sc, int gate) {
    const int rows = lv.tile_rows[tile];
    if (!lv.tile_sweep[tile] || !gate_open(sc, lv.tile_inst[tile], gate)) return;
    if (lane >= rows) return;
    const int row = tile * kTile + lane;
    const std::uint32_t P = lv.rows;
    T s = b[row] - lv.vd[W * P + row] * x[row];
#pragma unroll
    for (int j = 0; j < W; ++j) s -= lv.vd[j * P + row] * x[lv.col[j * P + row]];
    r[row] = s;
}

template <typename T, int W>
__device__ void spmv(const LevelView<T>& lv, int tile, int lane, const T* PSGB_PHASE_RESTRICT x, T* PSGB_PHASE_RESTRICT y) {
    if (lane >= lv.tile_rows[tile]) return;
    const int row = tile * kTile + lane;
    const std::uint32_t P = lv.rows;
    T s = lv.vd[W * P + row] * x[row];
#pragma unroll
    for (int j = 0; j < W; ++j) s += lv.vd[j * P + row] * x[lv.col[j * P + row]];
    y[row] = s;
}

// Restriction fused with the coarse level's zero-start sweep: b_c = sum of the members'
// residuals in ascending fine-row order (the reference's order, heat_transport.cpp:316-319);
// x_c = omega b_c / diag where the planet smooths on the coarse level.
template <typename T>
__device__ void restrict_zero(const LevelView<T>& coarse, int tile, int lane, const std::uint32_t* PSGB_PHASE_RESTRICT moff,
                              const std::uint32_t* PSGB_PHASE_RESTRICT member, const T* PSGB_PHASE_RESTRICT r, T* PSGB_PHASE_RESTRICT bc,
                              T* PSGB_PHASE_RESTRICT xc, T omega, const InstanceScalars* sc, int gate) {
    const int rows = coarse.tile_rows[tile];
    if (!gate_open(sc, coarse.tile_inst[tile], gate)) return;
    if (lane >= rows) return;
    const int row = tile * kTile + lane;
    const T s = member_sum(member, moff[row], moff[row + 1], r);
    bc[row] = s;
    if (coarse.tile_sweep[tile]) xc[row] = omega * coarse.inv[row] * s;
}

template <typename T>
__device__ void restrict_only(const LevelView<T>& coarse, int tile, int lane, const std::uint32_t* PSGB_PHASE_RESTRICT moff,
                              const std::uint32_t* PSGB_PHASE_RESTRICT member, const T* PSGB_PHASE_RESTRICT r, T* PSGB_PHASE_RESTRICT bc,
                              const InstanceScalars* sc, int gate) {
    if (lane >= coarse.tile_rows[tile]) return;
    if (!gate_open(sc, coarse.tile_inst[tile], gate)) return;
    const int row = tile * kTile + lane;
    bc[row] = member_sum(member, moff[row], moff[row + 1], r);
}

// Prolongation fused with the first post-smoothing sweep: with x' = x + e[agg] (formed on
// the fly for the row and its neighbours), y = x' + omega (D^-1 (b - O x') - x').
template <typename T, int W>
__device__ void prolong_smooth(const LevelView<T>& lv, int tile, int lane, const std::int32_t* PSGB_PHASE_RESTRICT agg,
                               const T* PSGB_PHASE_RESTRICT e, const T* PSGB_PHASE_RESTRICT b, const T* PSGB_PHASE_RESTRICT x,
                               T* PSGB_PHASE_RESTRICT y, T omega, const InstanceScalars* sc, int gate) {
    const int rows = lv.tile_rows[tile];
    if (!lv.tile_sweep[tile] || !gate_open(sc, lv.tile_inst[tile], gate)) return;
    count_bytes(lv.bytes, lane, static_cast<unsigned long long>(rows) * (8ull * W + sizeof(T) * (W + 4ull) + 4ull));
    if (lane >= rows) return;
    const int row = tile * kTile + lane;
    const std::uint32_t P = lv.rows;
    T s = b[row];
#pragma unroll
    for (int j = 0; j < W; ++j) {
        const int c = lv.col[j * P + row];
        s -= lv.vd[j * P + row] * (x[c] + e[agg[c]]);
    }
    const T xo = x[row] + e[agg[row]];
    y[row] = xo + omega * (lv.inv[row] * s - xo);
}

template <typename T>
__device__ void prolong(const LevelView<T>& lv, int tile, int lane, const std::int32_t* PSGB_PHASE_RESTRICT agg,
                        const T* PSGB_PHASE_RESTRICT xc, T* PSGB_PHASE_RESTRICT x, const InstanceScalars* sc, int gate) {
    if (lane >= lv.tile_rows[tile]) return;
    if (!lv.tile_sweep[tile] || !gate_open(sc, lv.tile_inst[tile], gate)) return;
    const int row = tile * kTile + lane;
    x[row] += xc[agg[row]];
}

// Coarsest level: x = A^-1 b for one row of one planet, one warp per row.
template <typename T>
__device__ void dense_row(const DenseView& dense, int inst, int rowi, int lane32, const T* PSGB_PHASE_RESTRICT inv,
                          const T* PSGB_PHASE_RESTRICT b, T* PSGB_PHASE_RESTRICT x) {
    const int n = static_cast<int>(dense.size[inst]);
    const std::int64_t base = dense.row_base[inst];
    const T* a = inv + dense.offset[inst] + static_cast<std::int64_t>(rowi) * n;
    T s = T(0);
    for (int j = lane32; j < n; j += 32) s += a[j] * b[base + j];
    s = warp_sum(s);
    if (lane32 == 0) x[base + rowi] = s;
}

// Block k of a dense task: eight rows of one planet, one warp per row (256 threads).
template <typename T>
__device__ void dense_block(const DenseTask<T>& task, unsigned k, int lane, const InstanceScalars* sc, int gate) {
    const int2 blk = task.blocks[k];
    if (!gate_open(sc, blk.x, gate)) return;
    const int row = blk.y + (lane >> 5);
    if (row >= static_cast<int>(task.dense.size[blk.x])) return;
    dense_row<T>(task.dense, blk.x, row, lane & 31, task.inv, task.b, task.x);
}

// ---- Krylov phases (fine level) ----------------------------------------------------------

__device__ __forceinline__ bool running(const InstanceScalars& s) { return s.status == kRunning; }

template <typename T>
__device__ void bicg_init(const LevelView<T>& lv, int tile, int gid, int lane, const T* PSGB_PHASE_RESTRICT b, T* x, T* r,
                          T* shadow, T* p, T* v, const ReduceCtx& ctx, double tol, int max_it) {
    const int inst = lv.tile_inst[tile];
    if (ctx.sc[inst].outer_status != kRunning) return;
    const int row = lane < lv.tile_rows[tile] ? tile * kTile + lane : -1;
    T q[1] = {T(0)};
    if (row >= 0) {
        const T bv = b[row];
        x[row] = T(0); r[row] = bv; shadow[row] = bv; p[row] = T(0); v[row] = T(0);
        q[0] = bv * bv;
    }
    double out[1];
    if (tile_reduce(q, ctx, inst, tile, out, gid, lane)) {
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
__device__ void bicg_p(const LevelView<T>& lv, int tile, int lane, const T* PSGB_PHASE_RESTRICT r, const T* PSGB_PHASE_RESTRICT v,
                       T* p, T* xv, T omega_j, const InstanceScalars* sc) {
    const int inst = lv.tile_inst[tile];
    if (lane >= lv.tile_rows[tile] || !running(sc[inst])) return;
    const int row = tile * kTile + lane;
    const T beta = T(sc[inst].beta), omega = T(sc[inst].omega);
    const T pv = r[row] + beta * (p[row] - omega * v[row]);
    p[row] = pv;
    if (lv.tile_sweep[tile]) xv[row] = omega_j * lv.inv[row] * pv;
}

// out = A in; dot(shadow, out) -> alpha = rho / (shadow . v)
template <typename T, int W>
__device__ void bicg_v(const LevelView<T>& lv, int tile, int gid, int lane, const T* PSGB_PHASE_RESTRICT in,
                       T* PSGB_PHASE_RESTRICT out, const T* PSGB_PHASE_RESTRICT shadow, const ReduceCtx& ctx) {
    const int inst = lv.tile_inst[tile];
    if (!running(ctx.sc[inst])) return;
    const int row = lane < lv.tile_rows[tile] ? tile * kTile + lane : -1;
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
    if (tile_reduce(q, ctx, inst, tile, sum, gid, lane)) {
        InstanceScalars& s = ctx.sc[inst];
        if (!finite(sum[0])) { s.status = kNonFinite; return; }
        if (sum[0] == 0.0) { s.status = kBreakdown; return; }
        s.alpha = s.rho / sum[0];
    }
}

// s = r - alpha v; ||s||: converged at s -> finish with x += alpha p_hat.
template <typename T>
__device__ void bicg_s(const LevelView<T>& lv, int tile, int gid, int lane, const T* PSGB_PHASE_RESTRICT r,
                       const T* PSGB_PHASE_RESTRICT v, T* PSGB_PHASE_RESTRICT s_out, T* xv, T omega_j, const ReduceCtx& ctx) {
    const int inst = lv.tile_inst[tile];
    if (!running(ctx.sc[inst])) return;
    const int row = lane < lv.tile_rows[tile] ? tile * kTile + lane : -1;
    T q[1] = {T(0)};
    const T alpha = T(ctx.sc[inst].alpha);
    if (row >= 0) {
        const T sv = r[row] - alpha * v[row];
        s_out[row] = sv;
        q[0] = sv * sv;
        if (lv.tile_sweep[tile]) xv[row] = omega_j * lv.inv[row] * sv;
    }
    double sum[1];
    if (tile_reduce(q, ctx, inst, tile, sum, gid, lane)) {
        InstanceScalars& s = ctx.sc[inst];
        s.s_norm = sqrt(sum[0]);
        s.iterations += 1;
        if (!finite(s.s_norm)) { s.status = kNonFinite; return; }
        if (s.s_norm <= s.target) s.half_done = 1;
    }
}

// t = A s_hat; (t.t, t.s) -> omega
template <typename T, int W>
__device__ void bicg_t(const LevelView<T>& lv, int tile, int gid, int lane, const T* PSGB_PHASE_RESTRICT shat,
                       T* PSGB_PHASE_RESTRICT t, const T* PSGB_PHASE_RESTRICT s_vec, const ReduceCtx& ctx) {
    const int inst = lv.tile_inst[tile];
    const InstanceScalars& sc = ctx.sc[inst];
    if (!running(sc) || sc.half_done) return;
    const int row = lane < lv.tile_rows[tile] ? tile * kTile + lane : -1;
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
    if (tile_reduce(q, ctx, inst, tile, sum, gid, lane)) {
        InstanceScalars& s = ctx.sc[inst];
        s.omega = sum[0] > 0.0 ? sum[1] / sum[0] : 0.0;
        if (!finite(s.omega)) s.status = kNonFinite;
    }
}

// x += alpha p_hat + omega s_hat; r = s - omega t; (r.r, shadow.r) -> next rho/beta.
template <typename T>
__device__ void bicg_x(const LevelView<T>& lv, int tile, int gid, int lane, const T* PSGB_PHASE_RESTRICT phat,
                       const T* PSGB_PHASE_RESTRICT shat, const T* PSGB_PHASE_RESTRICT s_vec, const T* PSGB_PHASE_RESTRICT t, T* x, T* r,
                       const T* PSGB_PHASE_RESTRICT shadow, const ReduceCtx& ctx) {
    __shared__ int last[kGroups];
    const int inst = lv.tile_inst[tile];
    const InstanceScalars& sc = ctx.sc[inst];
    if (!running(sc)) return;
    const T alpha = T(sc.alpha), omega = T(sc.omega);
    const int row = lane < lv.tile_rows[tile] ? tile * kTile + lane : -1;
    if (sc.half_done) {
        // uniform over the planet: finish at s without a reduction
        if (row >= 0) x[row] += alpha * phat[row];
        group_sync(gid);
        if (lane == 0) {
            __threadfence();
            const unsigned begin = ctx.tile_begin[inst], end = ctx.tile_begin[inst + 1];
            const unsigned ticket = atomicAdd(&ctx.ticket[inst], 1u);
            last[gid] = ticket == end - begin - 1;
            if (last[gid]) {
                ctx.ticket[inst] = 0;
                InstanceScalars& s = ctx.sc[inst];
                s.r_norm = s.s_norm;
                s.half_done = 0;
                s.status = kConverged;
            }
        }
        group_sync(gid);
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
    if (tile_reduce(q, ctx, inst, tile, sum, gid, lane)) {
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

template <typename T>
__device__ void pcg_init(const LevelView<T>& lv, int tile, int gid, int lane, const T* PSGB_PHASE_RESTRICT b, T* x, T* r,
                         T* p, T* xv, T omega_j, const ReduceCtx& ctx, double tol, int max_it) {
    const int inst = lv.tile_inst[tile];
    if (ctx.sc[inst].outer_status != kRunning) return;
    const int row = lane < lv.tile_rows[tile] ? tile * kTile + lane : -1;
    T q[1] = {T(0)};
    if (row >= 0) {
        const T bv = b[row];
        x[row] = T(0); r[row] = bv; p[row] = T(0);
        if (lv.tile_sweep[tile]) xv[row] = omega_j * lv.inv[row] * bv;
        q[0] = bv * bv;
    }
    double out[1];
    if (tile_reduce(q, ctx, inst, tile, out, gid, lane)) {
        InstanceScalars& s = ctx.sc[inst];
        s.b_norm = sqrt(out[0]);
        s.target = fmax(tol * s.b_norm, 0.5 * s.outer_target);
        s.r_norm = s.b_norm;
        s.iterations = 0; s.half_done = 0; s.max_iterations = max_it; s.first = 1;
        s.rho = 0.0; s.beta = 0.0; s.alpha = 0.0;
        s.status = !finite(s.b_norm) ? kNonFinite : (s.b_norm > 0.0 ? kRunning : kConverged);
    }
}

// rho = r.z, beta = rho / rho_old
template <typename T>
__device__ void pcg_rz(const LevelView<T>& lv, int tile, int gid, int lane, const T* PSGB_PHASE_RESTRICT r,
                       const T* PSGB_PHASE_RESTRICT z, const ReduceCtx& ctx) {
    const int inst = lv.tile_inst[tile];
    if (!running(ctx.sc[inst])) return;
    const int row = lane < lv.tile_rows[tile] ? tile * kTile + lane : -1;
    T q[1] = {T(0)};
    if (row >= 0) q[0] = r[row] * z[row];
    double sum[1];
    if (tile_reduce(q, ctx, inst, tile, sum, gid, lane)) {
        InstanceScalars& s = ctx.sc[inst];
        if (!finite(sum[0])) { s.status = kNonFinite; return; }
        if (!(sum[0] > 0.0)) { s.status = s.first ? kConverged : kBreakdown; return; }
        s.beta = s.first ? 0.0 : sum[0] / s.rho;
        s.rho = sum[0];
        s.first = 0;
    }
}

template <typename T>
__device__ void pcg_p(const LevelView<T>& lv, int tile, int lane, const T* PSGB_PHASE_RESTRICT z, T* p,
                      const InstanceScalars* sc) {
    const int inst = lv.tile_inst[tile];
    if (lane >= lv.tile_rows[tile] || !running(sc[inst])) return;
    const int row = tile * kTile + lane;
    p[row] = z[row] + T(sc[inst].beta) * p[row];
}

// q = A p; alpha = rho / p.q
template <typename T, int W>
__device__ void pcg_q(const LevelView<T>& lv, int tile, int gid, int lane, const T* PSGB_PHASE_RESTRICT p,
                      T* PSGB_PHASE_RESTRICT q_out, const ReduceCtx& ctx) {
    const int inst = lv.tile_inst[tile];
    if (!running(ctx.sc[inst])) return;
    const int row = lane < lv.tile_rows[tile] ? tile * kTile + lane : -1;
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
    if (tile_reduce(q, ctx, inst, tile, sum, gid, lane)) {
        InstanceScalars& s = ctx.sc[inst];
        if (!finite(sum[0])) { s.status = kNonFinite; return; }
        if (!(sum[0] > 0.0)) { s.status = kBreakdown; return; }
        s.alpha = s.rho / sum[0];
    }
}

// x += alpha p; r -= alpha q; ||r|| -> converged?; first sweep of M r.
template <typename T>
__device__ void pcg_xr(const LevelView<T>& lv, int tile, int gid, int lane, const T* PSGB_PHASE_RESTRICT p,
                       const T* PSGB_PHASE_RESTRICT q_in, T* x, T* r, T* xv, T omega_j, const ReduceCtx& ctx) {
    const int inst = lv.tile_inst[tile];
    if (!running(ctx.sc[inst])) return;
    const T alpha = T(ctx.sc[inst].alpha);
    const int row = lane < lv.tile_rows[tile] ? tile * kTile + lane : -1;
    T q[1] = {T(0)};
    if (row >= 0) {
        x[row] += alpha * p[row];
        const T rv = r[row] - alpha * q_in[row];
        r[row] = rv;
        q[0] = rv * rv;
        if (lv.tile_sweep[tile]) xv[row] = omega_j * lv.inv[row] * rv;
    }
    double sum[1];
    if (tile_reduce(q, ctx, inst, tile, sum, gid, lane)) {
        InstanceScalars& s = ctx.sc[inst];
        s.r_norm = sqrt(sum[0]);
        s.iterations += 1;
        if (!finite(s.r_norm)) { s.status = kNonFinite; return; }
        if (s.r_norm <= s.target) { s.status = kConverged; return; }
        if (s.iterations >= s.max_iterations) s.status = kCap;
    }
}

// ---- FP64 refinement ----------------------------------------------------------------------

__device__ inline void outer_init(const LevelView<double>& lv, int tile, int gid, int lane,
                                  const double* PSGB_PHASE_RESTRICT b, const ReduceCtx& ctx, double tol,
                                  const std::uint8_t* PSGB_PHASE_RESTRICT active) {
    const int inst = lv.tile_inst[tile];
    if (active != nullptr && !active[inst]) {
        // a planet left out of this step: nothing runs for it
        if (lane == 0 && static_cast<unsigned>(tile) == ctx.tile_begin[inst]) {
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
    const int row = lane < lv.tile_rows[tile] ? tile * kTile + lane : -1;
    double q[1] = {0.0};
    if (row >= 0) q[0] = dmul(b[row], b[row]);
    double sum[1];
    if (tile_reduce(q, ctx, inst, tile, sum, gid, lane)) {
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
__device__ void outer_residual(const LevelView<double>& lv, int tile, int gid, int lane, const double* PSGB_PHASE_RESTRICT b,
                               const double* PSGB_PHASE_RESTRICT x, double* PSGB_PHASE_RESTRICT r64, TI* PSGB_PHASE_RESTRICT rin,
                               const ReduceCtx& ctx, int max_refine) {
    const int inst = lv.tile_inst[tile];
    if (ctx.sc[inst].outer_status != kRunning) return;
    const int row = lane < lv.tile_rows[tile] ? tile * kTile + lane : -1;
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
    if (tile_reduce(q, ctx, inst, tile, sum, gid, lane)) {
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
__device__ void outer_update(const LevelView<double>& lv, int tile, int lane, const TI* PSGB_PHASE_RESTRICT delta, double* x,
                             const InstanceScalars* sc) {
    const int inst = lv.tile_inst[tile];
    if (sc[inst].outer_status != kRunning) return;
    if (lane < lv.tile_rows[tile]) {
        const int row = tile * kTile + lane;
        x[row] += static_cast<double>(delta[row]);
    }
}

__device__ inline void outer_account(InstanceScalars& s) {
    if (s.outer_status != kRunning) return;
    s.inner_total += s.iterations;
    if (s.status == kNonFinite) s.outer_status = kNonFinite;
}

}  // namespace ph
}  // namespace psgb

// Multi-right-hand-side block solve: up to 32 sub-steps of ONE planet, one matrix, solved
// together (the 32-RHS L8 workload). The reference solves each right-hand side with its own
// call of solve_implicit_transport / solve_newton_system (sim/planet/surface/
// heat_transport.cpp:337-429, 595-772), reading the matrix once per right-hand side; here
// every sweep reads the matrix and its column indices once for all of them.
//
// Layout: every vector interleaved, entry (row, rhs) at row * 32 + rhs. One block per
// 256-row tile of the planet's level, one warp per 32 of its rows, lane = right-hand side:
// a row's columns, values and inverse diagonal are one broadcast load per warp, and each
// neighbour gather is one 128-byte (FP32) or 256-byte (FP64) line for all 32 right-hand
// sides. The matrix and its hierarchy are the planet's one-planet batch's (assembled, the
// Galerkin values and coarsest inverses computed as for a single solve).
//
// Every row's arithmetic is the single-RHS phase's (phases.cuh), expression for
// expression, and every reduction reproduces the single-RHS tree: a tile's partial is the
// warp butterfly over each 32-row run (formed here in registers in the butterfly's own
// order), then the eight warps in order, in the phase's precision; the per-RHS finish sums
// the tile partials exactly as the single solve's finish does. Each right-hand side
// therefore follows the single solve of that sub-step bit for bit.
#include "common.cuh"
#include "kernels.hpp"
#include "multirhs.hpp"
#include "phases.cuh"
#include "profile.hpp"

#include <stdexcept>

namespace psgb {
namespace mr {
namespace {

struct TileInfo {
    int rows;     // valid rows of the tile
    bool sweep;   // the planet smooths on this level
};

__device__ __forceinline__ TileInfo tile_info(const std::uint32_t* meta, int tile) {
    const std::uint32_t w = meta[tile];
    return TileInfo{static_cast<int>((w >> 22) & 0x1FFu), (w >> 31) != 0u};
}

__device__ __forceinline__ std::size_t at(int row, int lane) {
    return static_cast<std::size_t>(row) * kRhs + static_cast<std::size_t>(lane);
}

// Row of the tile handled by this warp for run g (0..7) and slot i (0..3): the warp's 32
// rows are visited four at a time, {g, g+8, g+16, g+24}, the pairs the butterfly combines.
__device__ __forceinline__ int local_row(int warp, int g, int i) { return warp * 32 + g + 8 * i; }

// The warp butterfly of warp_sum over the warp's 32 row values, from the per-run values
// b[g] = (v[g] + v[g+16]) + (v[g+8] + v[g+24]).
template <typename A>
__device__ __forceinline__ A butterfly(const A (&b)[8]) {
    A c[4], d[2];
#pragma unroll
    for (int k = 0; k < 4; ++k) c[k] = b[k] + b[k + 4];
#pragma unroll
    for (int k = 0; k < 2; ++k) d[k] = c[k] + c[k + 2];
    return d[0] + d[1];
}

template <typename A>
__device__ __forceinline__ A run_value(const A (&v)[4]) {
    return (v[0] + v[2]) + (v[1] + v[3]);
}

// Tile partials of NQ quantities: warp values in order of warps, as group_sum, stored in
// FP64 at part[(q * tiles + tile) * 32 + lane].
template <typename A, int NQ>
__device__ __forceinline__ void tile_partials(const A (&warp_value)[NQ], double* part, int tiles, int tile, bool store) {
    __shared__ A sm[NQ][8][kRhs];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NQ; ++q) sm[q][warp][lane] = warp_value[q];
    __syncthreads();
    if (warp == 0 && store) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            A s = sm[q][0][lane];
#pragma unroll
            for (int w = 1; w < 8; ++w) s += sm[q][w][lane];
            part[(static_cast<std::size_t>(q) * tiles + tile) * kRhs + lane] = static_cast<double>(s);
        }
    }
}

__device__ __forceinline__ void count(unsigned long long* counter, unsigned long long bytes) {
    if (counter != nullptr && threadIdx.x == 0 && bytes != 0) atomicAdd(counter, bytes);
}

// A tile's 256 rows of a level's matrix (columns, off-diagonal values, optionally the
// diagonal and its inverse) staged in shared memory with coalesced loads, thread t taking
// row t: the warps' row loops then read their rows' columns and values there (broadcast)
// and go to global memory only for the right-hand sides' vectors, one dependent round
// trip per group of rows instead of two.
template <typename T, int W, bool Diag, bool Inv>
struct TileRows {
    int col[W][kTile];
    T val[W + (Diag ? 1 : 0)][kTile];
    T inv[Inv ? kTile : 1];
};

template <typename T, int W, bool Diag, bool Inv>
__device__ __forceinline__ void stage_rows(const LevelView<T>& L, int tile, TileRows<T, W, Diag, Inv>& m) {
    const std::uint32_t P = L.rows;
    const int t = threadIdx.x, row = tile * kTile + t;
#pragma unroll
    for (int j = 0; j < W; ++j) {
        m.col[j][t] = L.col[j * P + row];
        m.val[j][t] = L.vd[j * P + row];
    }
    if constexpr (Diag) m.val[W][t] = L.vd[W * P + row];
    if constexpr (Inv) m.inv[t] = L.inv[row];
    __syncthreads();
}

// ---- V-cycle ----------------------------------------------------------------------------

template <typename T>
__global__ void k_smooth_zero(LevelView<T> L, const T* __restrict__ b, T* __restrict__ x, T omega,
                              const InstanceScalars* sc, int gate) {
    pdl_begin();
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(L.tile_meta, tile);
    if (!ti.sweep) return;
    count(L.bytes, static_cast<unsigned long long>(ti.rows) * (sizeof(T) + 2ull * kRhs * sizeof(T)));
    if (!ph::gate_open(sc, lane, gate)) return;
    for (int g = 0; g < 8; ++g) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i), row = tile * kTile + local;
            const T y = omega * L.inv[row] * b[at(row, lane)];
            if (local < ti.rows) x[at(row, lane)] = y;
        }
    }
}

template <typename T, int W>
__global__ void k_smooth(LevelView<T> L, const T* __restrict__ b, const T* __restrict__ x, T* __restrict__ y, T omega,
                         const InstanceScalars* sc, int gate) {
    pdl_begin();
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(L.tile_meta, tile);
    if (!ti.sweep) return;
    __shared__ TileRows<T, W, false, true> m;
    stage_rows(L, tile, m);
    count(L.bytes, static_cast<unsigned long long>(ti.rows) * (4ull * W + sizeof(T) * (W + 1ull) + 3ull * kRhs * sizeof(T)));
    if (!ph::gate_open(sc, lane, gate)) return;
    for (int g = 0; g < 8; ++g) {
        T out[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i), row = tile * kTile + local;
            T s = b[at(row, lane)];
#pragma unroll
            for (int j = 0; j < W; ++j) s -= m.val[j][local] * x[at(m.col[j][local], lane)];
            if (omega == T(1)) {
                out[i] = m.inv[local] * s;
            } else {
                const T xo = x[at(row, lane)];
                out[i] = xo + omega * (m.inv[local] * s - xo);
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i);
            if (local < ti.rows) y[at(tile * kTile + local, lane)] = out[i];
        }
    }
}

// Block-local Jacobi for every right-hand side: `inner` sweeps of one tile in one launch,
// the tile's own rows updated in shared memory between sweeps (double-buffered) and the
// neighbours in other tiles held at x, the single solve's block sweep (ph::smooth_block)
// term for term. Dynamic shared memory: the tile's columns, values, 1/diag and two copies
// of its 256 rows x 32 right-hand sides. A right-hand side whose solve is not running still
// computes (the block's barriers need every thread) but stores nothing.
template <typename T, int W>
struct BlockSweepSmem {
    static constexpr std::size_t kCol = std::size_t(W) * kTile * sizeof(int);
    static constexpr std::size_t kVal = std::size_t(W) * kTile * sizeof(T);
    static constexpr std::size_t kInv = std::size_t(kTile) * sizeof(T);
    static constexpr std::size_t kX = std::size_t(kTile) * kRhs * sizeof(T);
    static constexpr std::size_t bytes = kCol + kVal + kInv + 2 * kX;
};

template <typename T, int W>
__global__ void __launch_bounds__(kTile) k_smooth_block(LevelView<T> L, const T* __restrict__ b,
                                                        const T* __restrict__ x, T* __restrict__ y, T omega, int inner,
                                                        const InstanceScalars* sc, int gate) {
    pdl_begin();
    using S = BlockSweepSmem<T, W>;
    extern __shared__ __align__(16) unsigned char block_sweep_bytes[];
    int(*col)[kTile] = reinterpret_cast<int(*)[kTile]>(block_sweep_bytes);
    T(*val)[kTile] = reinterpret_cast<T(*)[kTile]>(block_sweep_bytes + S::kCol);
    T* inv = reinterpret_cast<T*>(block_sweep_bytes + S::kCol + S::kVal);
    T(*xs[2])[kRhs] = {reinterpret_cast<T(*)[kRhs]>(block_sweep_bytes + S::kCol + S::kVal + S::kInv),
                       reinterpret_cast<T(*)[kRhs]>(block_sweep_bytes + S::kCol + S::kVal + S::kInv + S::kX)};
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(L.tile_meta, tile);
    if (!ti.sweep) return;   // the whole block
    const std::uint32_t P = L.rows;
    const int first = tile * kTile;
    {
        const int t = threadIdx.x, row = first + t;
#pragma unroll
        for (int j = 0; j < W; ++j) {
            col[j][t] = L.col[j * P + row];
            val[j][t] = L.vd[j * P + row];
        }
        inv[t] = L.inv[row];
    }
    count(L.bytes, static_cast<unsigned long long>(ti.rows) * (4ull * W + sizeof(T) * (W + 1ull) + 3ull * kRhs * sizeof(T)));
    const bool on = ph::gate_open(sc, lane, gate);
    // the iterate the sweeps start from: the tile's rows of x (0 on padding rows)
    for (int k = 0; k < 32; ++k) {
        const int local = warp * 32 + k;
        xs[0][local][lane] = local < ti.rows ? x[at(first + local, lane)] : T(0);
    }
    __syncthreads();
    int cur = 0;
    for (int sweep = 0; sweep < inner; ++sweep) {
        for (int k = 0; k < 32; ++k) {
            const int local = warp * 32 + k;
            const T xo = xs[cur][local][lane];
            T out = xo;
            if (local < ti.rows) {
                T s = b[at(first + local, lane)];
#pragma unroll
                for (int j = 0; j < W; ++j) {
                    const int c = col[j][local];
                    const T v = (c >= first && c < first + kTile) ? xs[cur][c - first][lane] : x[at(c, lane)];
                    s = ph::fnma(val[j][local], v, s);
                }
                out = ph::jacobi_update(xo, omega, inv[local], s);
            }
            xs[cur ^ 1][local][lane] = out;
        }
        __syncthreads();
        cur ^= 1;
    }
    if (!on) return;
    for (int k = 0; k < 32; ++k) {
        const int local = warp * 32 + k;
        if (local < ti.rows) y[at(first + local, lane)] = xs[cur][local][lane];
    }
}

template <typename T, int W>
void set_block_sweep_smem() {
    static const bool done = [] {
        PSGB_CUDA(cudaFuncSetAttribute(k_smooth_block<T, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(BlockSweepSmem<T, W>::bytes)));
        return true;
    }();
    (void)done;
}

template <typename T, int W>
__global__ void k_residual(LevelView<T> L, const T* __restrict__ b, const T* __restrict__ x, T* __restrict__ r,
                           const InstanceScalars* sc, int gate) {
    pdl_begin();
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(L.tile_meta, tile);
    if (!ti.sweep) return;
    __shared__ TileRows<T, W, true, false> m;
    stage_rows(L, tile, m);
    count(L.bytes, static_cast<unsigned long long>(ti.rows) * (4ull * W + sizeof(T) * (W + 1ull) + 3ull * kRhs * sizeof(T)));
    if (!ph::gate_open(sc, lane, gate)) return;
    for (int g = 0; g < 8; ++g) {
        T out[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i), row = tile * kTile + local;
            T s = b[at(row, lane)] - m.val[W][local] * x[at(row, lane)];
#pragma unroll
            for (int j = 0; j < W; ++j) s -= m.val[j][local] * x[at(m.col[j][local], lane)];
            out[i] = s;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i);
            if (local < ti.rows) r[at(tile * kTile + local, lane)] = out[i];
        }
    }
}

// b_c = sum of the members' residuals in ascending order; x_c = omega b_c / diag.
template <typename T>
__global__ void k_restrict_zero(LevelView<T> C, const std::uint32_t* __restrict__ moff,
                                const std::uint32_t* __restrict__ member, const T* __restrict__ r,
                                T* __restrict__ bc, T* __restrict__ xc, T omega, const InstanceScalars* sc, int gate) {
    pdl_begin();
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(C.tile_meta, tile);
    if (ti.rows == 0 || !ph::gate_open(sc, lane, gate)) return;
    unsigned long long moved = 0;
    for (int k = 0; k < 32; ++k) {
        const int local = warp * 32 + k;
        if (local >= ti.rows) break;
        const int row = tile * kTile + local;
        const std::uint32_t k0 = moff[row], k1 = moff[row + 1];
        T s = T(0);
        for (std::uint32_t m = k0; m < k1; m += 8) {
            T v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = (m + u < k1) ? r[at(static_cast<int>(member[m + u]), lane)] : T(0);
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if (m + u < k1) s += v[u];
            }
        }
        bc[at(row, lane)] = s;
        if (ti.sweep) xc[at(row, lane)] = omega * C.inv[row] * s;
        moved += 4ull + (k1 - k0) * (4ull + kRhs * sizeof(T)) + sizeof(T) + 2ull * kRhs * sizeof(T);
    }
    if (C.bytes != nullptr && lane == 0 && moved != 0) atomicAdd(C.bytes, moved);
}

// With x' = x + e[agg]: y = x' + omega (D^-1 (b - O x') - x').
template <typename T, int W>
__global__ void k_prolong_smooth(LevelView<T> L, const std::int32_t* __restrict__ agg, const T* __restrict__ e,
                                 const T* __restrict__ b, const T* __restrict__ x, T* __restrict__ y, T omega,
                                 const InstanceScalars* sc, int gate) {
    pdl_begin();
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(L.tile_meta, tile);
    if (!ti.sweep) return;
    __shared__ TileRows<T, W, false, true> m;
    stage_rows(L, tile, m);
    count(L.bytes, static_cast<unsigned long long>(ti.rows) * (4ull * W + sizeof(T) * (W + 1ull) + 4ull + 3ull * kRhs * sizeof(T)));
    if (!ph::gate_open(sc, lane, gate)) return;
    for (int g = 0; g < 8; ++g) {
        T out[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i), row = tile * kTile + local;
            T s = b[at(row, lane)];
#pragma unroll
            for (int j = 0; j < W; ++j) {
                const int c = m.col[j][local];
                s -= m.val[j][local] * (x[at(c, lane)] + ph::prod(L.correction, e[at(agg[c], lane)]));
            }
            if (omega == T(1)) {
                out[i] = m.inv[local] * s;
            } else {
                const T xo = x[at(row, lane)] + ph::prod(L.correction, e[at(agg[row], lane)]);
                out[i] = xo + omega * (m.inv[local] * s - xo);
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i);
            if (local < ti.rows) y[at(tile * kTile + local, lane)] = out[i];
        }
    }
}

template <typename T>
__global__ void k_prolong(LevelView<T> L, const std::int32_t* __restrict__ agg, const T* __restrict__ xc, T* x,
                          const InstanceScalars* sc, int gate) {
    pdl_begin();
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(L.tile_meta, tile);
    if (!ti.sweep) return;
    count(L.bytes, static_cast<unsigned long long>(ti.rows) * (4ull + 2ull * kRhs * sizeof(T)));
    if (!ph::gate_open(sc, lane, gate)) return;
    for (int k = 0; k < 32; ++k) {
        const int local = warp * 32 + k;
        if (local >= ti.rows) break;
        const int row = tile * kTile + local;
        x[at(row, lane)] += ph::prod(L.correction, xc[at(agg[row], lane)]);
    }
}

// Coarsest level: x = A^-1 b, row i in warp i of the grid, lane = right-hand side. The
// single solve's warp sums a[k] b[k] over k = l, l + 32, ... in lane l, then the butterfly
// over l; here each lane forms those 32 sums itself, in the butterfly's pairing.
template <typename T>
__global__ void k_dense(int n, const T* __restrict__ inv, const T* __restrict__ b, T* __restrict__ x,
                        const InstanceScalars* sc, int gate, unsigned long long* bytes) {
    pdl_begin();
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= n) return;
    if (bytes != nullptr && lane == 0) atomicAdd(bytes, static_cast<unsigned long long>(n) * sizeof(T) + kRhs * sizeof(T));
    if (!ph::gate_open(sc, lane, gate)) return;
    const T* a = inv + static_cast<std::size_t>(i) * n;
    T run[8];
#pragma unroll
    for (int g = 0; g < 8; ++g) {
        T v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int l = g + 8 * u;
            T s = T(0);
            for (int k = l; k < n; k += 32) s += a[k] * b[at(k, lane)];
            v[u] = s;
        }
        run[g] = run_value(v);
    }
    x[at(i, lane)] = butterfly(run);
}

// ---- Krylov (fine level) ---------------------------------------------------------------------

template <typename T>
__global__ void k_bicg_init(LevelView<T> L, const T* __restrict__ b, T* x, T* r, T* shadow, T* p, T* v,
                            Ctx ctx) {
    pdl_begin();
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(L.tile_meta, tile);
    const bool on = ti.rows > 0 && ctx.sc[lane].outer_status == kRunning;
    count(L.bytes, static_cast<unsigned long long>(ti.rows) * 6ull * kRhs * sizeof(T));
    T run[8];
    for (int g = 0; g < 8; ++g) {
        T q[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i), row = tile * kTile + local;
            q[i] = T(0);
            if (!on || local >= ti.rows) continue;
            const T bv = b[at(row, lane)];
            x[at(row, lane)] = T(0); r[at(row, lane)] = bv; shadow[at(row, lane)] = bv; p[at(row, lane)] = T(0);
            v[at(row, lane)] = T(0);
            q[i] = ph::prod(bv, bv);
        }
        run[g] = run_value(q);
    }
    const T wv[1] = {butterfly(run)};
    tile_partials<T, 1>(wv, ctx.part, L.tiles, tile, true);
}

template <typename T>
__global__ void k_bicg_p(LevelView<T> L, const T* __restrict__ r, const T* __restrict__ v, T* p, T* xv, T omega_j,
                         const InstanceScalars* sc) {
    pdl_begin();
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(L.tile_meta, tile);
    count(L.bytes, static_cast<unsigned long long>(ti.rows) * (sizeof(T) + 5ull * kRhs * sizeof(T)));
    if (ti.rows == 0 || !ph::running(sc[lane])) return;
    const T beta = T(sc[lane].beta), omega = T(sc[lane].omega);
    for (int g = 0; g < 8; ++g) {
        T pv[4], zv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int row = tile * kTile + local_row(warp, g, i);
            pv[i] = r[at(row, lane)] + beta * (p[at(row, lane)] - omega * v[at(row, lane)]);
            zv[i] = omega_j * L.inv[row] * pv[i];
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i), row = tile * kTile + local;
            if (local >= ti.rows) continue;
            p[at(row, lane)] = pv[i];
            if (ti.sweep) xv[at(row, lane)] = zv[i];
        }
    }
}

// out = A in; shadow . out
template <typename T, int W>
__global__ void k_bicg_v(LevelView<T> L, const T* __restrict__ in, T* __restrict__ out, const T* __restrict__ shadow,
                         Ctx ctx) {
    pdl_begin();
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(L.tile_meta, tile);
    __shared__ TileRows<T, W, true, false> m;
    stage_rows(L, tile, m);
    const bool on = ti.rows > 0 && ph::running(ctx.sc[lane]);
    count(L.bytes, static_cast<unsigned long long>(ti.rows) * (4ull * W + sizeof(T) * (W + 1ull) + 3ull * kRhs * sizeof(T)));
    T run[8];
    for (int g = 0; g < 8; ++g) {
        T q[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i), row = tile * kTile + local;
            T s = m.val[W][local] * in[at(row, lane)];
#pragma unroll
            for (int j = 0; j < W; ++j) s += m.val[j][local] * in[at(m.col[j][local], lane)];
            q[i] = ph::prod(shadow[at(row, lane)], s);
            const bool store = on && local < ti.rows;
            if (store) out[at(row, lane)] = s;
            if (!store) q[i] = T(0);
        }
        run[g] = run_value(q);
    }
    const T wv[1] = {butterfly(run)};
    tile_partials<T, 1>(wv, ctx.part, L.tiles, tile, true);
}

// s = r - alpha v; s . s; first sweep of M s.
template <typename T>
__global__ void k_bicg_s(LevelView<T> L, const T* __restrict__ r, const T* __restrict__ v, T* __restrict__ s_out,
                         T* xv, T omega_j, Ctx ctx) {
    pdl_begin();
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(L.tile_meta, tile);
    const bool on = ti.rows > 0 && ph::running(ctx.sc[lane]);
    const T alpha = T(ctx.sc[lane].alpha);
    count(L.bytes, static_cast<unsigned long long>(ti.rows) * (sizeof(T) + 4ull * kRhs * sizeof(T)));
    T run[8];
    for (int g = 0; g < 8; ++g) {
        T q[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i), row = tile * kTile + local;
            const T sv = r[at(row, lane)] - alpha * v[at(row, lane)];
            const T zv = omega_j * L.inv[row] * sv;
            q[i] = T(0);
            if (!on || local >= ti.rows) continue;
            s_out[at(row, lane)] = sv;
            q[i] = ph::prod(sv, sv);
            if (ti.sweep) xv[at(row, lane)] = zv;
        }
        run[g] = run_value(q);
    }
    const T wv[1] = {butterfly(run)};
    tile_partials<T, 1>(wv, ctx.part, L.tiles, tile, true);
}

// t = A s_hat; (t . t, t . s)
template <typename T, int W>
__global__ void k_bicg_t(LevelView<T> L, const T* __restrict__ shat, T* __restrict__ t, const T* __restrict__ s_vec,
                         Ctx ctx) {
    pdl_begin();
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(L.tile_meta, tile);
    __shared__ TileRows<T, W, true, false> m;
    stage_rows(L, tile, m);
    const bool on = ti.rows > 0 && ph::running(ctx.sc[lane]) && !ctx.sc[lane].half_done;
    count(L.bytes, static_cast<unsigned long long>(ti.rows) * (4ull * W + sizeof(T) * (W + 1ull) + 3ull * kRhs * sizeof(T)));
    T run0[8], run1[8];
    for (int g = 0; g < 8; ++g) {
        T q0[4], q1[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i), row = tile * kTile + local;
            T s = m.val[W][local] * shat[at(row, lane)];
#pragma unroll
            for (int j = 0; j < W; ++j) s += m.val[j][local] * shat[at(m.col[j][local], lane)];
            q0[i] = ph::prod(s, s);
            q1[i] = ph::prod(s, s_vec[at(row, lane)]);
            const bool store = on && local < ti.rows;
            if (store) t[at(row, lane)] = s;
            if (!store) { q0[i] = T(0); q1[i] = T(0); }
        }
        run0[g] = run_value(q0);
        run1[g] = run_value(q1);
    }
    const T wv[2] = {butterfly(run0), butterfly(run1)};
    tile_partials<T, 2>(wv, ctx.part, L.tiles, tile, true);
}

// x += alpha p_hat + omega s_hat; r = s - omega t; (r . r, shadow . r); a right-hand side
// converged at s finishes with x += alpha p_hat.
template <typename T>
__global__ void k_bicg_x(LevelView<T> L, const T* __restrict__ phat, const T* __restrict__ shat,
                         const T* __restrict__ s_vec, const T* __restrict__ t, T* x, T* r,
                         const T* __restrict__ shadow, Ctx ctx) {
    pdl_begin();
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(L.tile_meta, tile);
    const InstanceScalars& sc = ctx.sc[lane];
    const bool on = ti.rows > 0 && ph::running(sc);
    const bool half = sc.half_done != 0;
    const T alpha = T(sc.alpha), omega = T(sc.omega);
    count(L.bytes, static_cast<unsigned long long>(ti.rows) * 8ull * kRhs * sizeof(T));
    T run0[8], run1[8];
    for (int g = 0; g < 8; ++g) {
        T q0[4], q1[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i), row = tile * kTile + local;
            T xv, rv;
            if (half) {
                xv = x[at(row, lane)] + alpha * phat[at(row, lane)];
                rv = T(0);
            } else {
                xv = x[at(row, lane)] + (alpha * phat[at(row, lane)] + omega * shat[at(row, lane)]);
                rv = s_vec[at(row, lane)] - omega * t[at(row, lane)];
            }
            q0[i] = ph::prod(rv, rv);
            q1[i] = ph::prod(shadow[at(row, lane)], rv);
            const bool store = on && local < ti.rows;
            if (store) {
                x[at(row, lane)] = xv;
                if (!half) r[at(row, lane)] = rv;
            }
            if (!store || half) { q0[i] = T(0); q1[i] = T(0); }
        }
        run0[g] = run_value(q0);
        run1[g] = run_value(q1);
    }
    const T wv[2] = {butterfly(run0), butterfly(run1)};
    tile_partials<T, 2>(wv, ctx.part, L.tiles, tile, true);
}

// ---- FP64 refinement ----------------------------------------------------------------------

__global__ void k_outer_init(LevelView<double> L, const double* __restrict__ b, Ctx ctx) {
    pdl_begin();
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(L.tile_meta, tile);
    count(L.bytes, static_cast<unsigned long long>(ti.rows) * 8ull * kRhs);
    double run[8];
    for (int g = 0; g < 8; ++g) {
        double q[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i), row = tile * kTile + local;
            q[i] = (ti.rows > 0 && local < ti.rows) ? dmul(b[at(row, lane)], b[at(row, lane)]) : 0.0;
        }
        run[g] = run_value(q);
    }
    const double wv[1] = {butterfly(run)};
    tile_partials<double, 1>(wv, ctx.part, L.tiles, tile, true);
}

// r = b - A x in FP64, cast to the inner precision; r . r
template <typename TI, int W>
__global__ void k_outer_residual(LevelView<double> L, const double* __restrict__ b, const double* __restrict__ x,
                                 double* __restrict__ r64, TI* __restrict__ rin, Ctx ctx) {
    pdl_begin();
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(L.tile_meta, tile);
    __shared__ TileRows<double, W, true, false> m;
    stage_rows(L, tile, m);
    const bool on = ti.rows > 0 && ctx.sc[lane].outer_status == kRunning;
    count(L.bytes, static_cast<unsigned long long>(ti.rows) * (4ull * W + 8ull * (W + 1ull) + kRhs * (24ull + sizeof(TI))));
    double run[8];
    for (int g = 0; g < 8; ++g) {
        double q[4], rv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i), row = tile * kTile + local;
            double s = b[at(row, lane)] - m.val[W][local] * x[at(row, lane)];
#pragma unroll
            for (int j = 0; j < W; ++j) s -= m.val[j][local] * x[at(m.col[j][local], lane)];
            rv[i] = s;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int local = local_row(warp, g, i), row = tile * kTile + local;
            q[i] = 0.0;
            if (!on || local >= ti.rows) continue;
            r64[at(row, lane)] = rv[i];
            rin[at(row, lane)] = static_cast<TI>(rv[i]);
            q[i] = ph::prod(rv[i], rv[i]);
        }
        run[g] = run_value(q);
    }
    const double wv[1] = {butterfly(run)};
    tile_partials<double, 1>(wv, ctx.part, L.tiles, tile, true);
}

template <typename TI>
__global__ void k_outer_update(LevelView<double> L, const TI* __restrict__ delta, double* x, const InstanceScalars* sc) {
    pdl_begin();
    const int tile = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileInfo ti = tile_info(L.tile_meta, tile);
    count(L.bytes, static_cast<unsigned long long>(ti.rows) * kRhs * (16ull + sizeof(TI)));
    if (ti.rows == 0 || sc[lane].outer_status != kRunning) return;
    for (int k = 0; k < 32; ++k) {
        const int local = warp * 32 + k;
        if (local >= ti.rows) break;
        const int row = tile * kTile + local;
        x[at(row, lane)] += static_cast<double>(delta[at(row, lane)]);
    }
}

__global__ void k_outer_account(InstanceScalars* sc) {
    pdl_begin();
    if (threadIdx.x < kRhs) ph::outer_account(sc[threadIdx.x]);
}

// ---- per-RHS completion of a reduction --------------------------------------------------

// Right-hand side blockIdx.x: its tile partials in tile order exactly as the single
// solve's finish sums a planet's (lane l: tiles l, l + 256, ..., four loads in flight),
// the group's fixed tree, then the scalar step.
template <int K>
__global__ void k_finish(Ctx ctx, int tiles, ph::FinishParams p) {
    pdl_begin();
    constexpr int NQ = ph::FinishSums<K>::value;
    const int j = blockIdx.x, lane = threadIdx.x;
    if (!ph::finish_gate<K>(ctx.sc[j], j, p)) return;
    double acc[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] = 0.0;
    for (int t0 = lane; t0 < tiles; t0 += 4 * kTile) {
        double v[4][NQ];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int t = t0 + u * kTile;
#pragma unroll
            for (int q = 0; q < NQ; ++q)
                v[u][q] = t < tiles ? __ldcg(&ctx.part[(static_cast<std::size_t>(q) * tiles + t) * kRhs + j]) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (t0 + u * kTile < tiles) {
#pragma unroll
                for (int q = 0; q < NQ; ++q) acc[q] += v[u][q];
            }
        }
    }
    ph::group_sum<double, NQ>(acc, 0, lane);
    if (lane == 0) ph::finish_step<K>(ctx.sc[j], acc, p);
}

// ---- the step's inputs and outputs ---------------------------------------------------------

// Right-hand sides (A / s) T0_j + A S_j and initial guesses T0_j, as k_step_rhs forms them;
// padding rows and unused right-hand sides zero.
__global__ void k_load(std::uint32_t n, std::uint32_t P, int count, const double* const* __restrict__ t0,
                       const double* const* __restrict__ src, const double* __restrict__ area, double s,
                       double* __restrict__ rhs, double* __restrict__ x0) {
    const std::size_t k = blockIdx.x * std::size_t(blockDim.x) + threadIdx.x;
    if (k >= std::size_t(P) * kRhs) return;
    const std::uint32_t row = static_cast<std::uint32_t>(k / kRhs);
    const int j = static_cast<int>(k % kRhs);
    if (row >= n || j >= count) {
        rhs[k] = 0.0;
        x0[k] = 0.0;
        return;
    }
    const double a = area[row];
    rhs[k] = dadd(dmul(__ddiv_rn(a, s), t0[j][row]), dmul(a, src[j][row]));
    x0[k] = t0[j][row];
}

// Right-hand side j's entries into a vector of the planet's layout.
__global__ void k_take(std::uint32_t P, int j, const double* __restrict__ x, double* __restrict__ out) {
    const std::uint32_t row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row < P) out[row] = x[at(static_cast<int>(row), j)];
}

}  // namespace

// ---- launchers --------------------------------------------------------------------------

#define PSGB_MR_WIDTHS(width, ...)                                             \
    switch (width) {                                                           \
        case 6: { constexpr int W = 6; __VA_ARGS__; } break;                   \
        case 8: { constexpr int W = 8; __VA_ARGS__; } break;                   \
        case 12: { constexpr int W = 12; __VA_ARGS__; } break;                 \
        case 16: { constexpr int W = 16; __VA_ARGS__; } break;                 \
        default: throw std::logic_error("unsupported ELL width");              \
    }

template <int K>
void finish(const Ctx& ctx, int tiles, int family, cudaStream_t st, ph::FinishParams p = {}) {
    PSGB_LAUNCH(family, st, launch_pdl(k_finish<K>, kRhs, kTile, st, ctx, tiles, p));
}

template <typename T>
void Launch<T>::smooth_zero(const LevelView<T>& L, const T* b, T* x, T omega, const InstanceScalars* sc, int gate,
                            cudaStream_t st) {
    const int fam = L.level == 0 ? kFamSmooth : kFamSmoothCoarse;
    PSGB_LAUNCH(fam, st, launch_pdl(k_smooth_zero<T>, L.tiles, kTile, st, counted(L, fam), b, x, omega, sc, gate));
}
template <typename T>
void Launch<T>::smooth(const LevelView<T>& L, const T* b, const T* x, T* y, T omega, const InstanceScalars* sc,
                       int gate, cudaStream_t st, int inner) {
    const int fam = L.level == 0 ? kFamSmooth : kFamSmoothCoarse;
    if (inner > 1) {
        PSGB_LAUNCH(fam, st, PSGB_MR_WIDTHS(L.width, {
            set_block_sweep_smem<T, W>();
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            attr[0].val.programmaticStreamSerializationAllowed = 1;
            cudaLaunchConfig_t cfg{};
            cfg.gridDim = dim3(L.tiles);
            cfg.blockDim = dim3(kTile);
            cfg.dynamicSmemBytes = BlockSweepSmem<T, W>::bytes;
            cfg.stream = st;
            cfg.attrs = attr;
            cfg.numAttrs = L.tiles <= kPdlMaxBlocks ? 1 : 0;
            const cudaError_t e = cudaLaunchKernelEx(&cfg, k_smooth_block<T, W>, counted(L, fam), b, x, y, omega, inner,
                                                     sc, gate);
            if (e != cudaSuccess) throw std::runtime_error(std::string("block sweep launch: ") + cudaGetErrorString(e));
        }));
        return;
    }
    PSGB_LAUNCH(fam, st, PSGB_MR_WIDTHS(L.width, launch_pdl(k_smooth<T, W>, L.tiles, kTile, st, counted(L, fam), b, x, y,
                                                            omega, sc, gate)));
}
template <typename T>
void Launch<T>::residual(const LevelView<T>& L, const T* b, const T* x, T* r, const InstanceScalars* sc, int gate,
                         cudaStream_t st) {
    const int fam = L.level == 0 ? kFamResidual : kFamResidualCoarse;
    PSGB_LAUNCH(fam, st, PSGB_MR_WIDTHS(L.width, launch_pdl(k_residual<T, W>, L.tiles, kTile, st, counted(L, fam), b, x,
                                                            r, sc, gate)));
}
template <typename T>
void Launch<T>::restrict_zero(const LevelView<T>& C, const std::uint32_t* moff, const std::uint32_t* member, const T* r,
                              T* bc, T* xc, T omega, const InstanceScalars* sc, int gate, cudaStream_t st) {
    const int fam = C.level <= 1 ? kFamRestrict : kFamRestrictCoarse;
    PSGB_LAUNCH(fam, st, launch_pdl(k_restrict_zero<T>, C.tiles, kTile, st, counted(C, fam), moff, member, r, bc, xc,
                                    omega, sc, gate));
}
template <typename T>
void Launch<T>::prolong_smooth(const LevelView<T>& L, const std::int32_t* agg, const T* e, const T* b, const T* x,
                               T* y, T omega, const InstanceScalars* sc, int gate, cudaStream_t st) {
    const int fam = L.level == 0 ? kFamSmooth : kFamSmoothCoarse;
    PSGB_LAUNCH(fam, st, PSGB_MR_WIDTHS(L.width, launch_pdl(k_prolong_smooth<T, W>, L.tiles, kTile, st, counted(L, fam),
                                                            agg, e, b, x, y, omega, sc, gate)));
}
template <typename T>
void Launch<T>::prolong(const LevelView<T>& L, const std::int32_t* agg, const T* xc, T* x, const InstanceScalars* sc,
                        int gate, cudaStream_t st) {
    const int fam = L.level == 0 ? kFamProlong : kFamProlongCoarse;
    PSGB_LAUNCH(fam, st, launch_pdl(k_prolong<T>, L.tiles, kTile, st, counted(L, fam), agg, xc, x, sc, gate));
}
template <typename T>
void Launch<T>::dense(int n, const T* inv, const T* b, T* x, const InstanceScalars* sc, int gate, cudaStream_t st) {
    PSGB_LAUNCH(kFamDense, st, launch_pdl(k_dense<T>, (n + 7) / 8, kTile, st, n, inv, b, x, sc, gate,
                                          profile_bytes_for(kFamDense)));
}
template <typename T>
void Launch<T>::bicg_init(const LevelView<T>& L, const T* b, T* x, T* r, T* shadow, T* p, T* v, const Ctx& ctx,
                          double tol, int max_it, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, launch_pdl(k_bicg_init<T>, L.tiles, kTile, st, counted(L, kFamKrylovVector), b, x,
                                                 r, shadow, p, v, ctx));
    finish<ph::kFinBicgInit>(ctx, L.tiles, kFamKrylovVector, st, ph::FinishParams{tol, max_it, 0, nullptr});
}
template <typename T>
void Launch<T>::bicg_p(const LevelView<T>& L, const T* r, const T* v, T* p, T* xv, T omega_j, const InstanceScalars* sc,
                       cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, launch_pdl(k_bicg_p<T>, L.tiles, kTile, st, counted(L, kFamKrylovVector), r, v, p,
                                                 xv, omega_j, sc));
}
template <typename T>
void Launch<T>::bicg_v(const LevelView<T>& L, const T* in, T* out, const T* shadow, const Ctx& ctx, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovSpmv, st, PSGB_MR_WIDTHS(L.width, launch_pdl(k_bicg_v<T, W>, L.tiles, kTile, st,
                                                                       counted(L, kFamKrylovSpmv), in, out, shadow, ctx)));
    finish<ph::kFinBicgV>(ctx, L.tiles, kFamKrylovSpmv, st);
}
template <typename T>
void Launch<T>::bicg_s(const LevelView<T>& L, const T* r, const T* v, T* s, T* xv, T omega_j, const Ctx& ctx,
                       cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, launch_pdl(k_bicg_s<T>, L.tiles, kTile, st, counted(L, kFamKrylovVector), r, v, s,
                                                 xv, omega_j, ctx));
    finish<ph::kFinBicgS>(ctx, L.tiles, kFamKrylovVector, st);
}
template <typename T>
void Launch<T>::bicg_t(const LevelView<T>& L, const T* shat, T* t, const T* s, const Ctx& ctx, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovSpmv, st, PSGB_MR_WIDTHS(L.width, launch_pdl(k_bicg_t<T, W>, L.tiles, kTile, st,
                                                                       counted(L, kFamKrylovSpmv), shat, t, s, ctx)));
    finish<ph::kFinBicgT>(ctx, L.tiles, kFamKrylovSpmv, st);
}
template <typename T>
void Launch<T>::bicg_x(const LevelView<T>& L, const T* phat, const T* shat, const T* s, const T* t, T* x, T* r,
                       const T* shadow, const Ctx& ctx, cudaStream_t st) {
    PSGB_LAUNCH(kFamKrylovVector, st, launch_pdl(k_bicg_x<T>, L.tiles, kTile, st, counted(L, kFamKrylovVector), phat,
                                                 shat, s, t, x, r, shadow, ctx));
    finish<ph::kFinBicgX>(ctx, L.tiles, kFamKrylovVector, st);
}

void outer_init(const LevelView<double>& L, const double* b, const Ctx& ctx, double tol, int max_refine,
                cudaStream_t st) {
    PSGB_LAUNCH(kFamRefine, st, launch_pdl(k_outer_init, L.tiles, kTile, st, counted(L, kFamRefine), b, ctx));
    finish<ph::kFinOuterInit>(ctx, L.tiles, kFamRefine, st, ph::FinishParams{tol, 0, max_refine, nullptr});
}

template <typename TI>
void outer_residual(const LevelView<double>& L, const double* b, const double* x, double* r64, TI* rin, const Ctx& ctx,
                    int max_refine, cudaStream_t st) {
    PSGB_LAUNCH(kFamRefine, st, PSGB_MR_WIDTHS(L.width, launch_pdl(k_outer_residual<TI, W>, L.tiles, kTile, st,
                                                                   counted(L, kFamRefine), b, x, r64, rin, ctx)));
    finish<ph::kFinOuterResidual>(ctx, L.tiles, kFamRefine, st, ph::FinishParams{0.0, 0, max_refine, nullptr});
}

template <typename TI>
void outer_update(const LevelView<double>& L, const TI* delta, double* x, InstanceScalars* sc, cudaStream_t st) {
    PSGB_LAUNCH(kFamRefine, st, launch_pdl(k_outer_account, 1, kRhs, st, sc));
    PSGB_LAUNCH(kFamRefine, st, launch_pdl(k_outer_update<TI>, L.tiles, kTile, st, counted(L, kFamRefine), delta, x, sc));
}

void load(std::uint32_t n, std::uint32_t P, int count, const double* const* t0, const double* const* src,
          const double* area, double slope, double* rhs, double* x0, cudaStream_t st) {
    const std::size_t total = std::size_t(P) * kRhs;
    PSGB_LAUNCH(kFamStep, st, (k_load<<<static_cast<unsigned>((total + 255) / 256), 256, 0, st>>>(n, P, count, t0, src,
                                                                                                  area, slope, rhs, x0)));
}

void take(std::uint32_t P, int j, const double* x, double* out, cudaStream_t st) {
    PSGB_LAUNCH(kFamStep, st, (k_take<<<(P + 255) / 256, 256, 0, st>>>(P, j, x, out)));
}

template struct Launch<float>;
template struct Launch<double>;
template void outer_residual<float>(const LevelView<double>&, const double*, const double*, double*, float*, const Ctx&,
                                    int, cudaStream_t);
template void outer_residual<double>(const LevelView<double>&, const double*, const double*, double*, double*,
                                     const Ctx&, int, cudaStream_t);
template void outer_update<float>(const LevelView<double>&, const float*, double*, InstanceScalars*, cudaStream_t);
template void outer_update<double>(const LevelView<double>&, const double*, double*, InstanceScalars*, cudaStream_t);

}  // namespace mr
}  // namespace psgb

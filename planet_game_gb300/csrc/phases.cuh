// Per-tile phases of the solve, shared by the one-kernel-per-phase path (multigrid.cu,
// krylov.cu) and the persistent solver (persistent.cu), so both compute every row and
// every reduction with the same arithmetic in the same order.
//
// A "group" is 256 consecutive threads of a block. A phase call works on a tile set: R
// consecutive 256-row tiles starting at t0 (a multiple of R), lane l of the group owning
// row l of each of them. The R rows of a thread are independent, so their loads are in
// flight together; tiles past the end of the level take part in no store. Per tile, the
// arithmetic and every reduction tree are those of one tile alone: a dot product's tile
// partial is the same 256-row tree whatever R is, so results do not depend on R.
//
// Loads may run through rows that store nothing (padding rows, tiles of a planet that is
// masked out, a tile set's tail past the level): every such row indexes valid memory
// (padded rows point at themselves in `col`, at coarse row 0 in `agg`, and own an empty
// member range), and only rows of open tiles are stored.
//
// Groups synchronise with named barriers (id 1 + group), never with __syncthreads, so the
// groups of a block can work on different tile sets independently.
#pragma once

#include "common.cuh"
#include "kernels.hpp"
#include "profile.hpp"

#include <stdexcept>

// Vectors a phase reads were written by an earlier phase. A kernel per phase may read
// them through the read-only (non-coherent) path; the persistent solver, where earlier
// phases ran in the same kernel, must not: it defines PSGB_PHASE_RESTRICT empty.
#ifndef PSGB_PHASE_RESTRICT
#define PSGB_PHASE_RESTRICT __restrict__
#endif

namespace psgb {
namespace ph {

constexpr int kGroups = 4;   // groups per block at most (1024 threads)

// Tiles per tile set (rows per thread) of the kernel path's launches.
constexpr int kRowsStencil = 2;   // smoothing, residual, prolongation, Krylov products
constexpr int kRowsVector = 4;    // vector updates and their dot products
constexpr int kRowsCoarse = 1;    // restriction (a member loop per row)

__host__ __device__ constexpr unsigned tile_sets(unsigned tiles, int rows) { return (tiles + rows - 1) / rows; }

// Host dispatch on a level's tile-set sizes and ELL width (R and W constexpr in the body).
#define PSGB_STENCIL_SETS(sets, ...)                                           \
    switch (sets) {                                                            \
        case 1: { constexpr int R = 1; __VA_ARGS__; } break;                   \
        case 2: { constexpr int R = 2; __VA_ARGS__; } break;                   \
        default: throw std::logic_error("unsupported stencil tile-set size");  \
    }
#define PSGB_VECTOR_SETS(sets, ...)                                            \
    switch (sets) {                                                            \
        case 1: { constexpr int R = 1; __VA_ARGS__; } break;                   \
        case 4: { constexpr int R = 4; __VA_ARGS__; } break;                   \
        default: throw std::logic_error("unsupported vector tile-set size");   \
    }
#define PSGB_WIDTHS(width, ...)                                                \
    switch (width) {                                                           \
        case 6: { constexpr int W = 6; __VA_ARGS__; } break;                   \
        case 8: { constexpr int W = 8; __VA_ARGS__; } break;                   \
        case 12: { constexpr int W = 12; __VA_ARGS__; } break;                 \
        case 16: { constexpr int W = 16; __VA_ARGS__; } break;                 \
        default: throw std::logic_error("unsupported ELL width");              \
    }

__device__ __forceinline__ void group_sync(int gid) {
    asm volatile("bar.sync %0, 256;" ::"r"(gid + 1) : "memory");
}

__device__ __forceinline__ void count_bytes(unsigned long long* counter, int lane, unsigned long long bytes) {
    if (counter != nullptr && lane == 0 && bytes != 0) atomicAdd(counter, bytes);
}

// A per-thread byte count summed over each warp (every lane of the warp calls it).
__device__ __forceinline__ void count_bytes_warp(unsigned long long* counter, unsigned bytes) {
    if (counter == nullptr) return;
    const unsigned s = __reduce_add_sync(0xffffffffu, bytes);
    if ((threadIdx.x & 31) == 0 && s != 0) atomicAdd(counter, static_cast<unsigned long long>(s));
}

// The view of one launch: its family's byte counter while a profile of it records.
template <typename T>
inline LevelView<T> counted(const LevelView<T>& lv, int family) {
    LevelView<T> v = lv;
    v.bytes = profile_bytes_for(family);
    return v;
}

// The warp sums of N values (N a power of two, at most 32) by recursive halving: at the
// exchanges with lane offsets 16, 8, ... while a lane holds several values, the lanes with
// that offset bit clear keep the first half of their values and the others the second
// half, each adding its partner's copy of what it keeps; once one value is left, plain
// butterfly steps. Every value is combined with the same partner at every step as in a
// butterfly of its own (warp_sum), so each total has warp_sum's bits, for N values at the
// cost of about N - 1 + log2(32 / N) additions a lane instead of 5 N. On return `mine` is
// the total of value `q`; `owner` is true in the lowest lane holding it.
template <typename A, int N>
__device__ __forceinline__ void warp_sum_halving(const A (&v)[N], int l32, A& mine, int& q, bool& owner) {
    static_assert(N >= 1 && N <= 32 && (N & (N - 1)) == 0, "a power of two, at most 32");
    A cur[N];
#pragma unroll
    for (int i = 0; i < N; ++i) cur[i] = v[i];
    int held = 0;        // index of the first value this lane holds
    unsigned mask = 0;   // lane bits that chose a half
#pragma unroll
    for (int step = 0; step < 5; ++step) {
        const int o = 16 >> step;
        const int m = (N >> step) > 1 ? (N >> step) : 1;   // values held before this step
        if (m > 1) {
            const int h = m / 2;
            const bool upper = (l32 & o) != 0;
#pragma unroll
            for (int i = 0; i < h; ++i) {
                const A send = upper ? cur[i] : cur[h + i];
                const A keep = upper ? cur[h + i] : cur[i];
                cur[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
            }
            if (upper) held += h;
            mask |= static_cast<unsigned>(o);
        } else {
            cur[0] += __shfl_xor_sync(0xffffffffu, cur[0], o);
        }
    }
    mine = cur[0];
    q = held;
    owner = (static_cast<unsigned>(l32) & ~mask) == 0u;
}

// Sum of N values over the 256 threads of a group, each value in its own fixed tree
// (warp butterflies, then the eight warp sums in order); results in lane 0.
template <typename A, int N>
__device__ __forceinline__ void group_sum(A (&v)[N], int gid, int lane) {
    __shared__ A scratch[kGroups][N][8];
    const int w = lane >> 5;
    if constexpr (N == 1 || N == 2 || N == 4 || N == 8) {
        A mine;
        int q;
        bool owner;
        warp_sum_halving<A, N>(v, lane & 31, mine, q, owner);
        if (owner) scratch[gid][q][w] = mine;
    } else {
#pragma unroll
        for (int q = 0; q < N; ++q) {
            const A s = warp_sum(v[q]);
            if ((lane & 31) == 0) scratch[gid][q][w] = s;
        }
    }
    group_sync(gid);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < N; ++q) {
            A s = scratch[gid][q][0];
#pragma unroll
            for (int k = 1; k < 8; ++k) s += scratch[gid][q][k];
            v[q] = s;
        }
    }
    group_sync(gid);
}

// ---- tile sets ----------------------------------------------------------------------------

template <int R>
struct TileSet {
    int tile[R];     // tile index (t0 for a tile past the level: loads stay in bounds)
    int inst[R];     // planet
    int rows[R];     // valid rows (0 past the level)
    bool sweep[R];   // the planet smooths on this level
};

template <int R>
__device__ __forceinline__ TileSet<R> tile_set(const std::uint32_t* meta, unsigned tiles, int t0) {
    std::uint32_t w[R];
    if constexpr (R == 4) {
        const uint4 v = *reinterpret_cast<const uint4*>(meta + t0);
        w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
    } else if constexpr (R == 2) {
        const uint2 v = *reinterpret_cast<const uint2*>(meta + t0);
        w[0] = v.x; w[1] = v.y;
    } else {
#pragma unroll
        for (int k = 0; k < R; ++k) w[k] = meta[t0 + k];
    }
    TileSet<R> s;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const bool valid = static_cast<unsigned>(t0 + k) < tiles;
        s.tile[k] = valid ? t0 + k : t0;
        s.inst[k] = static_cast<int>(w[k] & 0x3FFFFFu);
        s.rows[k] = valid ? static_cast<int>((w[k] >> 22) & 0x1FFu) : 0;
        s.sweep[k] = valid && (w[k] >> 31) != 0u;
    }
    return s;
}

// The ELL columns of one row: column j is `add + p[j * stride]`. A level without shared
// columns reads its own (add 0); a level whose planets share their graph's planet-local
// columns reads those and adds the planet's first row (the tile's shift), which gives the
// same row indices.
struct ColumnsOf {
    const std::int32_t* p;
    int stride;
    int add;
    __device__ __forceinline__ int operator[](int j) const { return add + p[j * stride]; }
};
template <typename T>
__device__ __forceinline__ ColumnsOf columns_of(const LevelView<T>& lv, int tile, int row) {
    if (lv.scol != nullptr) {
        const int2 sh = lv.tile_shift[tile];
        return ColumnsOf{lv.scol + (row - sh.y), static_cast<int>(lv.spitch), sh.x};
    }
    return ColumnsOf{lv.col + row, static_cast<int>(lv.rows), 0};
}
// Column-index bytes a row reads from HBM: none where the columns are shared (one small
// copy per graph, which stays in L2).
template <typename T>
__device__ __forceinline__ unsigned long long col_bytes(const LevelView<T>& lv, int W) {
    return lv.scol != nullptr ? 0ull : 4ull * static_cast<unsigned>(W);
}

// ---- before griddepcontrol.wait --------------------------------------------------------
// A launch scheduled early (programmatic dependent launch) waits for its predecessor in
// pdl_begin(). Before that it may touch only what nothing writes once the batch is built -
// tile words, ELL columns, aggregates, restriction lists, dense-block tables - and these
// prefetches bring the lines a phase reads first into L1 there, so two dependent loads of
// the phase's chain (tile word, then column) hit L1 after the wait. Never a value or a
// vector: those are written by the solve's or the assembly's kernels, and an L1 line
// fetched before the wait could be stale after it.
__device__ __forceinline__ void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

template <typename T>
__device__ __forceinline__ void prefetch_meta(const LevelView<T>& lv, int t0, int lane) {
    if (lane == 0 && static_cast<unsigned>(t0) < lv.tiles) prefetch_l1(lv.tile_meta + t0);
}

template <typename T, int W, int R>
__device__ __forceinline__ void prefetch_static(const LevelView<T>& lv, int t0, int lane) {
    if (static_cast<unsigned>(t0) >= lv.tiles) return;
    if (lane == 0) prefetch_l1(lv.tile_meta + t0);
    if (lv.scol != nullptr) return;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int tile = t0 + k;
        if (static_cast<unsigned>(tile) >= lv.tiles) break;
        const int row = tile * kTile + lane;
#pragma unroll
        for (int j = 0; j < W; ++j) prefetch_l1(lv.col + static_cast<std::size_t>(j) * lv.rows + row);
    }
}

// Algorithmic bytes of the open tiles of a tile set: `per_row` times their valid rows.
template <int R>
__device__ __forceinline__ void count_rows(unsigned long long* counter, int lane, const TileSet<R>& ts,
                                           const bool (&on)[R], unsigned long long per_row) {
    if (counter == nullptr || lane != 0) return;
    unsigned long long rows = 0;
#pragma unroll
    for (int k = 0; k < R; ++k) rows += on[k] ? static_cast<unsigned long long>(ts.rows[k]) : 0ull;
    if (rows != 0) atomicAdd(counter, rows * per_row);
}

template <int R>
__device__ __forceinline__ bool any_of(const bool (&on)[R]) {
    bool a = false;
#pragma unroll
    for (int k = 0; k < R; ++k) a = a || on[k];
    return a;
}

__device__ __forceinline__ bool gate_open(const InstanceScalars* sc, int inst, int gate) {
    if (gate == kGateAlways) return true;
    const InstanceScalars& s = sc[inst];
    if (gate == kGateOuter) return s.outer_status == kRunning;
    if (s.status != kRunning) return false;
    if (gate == kGateSecondHalf && s.half_done) return false;
    return true;
}

__device__ __forceinline__ bool running(const InstanceScalars& s) { return s.status == kRunning; }

// A dot-product term, rounded on its own (never fused into the reduction's first add), so
// that every layout that sums the same terms in the same tree gets the same bits.
__device__ __forceinline__ float prod(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double prod(double a, double b) { return __dmul_rn(a, b); }

// The block-local sweep's arithmetic spelled out, so that every kernel sweeping a tile
// block-locally (the kernel schedule, the coarse tails, the block step of many right-hand
// sides) forms the same bits whatever the compiler would fuse: s - a v as one fused
// multiply-add, and the damped update as the product inv s and its difference with xo
// each rounded, then xo + omega d as one fused multiply-add.
__device__ __forceinline__ float fnma(float a, float v, float s) { return __fmaf_rn(-a, v, s); }
__device__ __forceinline__ double fnma(double a, double v, double s) { return __fma_rn(-a, v, s); }
__device__ __forceinline__ float jacobi_update(float xo, float omega, float inv, float s) {
    return omega == 1.0f ? __fmul_rn(inv, s) : __fmaf_rn(omega, __fsub_rn(__fmul_rn(inv, s), xo), xo);
}
__device__ __forceinline__ double jacobi_update(double xo, double omega, double inv, double s) {
    return omega == 1.0 ? __dmul_rn(inv, s) : __fma_rn(omega, __dsub_rn(__dmul_rn(inv, s), xo), xo);
}

__device__ __forceinline__ bool finite(double v) { return isfinite(v); }

// Release/acquire fence at GPU scope: orders this thread's partial stores before its
// ticket, and the finaliser's ticket observation before its partial loads. Lighter than
// the sequentially consistent __threadfence(), which the reduction does not need.
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// How a reduction phase completes its planets' sums.
//   kTicket:   after writing its tile partials, a tile set takes one ticket per run of
//              its tiles that belong to one planet (release fence, integer atomic); the
//              last tile set of a planet to arrive sums that planet's partials and
//              performs the scalar step (the persistent solver: no launch boundary follows).
//   kDeferred: tile sets only write their partials; a finish launch per planet sums them
//              and performs the same step (the kernel schedule: no block waits on a ticket).
// Both sum a planet's partials with sum_partials, so both give the same bits.
enum Completion : int { kTicket = 0, kDeferred = 1 };

// A planet's tile partials in tile order: lane l sums tiles begin + l, + 256, ... (four
// loads in flight at a time), then the group's fixed tree; result in lane 0.
template <int NQ>
__device__ __forceinline__ void sum_partials(const ReduceCtx& ctx, unsigned begin, unsigned end, int gid, int lane,
                                             double (&acc)[NQ]) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] = 0.0;
    for (unsigned t0 = begin + lane; t0 < end; t0 += 4 * kTile) {
        double p[4][NQ];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const unsigned t = t0 + u * kTile;
#pragma unroll
            for (int q = 0; q < NQ; ++q) p[u][q] = t < end ? __ldcg(&ctx.partial[t * 8 + q]) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (t0 + u * kTile < end) {
#pragma unroll
                for (int q = 0; q < NQ; ++q) acc[q] += p[u][q];
            }
        }
    }
    group_sum<double, NQ>(acc, gid, lane);
}

template <int NQ>
__device__ __forceinline__ void sum_partials(const ReduceCtx& ctx, int inst, int gid, int lane, double (&acc)[NQ]) {
    sum_partials<NQ>(ctx, ctx.tile_begin[inst], ctx.tile_begin[inst + 1], gid, lane, acc);
}

// Tile partial sums (in the tiles' precision A) to FP64 partials, then completion C.
// fin[k]: (kTicket only) lane 0 holds planet inst[k]'s sums in out[k * NQ + q].
template <typename A, int NQ, int R, int C>
__device__ void tiles_reduce(A (&v)[R * NQ], const ReduceCtx& ctx, const TileSet<R>& ts, const bool (&on)[R],
                             double (&out)[R * NQ], bool (&fin)[R], int gid, int lane) {
    __shared__ int last[kGroups][R];
    group_sum<A, R * NQ>(v, gid, lane);
#pragma unroll
    for (int k = 0; k < R; ++k) fin[k] = false;
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < R; ++k) {
            if (!on[k]) continue;
#pragma unroll
            for (int q = 0; q < NQ; ++q) ctx.partial[ts.tile[k] * 8 + q] = static_cast<double>(v[k * NQ + q]);
        }
    }
    if constexpr (C == kDeferred) {
        return;
    } else {
        if (lane == 0) {
            fence_acq_rel_gpu();
            bool any_last = false;
#pragma unroll
            for (int k = 0; k < R; ++k) last[gid][k] = 0;
            for (int k = 0; k < R;) {
                if (!on[k]) { ++k; continue; }
                int e = k + 1;
                while (e < R && on[e] && ts.inst[e] == ts.inst[k]) ++e;
                const int inst = ts.inst[k];
                const unsigned n = ctx.tile_begin[inst + 1] - ctx.tile_begin[inst];
                const unsigned add = static_cast<unsigned>(e - k);
                const unsigned old = atomicAdd(&ctx.ticket[inst], add);
                last[gid][k] = (old + add == n) ? 1 : 0;
                any_last = any_last || old + add == n;
                k = e;
            }
            if (any_last) fence_acq_rel_gpu();   // acquire: the other tile sets' partials
        }
        group_sync(gid);
#pragma unroll
        for (int k = 0; k < R; ++k) {
            if (!last[gid][k]) continue;
            double acc[NQ];
            sum_partials<NQ>(ctx, ts.inst[k], gid, lane, acc);
            if (lane == 0) {
                ctx.ticket[ts.inst[k]] = 0;
#pragma unroll
                for (int q = 0; q < NQ; ++q) out[k * NQ + q] = acc[q];
                fin[k] = true;
            }
        }
    }
}

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

// Zero-start sweep: x = omega D^-1 b.
template <typename T, int R>
__device__ void smooth_zero(const LevelView<T>& lv, int t0, int lane, const T* PSGB_PHASE_RESTRICT b,
                            T* PSGB_PHASE_RESTRICT x, T omega, const InstanceScalars* sc, int gate) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.sweep[k] && gate_open(sc, ts.inst[k], gate);
    if (!any_of(on)) return;
    T y[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int row = ts.tile[k] * kTile + lane;
        y[k] = omega * lv.inv[row] * b[row];
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (!on[k]) continue;
        count_bytes(lv.bytes, lane, static_cast<unsigned long long>(ts.rows[k]) * 3ull * sizeof(T));
        if (lane < ts.rows[k]) x[ts.tile[k] * kTile + lane] = y[k];
    }
}

// Damped Jacobi sweep: y = x + omega (D^-1 (b - O x) - x); undamped (omega = 1, a
// uniform branch) y = D^-1 (b - O x), which neither reads x at the row nor spends the two
// FP64 operations of the damping.
template <typename T, int W, int R>
__device__ void smooth(const LevelView<T>& lv, int t0, int lane, const T* PSGB_PHASE_RESTRICT b,
                       const T* PSGB_PHASE_RESTRICT x, T* PSGB_PHASE_RESTRICT y, T omega, const InstanceScalars* sc,
                       int gate) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.sweep[k] && gate_open(sc, ts.inst[k], gate);
    if (!any_of(on)) return;
    const std::uint32_t P = lv.rows;
    T out[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int row = ts.tile[k] * kTile + lane;
        const ColumnsOf col = columns_of(lv, ts.tile[k], row);
        T s = b[row];
#pragma unroll
        for (int j = 0; j < W; ++j) s -= lv.vd[j * P + row] * x[col[j]];
        if (omega == T(1)) {
            out[k] = lv.inv[row] * s;
        } else {
            const T xo = x[row];
            out[k] = xo + omega * (lv.inv[row] * s - xo);
        }
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (!on[k]) continue;
        count_bytes(lv.bytes, lane, static_cast<unsigned long long>(ts.rows[k]) * (col_bytes(lv, W) + sizeof(T) * (W + 4ull)));
        if (lane < ts.rows[k]) y[ts.tile[k] * kTile + lane] = out[k];
    }
}

// Block-local Jacobi: `inner` damped sweeps of one tile in one call, the tile's own rows
// updated in shared memory between sweeps and its neighbours in other tiles held at x
// (loaded once). One inner sweep is exactly `smooth` (same terms, same order). Several
// smooth the tile's error like that many sweeps at the cost of one pass over HBM; the
// error between tiles is left to the next launch or the coarser levels. The tile-level
// counterpart of the reference's block-hybrid smoother (heat_transport.cpp:258-286), with
// Jacobi instead of sequential Gauss-Seidel inside the block.
// The block-local sweeps' tiles, one per tile group: a single array per element type,
// whichever ELL widths a kernel instantiates the sweep for.
template <typename T>
__device__ __forceinline__ T (*tile_buffer())[kTile] {
    __shared__ T xs[kGroups][kTile];
    return xs;
}

template <typename T, int W>
__device__ void smooth_block(const LevelView<T>& lv, int tile, int gid, int lane, const T* PSGB_PHASE_RESTRICT b,
                             const T* PSGB_PHASE_RESTRICT x, T* PSGB_PHASE_RESTRICT y, T omega, int inner,
                             const InstanceScalars* sc, int gate) {
    T (*xs)[kTile] = tile_buffer<T>();
    const TileSet<1> ts = tile_set<1>(lv.tile_meta, lv.tiles, tile);
    if (!ts.sweep[0] || !gate_open(sc, ts.inst[0], gate)) return;
    const std::uint32_t P = lv.rows;
    const int row = ts.tile[0] * kTile + lane;
    const int first = ts.tile[0] * kTile;
    const bool live = lane < ts.rows[0];
    // the row's couplings: within the tile (index into xs) or frozen at x
    T a[W], h[W];
    int local[W];
    T bv = T(0), inv = T(0), xo = T(0);
    if (live) {
        const ColumnsOf col = columns_of(lv, ts.tile[0], row);
        bv = b[row];
        inv = lv.inv[row];
        xo = x[row];
#pragma unroll
        for (int j = 0; j < W; ++j) {
            const int c = col[j];
            a[j] = lv.vd[j * P + row];
            local[j] = (c >= first && c < first + kTile) ? c - first : -1;
            h[j] = local[j] < 0 ? x[c] : T(0);
        }
    }
    xs[gid][lane] = xo;
    group_sync(gid);
    for (int sweep = 0; sweep < inner; ++sweep) {
        T out = xo;
        if (live) {
            T s = bv;
#pragma unroll
            for (int j = 0; j < W; ++j) s = fnma(a[j], local[j] >= 0 ? xs[gid][local[j]] : h[j], s);
            out = jacobi_update(xo, omega, inv, s);
        }
        group_sync(gid);
        xs[gid][lane] = out;
        xo = out;
        group_sync(gid);
    }
    count_bytes(lv.bytes, lane, static_cast<unsigned long long>(ts.rows[0]) * (col_bytes(lv, W) + sizeof(T) * (W + 4ull)));
    if (live) y[row] = xo;
}

// r = b - A x
template <typename T, int W, int R>
__device__ void residual(const LevelView<T>& lv, int t0, int lane, const T* PSGB_PHASE_RESTRICT b,
                         const T* PSGB_PHASE_RESTRICT x, T* PSGB_PHASE_RESTRICT r, const InstanceScalars* sc, int gate) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.sweep[k] && gate_open(sc, ts.inst[k], gate);
    if (!any_of(on)) return;
    const std::uint32_t P = lv.rows;
    T out[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int row = ts.tile[k] * kTile + lane;
        const ColumnsOf col = columns_of(lv, ts.tile[k], row);
        T s = b[row] - lv.vd[W * P + row] * x[row];
#pragma unroll
        for (int j = 0; j < W; ++j) s -= lv.vd[j * P + row] * x[col[j]];
        out[k] = s;
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (!on[k]) continue;
        count_bytes(lv.bytes, lane, static_cast<unsigned long long>(ts.rows[k]) * (col_bytes(lv, W) + sizeof(T) * (W + 4ull)));
        if (lane < ts.rows[k]) r[ts.tile[k] * kTile + lane] = out[k];
    }
}

// y = A x for every planet
template <typename T, int W, int R>
__device__ void spmv(const LevelView<T>& lv, int t0, int lane, const T* PSGB_PHASE_RESTRICT x, T* PSGB_PHASE_RESTRICT y) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    const std::uint32_t P = lv.rows;
    T out[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int row = ts.tile[k] * kTile + lane;
        const ColumnsOf col = columns_of(lv, ts.tile[k], row);
        T s = lv.vd[W * P + row] * x[row];
#pragma unroll
        for (int j = 0; j < W; ++j) s += lv.vd[j * P + row] * x[col[j]];
        out[k] = s;
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        count_bytes(lv.bytes, lane, static_cast<unsigned long long>(ts.rows[k]) * (col_bytes(lv, W) + sizeof(T) * (W + 3ull)));
        if (lane < ts.rows[k]) y[ts.tile[k] * kTile + lane] = out[k];
    }
}

// Restriction fused with the coarse level's zero-start sweep: b_c = sum of the members'
// residuals in ascending fine-row order (the reference's order, heat_transport.cpp:316-319);
// x_c = omega b_c / diag where the planet smooths on the coarse level.
template <typename T, int R>
__device__ void restrict_zero(const LevelView<T>& coarse, int t0, int lane, const std::uint32_t* PSGB_PHASE_RESTRICT moff,
                              const std::uint32_t* PSGB_PHASE_RESTRICT member, const T* PSGB_PHASE_RESTRICT r,
                              T* PSGB_PHASE_RESTRICT bc, T* PSGB_PHASE_RESTRICT xc, T omega, const InstanceScalars* sc,
                              int gate) {
    const TileSet<R> ts = tile_set<R>(coarse.tile_meta, coarse.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.rows[k] > 0 && gate_open(sc, ts.inst[k], gate);
    if (!any_of(on)) return;
    unsigned moved = 0;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (!on[k] || lane >= ts.rows[k]) continue;
        const int row = ts.tile[k] * kTile + lane;
        const std::uint32_t k0 = moff[row], k1 = moff[row + 1];
        const T s = member_sum(member, k0, k1, r);
        bc[row] = s;
        if (ts.sweep[k]) xc[row] = omega * coarse.inv[row] * s;
        // offsets, members and their residuals, 1/diag, b_c and x_c
        moved += 4u + (k1 - k0) * (4u + static_cast<unsigned>(sizeof(T))) + 3u * static_cast<unsigned>(sizeof(T));
    }
    count_bytes_warp(coarse.bytes, moved);
}

template <typename T, int R>
__device__ void restrict_only(const LevelView<T>& coarse, int t0, int lane, const std::uint32_t* PSGB_PHASE_RESTRICT moff,
                              const std::uint32_t* PSGB_PHASE_RESTRICT member, const T* PSGB_PHASE_RESTRICT r,
                              T* PSGB_PHASE_RESTRICT bc, const InstanceScalars* sc, int gate) {
    const TileSet<R> ts = tile_set<R>(coarse.tile_meta, coarse.tiles, t0);
    unsigned moved = 0;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (lane >= ts.rows[k] || !gate_open(sc, ts.inst[k], gate)) continue;
        const int row = ts.tile[k] * kTile + lane;
        const std::uint32_t k0 = moff[row], k1 = moff[row + 1];
        bc[row] = member_sum(member, k0, k1, r);
        moved += 4u + (k1 - k0) * (4u + static_cast<unsigned>(sizeof(T))) + static_cast<unsigned>(sizeof(T));
    }
    count_bytes_warp(coarse.bytes, moved);
}

// Prolongation fused with the first post-smoothing sweep: with x' = x + e[agg] (formed on
// the fly for the row and its neighbours), y = x' + omega (D^-1 (b - O x') - x').
template <typename T, int W, int R>
__device__ void prolong_smooth(const LevelView<T>& lv, int t0, int lane, const std::int32_t* PSGB_PHASE_RESTRICT agg,
                               const T* PSGB_PHASE_RESTRICT e, const T* PSGB_PHASE_RESTRICT b, const T* PSGB_PHASE_RESTRICT x,
                               T* PSGB_PHASE_RESTRICT y, T omega, const InstanceScalars* sc, int gate) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.sweep[k] && gate_open(sc, ts.inst[k], gate);
    if (!any_of(on)) return;
    const std::uint32_t P = lv.rows;
    T out[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int row = ts.tile[k] * kTile + lane;
        const ColumnsOf col = columns_of(lv, ts.tile[k], row);
        T s = b[row];
#pragma unroll
        for (int j = 0; j < W; ++j) {
            const int c = col[j];
            s -= lv.vd[j * P + row] * (x[c] + prod(lv.correction, e[agg[c]]));
        }
        if (omega == T(1)) {
            out[k] = lv.inv[row] * s;
        } else {
            const T xo = x[row] + prod(lv.correction, e[agg[row]]);
            out[k] = xo + omega * (lv.inv[row] * s - xo);
        }
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (!on[k]) continue;
        // each vector once: col, values, inv, b, x, y and the row's aggregate index (the
        // neighbours' x and agg are gathers of vectors already counted; e is 1/16 of a row)
        count_bytes(lv.bytes, lane, static_cast<unsigned long long>(ts.rows[k]) * (col_bytes(lv, W) + sizeof(T) * (W + 4ull) + 4ull));
        if (lane < ts.rows[k]) y[ts.tile[k] * kTile + lane] = out[k];
    }
}

template <typename T, int R>
__device__ void prolong(const LevelView<T>& lv, int t0, int lane, const std::int32_t* PSGB_PHASE_RESTRICT agg,
                        const T* PSGB_PHASE_RESTRICT xc, T* PSGB_PHASE_RESTRICT x, const InstanceScalars* sc, int gate) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (!ts.sweep[k] || !gate_open(sc, ts.inst[k], gate)) continue;
        // agg, x read and written (the coarse correction is 1/16 of a row)
        count_bytes(lv.bytes, lane, static_cast<unsigned long long>(ts.rows[k]) * (4ull + 2ull * sizeof(T)));
        if (lane >= ts.rows[k]) continue;
        const int row = ts.tile[k] * kTile + lane;
        x[row] += prod(lv.correction, xc[agg[row]]);
    }
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
    // the inverse's row and the solution's entry (b is read from cache by every row)
    if (task.bytes != nullptr && (lane & 31) == 0)
        atomicAdd(task.bytes, static_cast<unsigned long long>(task.dense.size[blk.x] + 1) * sizeof(T));
}

// ---- scalar steps: one planet, once its sums are complete (ticket or finish launch) ----

__device__ inline void finish_bicg_init(InstanceScalars& s, const double* sum, double tol, int max_it) {
    s.b_norm = sqrt(sum[0]);
    s.target = fmax(tol * s.b_norm, 0.5 * s.outer_target);
    s.rho = sum[0]; s.alpha = 1.0; s.omega = 1.0; s.beta = 0.0;
    s.iterations = 0; s.half_done = 0; s.max_iterations = max_it; s.first = 1;
    s.r_norm = s.b_norm;
    s.status = !finite(s.b_norm) ? kNonFinite : (s.b_norm > 0.0 ? kRunning : kConverged);
}

// alpha = rho / (shadow . v)
__device__ inline void finish_bicg_v(InstanceScalars& s, const double* sum) {
    if (!finite(sum[0])) { s.status = kNonFinite; return; }
    if (sum[0] == 0.0) { s.status = kBreakdown; return; }
    s.alpha = s.rho / sum[0];
}

// ||s||: converged at s -> the iteration finishes with x += alpha p_hat.
__device__ inline void finish_bicg_s(InstanceScalars& s, const double* sum) {
    s.s_norm = sqrt(sum[0]);
    s.iterations += 1;
    if (!finite(s.s_norm)) { s.status = kNonFinite; return; }
    if (s.s_norm <= s.target) s.half_done = 1;
}

// omega = (t.s) / (t.t)
__device__ inline void finish_bicg_t(InstanceScalars& s, const double* sum) {
    s.omega = sum[0] > 0.0 ? sum[1] / sum[0] : 0.0;
    if (!finite(s.omega)) s.status = kNonFinite;
}

// ||r||, rho_next = shadow . r -> beta; a planet converged at s closes its iteration.
__device__ inline void finish_bicg_x(InstanceScalars& s, const double* sum) {
    if (s.half_done) {
        s.r_norm = s.s_norm;
        s.half_done = 0;
        s.status = kConverged;
        return;
    }
    s.r_norm = sqrt(sum[0]);
    if (!finite(s.r_norm)) { s.status = kNonFinite; return; }
    if (s.r_norm <= s.target) { s.status = kConverged; return; }
    const double rho_next = sum[1];
    if (rho_next == 0.0 || s.omega == 0.0) { s.status = kBreakdown; return; }
    s.beta = rho_next / s.rho * (s.alpha / s.omega);
    s.rho = rho_next;
    if (s.iterations >= s.max_iterations) s.status = kCap;
}

__device__ inline void finish_pcg_init(InstanceScalars& s, const double* sum, double tol, int max_it) {
    s.b_norm = sqrt(sum[0]);
    s.target = fmax(tol * s.b_norm, 0.5 * s.outer_target);
    s.r_norm = s.b_norm;
    s.iterations = 0; s.half_done = 0; s.max_iterations = max_it; s.first = 1;
    s.rho = 0.0; s.beta = 0.0; s.alpha = 0.0;
    s.status = !finite(s.b_norm) ? kNonFinite : (s.b_norm > 0.0 ? kRunning : kConverged);
}

// rho = r.z, beta = rho / rho_old
__device__ inline void finish_pcg_rz(InstanceScalars& s, const double* sum) {
    if (!finite(sum[0])) { s.status = kNonFinite; return; }
    if (!(sum[0] > 0.0)) { s.status = s.first ? kConverged : kBreakdown; return; }
    s.beta = s.first ? 0.0 : sum[0] / s.rho;
    s.rho = sum[0];
    s.first = 0;
}

// alpha = rho / p.q
__device__ inline void finish_pcg_q(InstanceScalars& s, const double* sum) {
    if (!finite(sum[0])) { s.status = kNonFinite; return; }
    if (!(sum[0] > 0.0)) { s.status = kBreakdown; return; }
    s.alpha = s.rho / sum[0];
}

// ||r|| -> converged?
__device__ inline void finish_pcg_xr(InstanceScalars& s, const double* sum) {
    s.r_norm = sqrt(sum[0]);
    s.iterations += 1;
    if (!finite(s.r_norm)) { s.status = kNonFinite; return; }
    if (s.r_norm <= s.target) { s.status = kConverged; return; }
    if (s.iterations >= s.max_iterations) s.status = kCap;
}

__device__ inline void finish_outer_init(InstanceScalars& s, const double* sum, double tol) {
    s.outer_b_norm = sqrt(sum[0]);
    s.outer_target = tol * s.outer_b_norm;
    s.tolerance = tol;
    s.refinements = 0;
    s.inner_total = 0;
    s.outer_status = !finite(s.outer_b_norm) ? kNonFinite : kRunning;
    s.status = kConverged;   // no inner solve runs until an inner init starts one
}

// ||b - A x|| in FP64 decides: converged, capped, or one more refinement.
__device__ inline void finish_outer_residual(InstanceScalars& s, const double* sum, int max_refine) {
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

// ---- finish launches of the kernel schedule (kDeferred) --------------------------------------

enum FinishKind : int {
    kFinBicgInit, kFinBicgV, kFinBicgS, kFinBicgT, kFinBicgX,
    kFinPcgInit, kFinPcgRz, kFinPcgQ, kFinPcgXr,
    kFinOuterInit, kFinOuterResidual,
};

struct FinishParams {
    double tol;
    int max_it;
    int max_refine;
    const std::uint8_t* active;
};

template <int K>
struct FinishSums {
    static constexpr int value = (K == kFinBicgT || K == kFinBicgX) ? 2 : 1;
};

// The planets whose tiles took part in the reduction: the phase's own gate.
template <int K>
__device__ __forceinline__ bool finish_gate(const InstanceScalars& s, int inst, const FinishParams& p) {
    if constexpr (K == kFinBicgInit || K == kFinPcgInit || K == kFinOuterResidual) return s.outer_status == kRunning;
    else if constexpr (K == kFinOuterInit) return p.active == nullptr || p.active[inst] != 0;
    else if constexpr (K == kFinBicgT) return s.status == kRunning && !s.half_done;
    else return s.status == kRunning;
}

template <int K>
__device__ __forceinline__ void finish_step(InstanceScalars& s, const double* sum, const FinishParams& p) {
    if constexpr (K == kFinBicgInit) finish_bicg_init(s, sum, p.tol, p.max_it);
    else if constexpr (K == kFinBicgV) finish_bicg_v(s, sum);
    else if constexpr (K == kFinBicgS) finish_bicg_s(s, sum);
    else if constexpr (K == kFinBicgT) finish_bicg_t(s, sum);
    else if constexpr (K == kFinBicgX) finish_bicg_x(s, sum);
    else if constexpr (K == kFinPcgInit) finish_pcg_init(s, sum, p.tol, p.max_it);
    else if constexpr (K == kFinPcgRz) finish_pcg_rz(s, sum);
    else if constexpr (K == kFinPcgQ) finish_pcg_q(s, sum);
    else if constexpr (K == kFinPcgXr) finish_pcg_xr(s, sum);
    else if constexpr (K == kFinOuterInit) finish_outer_init(s, sum, p.tol);
    else finish_outer_residual(s, sum, p.max_refine);
}

// One planet per 256-thread block: its partials in tile order, then its scalar step. The
// planet's tile range [begin, end) is fixed when the batch is built (the finish launch
// reads it before its programmatic-launch wait); the partials are summed whether or not
// the planet took part, so that their loads need not wait for its status word.
template <int K>
__device__ void finish_planet(const ReduceCtx& ctx, int inst, int lane, const FinishParams& p, unsigned begin,
                              unsigned end) {
    const bool open = finish_gate<K>(ctx.sc[inst], inst, p);
    double acc[FinishSums<K>::value];
    sum_partials(ctx, begin, end, 0, lane, acc);
    if (open && lane == 0) finish_step<K>(ctx.sc[inst], acc, p);
}

// ---- Krylov phases (fine level) ----------------------------------------------------------

template <typename T, int R, int C = kTicket>
__device__ void bicg_init(const LevelView<T>& lv, int t0, int gid, int lane, const T* PSGB_PHASE_RESTRICT b, T* x, T* r,
                          T* shadow, T* p, T* v, const ReduceCtx& ctx, double tol, int max_it) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.rows[k] > 0 && ctx.sc[ts.inst[k]].outer_status == kRunning;
    if (!any_of(on)) return;
    count_rows<R>(lv.bytes, lane, ts, on, 6ull * sizeof(T));
    T q[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        q[k] = T(0);
        if (!on[k] || lane >= ts.rows[k]) continue;
        const int row = ts.tile[k] * kTile + lane;
        const T bv = b[row];
        x[row] = T(0); r[row] = bv; shadow[row] = bv; p[row] = T(0); v[row] = T(0);
        q[k] = prod(bv, bv);
    }
    double out[R];
    bool fin[R];
    tiles_reduce<T, 1, R, C>(q, ctx, ts, on, out, fin, gid, lane);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (fin[k]) finish_bicg_init(ctx.sc[ts.inst[k]], &out[k], tol, max_it);
    }
}

// p = r + beta (p - omega v); first smoothing sweep of M p from zero.
template <typename T, int R>
__device__ void bicg_p(const LevelView<T>& lv, int t0, int lane, const T* PSGB_PHASE_RESTRICT r, const T* PSGB_PHASE_RESTRICT v,
                       T* p, T* xv, T omega_j, const InstanceScalars* sc) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.rows[k] > 0 && running(sc[ts.inst[k]]);
    if (!any_of(on)) return;
    count_rows<R>(lv.bytes, lane, ts, on, 6ull * sizeof(T));
    T pv[R], zv[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int row = ts.tile[k] * kTile + lane;
        const T beta = T(sc[ts.inst[k]].beta), omega = T(sc[ts.inst[k]].omega);
        pv[k] = r[row] + beta * (p[row] - omega * v[row]);
        zv[k] = omega_j * lv.inv[row] * pv[k];
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (!on[k] || lane >= ts.rows[k]) continue;
        const int row = ts.tile[k] * kTile + lane;
        p[row] = pv[k];
        if (ts.sweep[k]) xv[row] = zv[k];
    }
}

// out = A in; dot(shadow, out) -> alpha = rho / (shadow . v)
template <typename T, int W, int R, int C = kTicket>
__device__ void bicg_v(const LevelView<T>& lv, int t0, int gid, int lane, const T* PSGB_PHASE_RESTRICT in,
                       T* PSGB_PHASE_RESTRICT out, const T* PSGB_PHASE_RESTRICT shadow, const ReduceCtx& ctx) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.rows[k] > 0 && running(ctx.sc[ts.inst[k]]);
    if (!any_of(on)) return;
    count_rows<R>(lv.bytes, lane, ts, on, col_bytes(lv, W) + sizeof(T) * (W + 4ull));
    const std::uint32_t P = lv.rows;
    T q[R], y[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int row = ts.tile[k] * kTile + lane;
        const ColumnsOf col = columns_of(lv, ts.tile[k], row);
        T s = lv.vd[W * P + row] * in[row];
#pragma unroll
        for (int j = 0; j < W; ++j) s += lv.vd[j * P + row] * in[col[j]];
        y[k] = s;
        q[k] = prod(shadow[row], s);
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const bool store = on[k] && lane < ts.rows[k];
        if (store) out[ts.tile[k] * kTile + lane] = y[k];
        if (!store) q[k] = T(0);
    }
    double sum[R];
    bool fin[R];
    tiles_reduce<T, 1, R, C>(q, ctx, ts, on, sum, fin, gid, lane);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (fin[k]) finish_bicg_v(ctx.sc[ts.inst[k]], &sum[k]);
    }
}

// s = r - alpha v; ||s||: converged at s -> finish with x += alpha p_hat.
template <typename T, int R, int C = kTicket>
__device__ void bicg_s(const LevelView<T>& lv, int t0, int gid, int lane, const T* PSGB_PHASE_RESTRICT r,
                       const T* PSGB_PHASE_RESTRICT v, T* PSGB_PHASE_RESTRICT s_out, T* xv, T omega_j, const ReduceCtx& ctx) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.rows[k] > 0 && running(ctx.sc[ts.inst[k]]);
    if (!any_of(on)) return;
    count_rows<R>(lv.bytes, lane, ts, on, 5ull * sizeof(T));
    T q[R], sv[R], zv[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int row = ts.tile[k] * kTile + lane;
        const T alpha = T(ctx.sc[ts.inst[k]].alpha);
        sv[k] = r[row] - alpha * v[row];
        zv[k] = omega_j * lv.inv[row] * sv[k];
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        q[k] = T(0);
        if (!on[k] || lane >= ts.rows[k]) continue;
        const int row = ts.tile[k] * kTile + lane;
        s_out[row] = sv[k];
        q[k] = prod(sv[k], sv[k]);
        if (ts.sweep[k]) xv[row] = zv[k];
    }
    double sum[R];
    bool fin[R];
    tiles_reduce<T, 1, R, C>(q, ctx, ts, on, sum, fin, gid, lane);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (fin[k]) finish_bicg_s(ctx.sc[ts.inst[k]], &sum[k]);
    }
}

// t = A s_hat; (t.t, t.s) -> omega
template <typename T, int W, int R, int C = kTicket>
__device__ void bicg_t(const LevelView<T>& lv, int t0, int gid, int lane, const T* PSGB_PHASE_RESTRICT shat,
                       T* PSGB_PHASE_RESTRICT t, const T* PSGB_PHASE_RESTRICT s_vec, const ReduceCtx& ctx) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const InstanceScalars& sc = ctx.sc[ts.inst[k]];
        on[k] = ts.rows[k] > 0 && running(sc) && !sc.half_done;
    }
    if (!any_of(on)) return;
    count_rows<R>(lv.bytes, lane, ts, on, col_bytes(lv, W) + sizeof(T) * (W + 4ull));
    const std::uint32_t P = lv.rows;
    T q[2 * R], y[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int row = ts.tile[k] * kTile + lane;
        const ColumnsOf col = columns_of(lv, ts.tile[k], row);
        T s = lv.vd[W * P + row] * shat[row];
#pragma unroll
        for (int j = 0; j < W; ++j) s += lv.vd[j * P + row] * shat[col[j]];
        y[k] = s;
        q[2 * k] = prod(s, s);
        q[2 * k + 1] = prod(s, s_vec[row]);
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const bool store = on[k] && lane < ts.rows[k];
        if (store) t[ts.tile[k] * kTile + lane] = y[k];
        if (!store) { q[2 * k] = T(0); q[2 * k + 1] = T(0); }
    }
    double sum[2 * R];
    bool fin[R];
    tiles_reduce<T, 2, R, C>(q, ctx, ts, on, sum, fin, gid, lane);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (fin[k]) finish_bicg_t(ctx.sc[ts.inst[k]], &sum[2 * k]);
    }
}

// x += alpha p_hat + omega s_hat; r = s - omega t; (r.r, shadow.r) -> next rho/beta.
// A planet that converged at s (half_done) finishes with x += alpha p_hat instead; its
// tiles still count through the reduction so that its last tile closes the iteration.
template <typename T, int R, int C = kTicket>
__device__ void bicg_x(const LevelView<T>& lv, int t0, int gid, int lane, const T* PSGB_PHASE_RESTRICT phat,
                       const T* PSGB_PHASE_RESTRICT shat, const T* PSGB_PHASE_RESTRICT s_vec, const T* PSGB_PHASE_RESTRICT t,
                       T* x, T* r, const T* PSGB_PHASE_RESTRICT shadow, const ReduceCtx& ctx) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R], half[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const InstanceScalars& sc = ctx.sc[ts.inst[k]];
        on[k] = ts.rows[k] > 0 && running(sc);
        half[k] = sc.half_done != 0;
    }
    if (!any_of(on)) return;
    count_rows<R>(lv.bytes, lane, ts, on, 8ull * sizeof(T));
    T q[2 * R], xv[R], rv[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int row = ts.tile[k] * kTile + lane;
        const InstanceScalars& sc = ctx.sc[ts.inst[k]];
        const T alpha = T(sc.alpha), omega = T(sc.omega);
        if (half[k]) {
            xv[k] = x[row] + alpha * phat[row];
            rv[k] = T(0);
        } else {
            xv[k] = x[row] + (alpha * phat[row] + omega * shat[row]);
            rv[k] = s_vec[row] - omega * t[row];
        }
        q[2 * k] = prod(rv[k], rv[k]);
        q[2 * k + 1] = prod(shadow[row], rv[k]);
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const bool store = on[k] && lane < ts.rows[k];
        if (store) {
            const int row = ts.tile[k] * kTile + lane;
            x[row] = xv[k];
            if (!half[k]) r[row] = rv[k];
        }
        if (!store || half[k]) { q[2 * k] = T(0); q[2 * k + 1] = T(0); }
    }
    double sum[2 * R];
    bool fin[R];
    tiles_reduce<T, 2, R, C>(q, ctx, ts, on, sum, fin, gid, lane);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (fin[k]) finish_bicg_x(ctx.sc[ts.inst[k]], &sum[2 * k]);
    }
}

template <typename T, int R, int C = kTicket>
__device__ void pcg_init(const LevelView<T>& lv, int t0, int gid, int lane, const T* PSGB_PHASE_RESTRICT b, T* x, T* r,
                         T* p, T* xv, T omega_j, const ReduceCtx& ctx, double tol, int max_it) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.rows[k] > 0 && ctx.sc[ts.inst[k]].outer_status == kRunning;
    if (!any_of(on)) return;
    count_rows<R>(lv.bytes, lane, ts, on, 5ull * sizeof(T));
    T q[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        q[k] = T(0);
        if (!on[k] || lane >= ts.rows[k]) continue;
        const int row = ts.tile[k] * kTile + lane;
        const T bv = b[row];
        x[row] = T(0); r[row] = bv; p[row] = T(0);
        if (ts.sweep[k]) xv[row] = omega_j * lv.inv[row] * bv;
        q[k] = prod(bv, bv);
    }
    double out[R];
    bool fin[R];
    tiles_reduce<T, 1, R, C>(q, ctx, ts, on, out, fin, gid, lane);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (fin[k]) finish_pcg_init(ctx.sc[ts.inst[k]], &out[k], tol, max_it);
    }
}

// rho = r.z, beta = rho / rho_old
template <typename T, int R, int C = kTicket>
__device__ void pcg_rz(const LevelView<T>& lv, int t0, int gid, int lane, const T* PSGB_PHASE_RESTRICT r,
                       const T* PSGB_PHASE_RESTRICT z, const ReduceCtx& ctx) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.rows[k] > 0 && running(ctx.sc[ts.inst[k]]);
    if (!any_of(on)) return;
    count_rows<R>(lv.bytes, lane, ts, on, 2ull * sizeof(T));
    T q[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int row = ts.tile[k] * kTile + lane;
        q[k] = (on[k] && lane < ts.rows[k]) ? prod(r[row], z[row]) : T(0);
    }
    double sum[R];
    bool fin[R];
    tiles_reduce<T, 1, R, C>(q, ctx, ts, on, sum, fin, gid, lane);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (fin[k]) finish_pcg_rz(ctx.sc[ts.inst[k]], &sum[k]);
    }
}

template <typename T, int R>
__device__ void pcg_p(const LevelView<T>& lv, int t0, int lane, const T* PSGB_PHASE_RESTRICT z, T* p,
                      const InstanceScalars* sc) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.rows[k] > 0 && running(sc[ts.inst[k]]);
    count_rows<R>(lv.bytes, lane, ts, on, 3ull * sizeof(T));   // z, p; p
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (lane >= ts.rows[k] || !on[k]) continue;
        const int row = ts.tile[k] * kTile + lane;
        p[row] = z[row] + T(sc[ts.inst[k]].beta) * p[row];
    }
}

// q = A p; alpha = rho / p.q
template <typename T, int W, int R, int C = kTicket>
__device__ void pcg_q(const LevelView<T>& lv, int t0, int gid, int lane, const T* PSGB_PHASE_RESTRICT p,
                      T* PSGB_PHASE_RESTRICT q_out, const ReduceCtx& ctx) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.rows[k] > 0 && running(ctx.sc[ts.inst[k]]);
    if (!any_of(on)) return;
    count_rows<R>(lv.bytes, lane, ts, on, col_bytes(lv, W) + sizeof(T) * (W + 3ull));
    const std::uint32_t P = lv.rows;
    T q[R], y[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int row = ts.tile[k] * kTile + lane;
        const ColumnsOf col = columns_of(lv, ts.tile[k], row);
        T s = lv.vd[W * P + row] * p[row];
#pragma unroll
        for (int j = 0; j < W; ++j) s += lv.vd[j * P + row] * p[col[j]];
        y[k] = s;
        q[k] = prod(p[row], s);
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const bool store = on[k] && lane < ts.rows[k];
        if (store) q_out[ts.tile[k] * kTile + lane] = y[k];
        if (!store) q[k] = T(0);
    }
    double sum[R];
    bool fin[R];
    tiles_reduce<T, 1, R, C>(q, ctx, ts, on, sum, fin, gid, lane);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (fin[k]) finish_pcg_q(ctx.sc[ts.inst[k]], &sum[k]);
    }
}

// x += alpha p; r -= alpha q; ||r|| -> converged?; first sweep of M r.
template <typename T, int R, int C = kTicket>
__device__ void pcg_xr(const LevelView<T>& lv, int t0, int gid, int lane, const T* PSGB_PHASE_RESTRICT p,
                       const T* PSGB_PHASE_RESTRICT q_in, T* x, T* r, T* xv, T omega_j, const ReduceCtx& ctx) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.rows[k] > 0 && running(ctx.sc[ts.inst[k]]);
    if (!any_of(on)) return;
    count_rows<R>(lv.bytes, lane, ts, on, 8ull * sizeof(T));
    T q[R], xn[R], rn[R], zn[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int row = ts.tile[k] * kTile + lane;
        const T alpha = T(ctx.sc[ts.inst[k]].alpha);
        xn[k] = x[row] + alpha * p[row];
        rn[k] = r[row] - alpha * q_in[row];
        zn[k] = omega_j * lv.inv[row] * rn[k];
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        q[k] = T(0);
        if (!on[k] || lane >= ts.rows[k]) continue;
        const int row = ts.tile[k] * kTile + lane;
        x[row] = xn[k];
        r[row] = rn[k];
        q[k] = prod(rn[k], rn[k]);
        if (ts.sweep[k]) xv[row] = zn[k];
    }
    double sum[R];
    bool fin[R];
    tiles_reduce<T, 1, R, C>(q, ctx, ts, on, sum, fin, gid, lane);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (fin[k]) finish_pcg_xr(ctx.sc[ts.inst[k]], &sum[k]);
    }
}

// ---- FP64 refinement ----------------------------------------------------------------------

template <int R, int C = kTicket>
__device__ void outer_init(const LevelView<double>& lv, int t0, int gid, int lane, const double* PSGB_PHASE_RESTRICT b,
                           const ReduceCtx& ctx, double tol, const std::uint8_t* PSGB_PHASE_RESTRICT active) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        on[k] = ts.rows[k] > 0;
        if (!on[k] || active == nullptr || active[ts.inst[k]]) continue;
        // a planet left out of this step: nothing runs for it
        on[k] = false;
        if (lane == 0 && static_cast<unsigned>(ts.tile[k]) == ctx.tile_begin[ts.inst[k]]) {
            InstanceScalars& s = ctx.sc[ts.inst[k]];
            s.outer_status = kConverged;
            s.status = kConverged;
            s.refinements = 0;
            s.inner_total = 0;
            s.outer_r_norm = 0.0;
            s.outer_b_norm = 0.0;
        }
    }
    if (!any_of(on)) return;
    count_rows<R>(lv.bytes, lane, ts, on, 8ull);
    double q[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int row = ts.tile[k] * kTile + lane;
        q[k] = (on[k] && lane < ts.rows[k]) ? dmul(b[row], b[row]) : 0.0;
    }
    double sum[R];
    bool fin[R];
    tiles_reduce<double, 1, R, C>(q, ctx, ts, on, sum, fin, gid, lane);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (fin[k]) finish_outer_init(ctx.sc[ts.inst[k]], &sum[k], tol);
    }
}

// r = b - A x in FP64 (FP64 matrix), cast to the inner precision; ||r|| decides.
template <typename TI, int W, int R, int C = kTicket>
__device__ void outer_residual(const LevelView<double>& lv, int t0, int gid, int lane, const double* PSGB_PHASE_RESTRICT b,
                               const double* PSGB_PHASE_RESTRICT x, double* PSGB_PHASE_RESTRICT r64, TI* PSGB_PHASE_RESTRICT rin,
                               const ReduceCtx& ctx, int max_refine) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.rows[k] > 0 && ctx.sc[ts.inst[k]].outer_status == kRunning;
    if (!any_of(on)) return;
    count_rows<R>(lv.bytes, lane, ts, on, col_bytes(lv, W) + 8ull * (W + 4ull) + sizeof(TI));
    const std::uint32_t P = lv.rows;
    double q[R], rv[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int row = ts.tile[k] * kTile + lane;
        const ColumnsOf col = columns_of(lv, ts.tile[k], row);
        double s = b[row] - lv.vd[W * P + row] * x[row];
#pragma unroll
        for (int j = 0; j < W; ++j) s -= lv.vd[j * P + row] * x[col[j]];
        rv[k] = s;
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        q[k] = 0.0;
        if (!on[k] || lane >= ts.rows[k]) continue;
        const int row = ts.tile[k] * kTile + lane;
        r64[row] = rv[k];
        rin[row] = static_cast<TI>(rv[k]);
        q[k] = prod(rv[k], rv[k]);
    }
    double sum[R];
    bool fin[R];
    tiles_reduce<double, 1, R, C>(q, ctx, ts, on, sum, fin, gid, lane);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (fin[k]) finish_outer_residual(ctx.sc[ts.inst[k]], &sum[k], max_refine);
    }
}

// x += delta (inner solution), for planets still refining.
template <typename TI, int R>
__device__ void outer_update(const LevelView<double>& lv, int t0, int lane, const TI* PSGB_PHASE_RESTRICT delta, double* x,
                             const InstanceScalars* sc) {
    const TileSet<R> ts = tile_set<R>(lv.tile_meta, lv.tiles, t0);
    bool on[R];
#pragma unroll
    for (int k = 0; k < R; ++k) on[k] = ts.rows[k] > 0 && sc[ts.inst[k]].outer_status == kRunning;
    count_rows<R>(lv.bytes, lane, ts, on, 16ull + sizeof(TI));   // delta, x; x
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (lane >= ts.rows[k] || !on[k]) continue;
        const int row = ts.tile[k] * kTile + lane;
        x[row] += static_cast<double>(delta[row]);
    }
}

__device__ inline void outer_account(InstanceScalars& s) {
    if (s.outer_status != kRunning) return;
    s.inner_total += s.iterations;
    if (s.status == kNonFinite) s.outer_status = kNonFinite;
}

}  // namespace ph

using ph::counted;

}  // namespace psgb

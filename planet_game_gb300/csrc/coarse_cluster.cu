// The coarse tail of the V-cycle on a thread-block cluster per planet (coarse_tail.hpp):
// the vectors (x, y, b, r) of every level from the tail level down are spread over the
// shared memory of the cluster's blocks, each block holding the slices of the tiles it
// owns, and every phase of the coarse cycle runs between cluster barriers. A row's
// neighbours held by another block of the cluster are read from that block's shared memory
// (distributed shared memory), so the dependent loads of a phase's gathers, restrictions
// and prolongations stay on chip; only the matrices stream from L2.
//
// Each phase is the per-tile arithmetic of phases.cuh written against these distributed
// vectors (same terms, same order), so the results are the other tails' bit for bit. In:
// the tail level's right-hand side and the iterate of its zero-start sweep; out: its final
// iterate, as for the other tails.
#include "coarse_tail.hpp"
#include "phases.cuh"
#include "planet.hpp"
#include "profile.hpp"

#include <cooperative_groups.h>

#include <algorithm>
#include <stdexcept>
#include <string>
#include <type_traits>

namespace cg = cooperative_groups;

namespace psgb {
namespace {

template <typename F>
__device__ __forceinline__ void cluster_widths(unsigned width, F&& f) {
    switch (width) {
        case 6: f(std::integral_constant<int, 6>{}); break;
        case 8: f(std::integral_constant<int, 8>{}); break;
        case 12: f(std::integral_constant<int, 12>{}); break;
        default: f(std::integral_constant<int, 16>{}); break;
    }
}

// One level vector of one planet spread over the cluster: block k holds rows
// [base + k span, base + (k + 1) span) at the same shared-memory offset `local`, span = q
// tiles. The holder of a row is its tile (within the planet) over q, by a multiply with
// inv_q = ceil(2^16 / q) and a shift: exact while tile * q < 2^16, which the shared memory
// bounds (q tiles of four vectors per block: q <= 55 and tiles <= 8 q).
//
// Every lookup is checked: a row outside the planet's slices (which no valid input makes)
// records kClusterIndexError in the launch's error word and is redirected to a scratch
// slot of this block, so a bad index never reaches another block's shared memory; the
// host turns the error word into an exception after the solve.
constexpr unsigned kClusterIndexError = 2u;

template <typename T>
struct DistVec {
    T* local;
    T* scratch;       // this block's scratch slot for refused lookups
    unsigned* error;  // the launch's error word
    int base;
    int span;
    int clusters;     // blocks of the cluster
    unsigned inv_q;
    int me;           // this block's rank in the cluster
    __device__ __forceinline__ T* at(int row, cg::cluster_group& cl) const {
        const int d = row - base;
        const int rank = static_cast<int>((static_cast<unsigned>(d >> 8) * inv_q) >> 16);
        const int off = d - rank * span;
        if (d < 0 || rank >= clusters || off >= span) {
            atomicCAS(error, 0u, kClusterIndexError);
            return scratch;
        }
        T* p = rank == me ? local : cl.map_shared_rank(local, static_cast<unsigned>(rank));
        return p + off;
    }
};

template <typename T>
struct DistLevel {
    DistVec<T> x, y, b, r;
    int tile0, tiles;   // the planet's tiles at the level
    int own0, own1;     // the tiles this block owns
};

// ---- phases on distributed vectors (the arithmetic of phases.cuh) -------------------------

template <typename T, int W>
__device__ void c_smooth(const LevelView<T>& lv, int tile, int lane, const DistVec<T>& b, const DistVec<T>& x,
                         const DistVec<T>& y, T omega, cg::cluster_group& cl) {
    const ph::TileSet<1> ts = ph::tile_set<1>(lv.tile_meta, lv.tiles, tile);
    if (!ts.sweep[0]) return;
    const std::uint32_t P = lv.rows;
    const int row = ts.tile[0] * kTile + lane;
    T s = *b.at(row, cl);
#pragma unroll
    for (int j = 0; j < W; ++j) s -= lv.vd[j * P + row] * *x.at(lv.col[j * P + row], cl);
    T out;
    if (omega == T(1)) {
        out = lv.inv[row] * s;
    } else {
        const T xo = *x.at(row, cl);
        out = xo + omega * (lv.inv[row] * s - xo);
    }
    ph::count_bytes(lv.bytes, lane, static_cast<unsigned long long>(ts.rows[0]) * (4ull * W + sizeof(T) * (W + 4ull)));
    if (lane < ts.rows[0]) *y.at(row, cl) = out;
}

template <typename T, int W>
__device__ void c_smooth_block(const LevelView<T>& lv, int tile, int gid, int lane, const DistVec<T>& b,
                               const DistVec<T>& x, const DistVec<T>& y, T omega, int inner, cg::cluster_group& cl) {
    T (*xs)[kTile] = ph::tile_buffer<T>();
    const ph::TileSet<1> ts = ph::tile_set<1>(lv.tile_meta, lv.tiles, tile);
    if (!ts.sweep[0]) return;
    const std::uint32_t P = lv.rows;
    const int row = ts.tile[0] * kTile + lane;
    const int first = ts.tile[0] * kTile;
    const bool live = lane < ts.rows[0];
    T a[W], h[W];
    int local[W];
    T bv = T(0), inv = T(0), xo = T(0);
    if (live) {
        bv = *b.at(row, cl);
        inv = lv.inv[row];
        xo = *x.at(row, cl);
#pragma unroll
        for (int j = 0; j < W; ++j) {
            const int c = lv.col[j * P + row];
            a[j] = lv.vd[j * P + row];
            local[j] = (c >= first && c < first + kTile) ? c - first : -1;
            h[j] = local[j] < 0 ? *x.at(c, cl) : T(0);
        }
    }
    xs[gid][lane] = xo;
    ph::group_sync(gid);
    for (int sweep = 0; sweep < inner; ++sweep) {
        T out = xo;
        if (live) {
            T s = bv;
#pragma unroll
            for (int j = 0; j < W; ++j) s = ph::fnma(a[j], local[j] >= 0 ? xs[gid][local[j]] : h[j], s);
            out = ph::jacobi_update(xo, omega, inv, s);
        }
        ph::group_sync(gid);
        xs[gid][lane] = out;
        xo = out;
        ph::group_sync(gid);
    }
    ph::count_bytes(lv.bytes, lane, static_cast<unsigned long long>(ts.rows[0]) * (4ull * W + sizeof(T) * (W + 4ull)));
    if (live) *y.at(row, cl) = xo;
}

template <typename T, int W>
__device__ void c_residual(const LevelView<T>& lv, int tile, int lane, const DistVec<T>& b, const DistVec<T>& x,
                           const DistVec<T>& r, cg::cluster_group& cl) {
    const ph::TileSet<1> ts = ph::tile_set<1>(lv.tile_meta, lv.tiles, tile);
    if (!ts.sweep[0]) return;
    const std::uint32_t P = lv.rows;
    const int row = ts.tile[0] * kTile + lane;
    T s = *b.at(row, cl) - lv.vd[W * P + row] * *x.at(row, cl);
#pragma unroll
    for (int j = 0; j < W; ++j) s -= lv.vd[j * P + row] * *x.at(lv.col[j * P + row], cl);
    ph::count_bytes(lv.bytes, lane, static_cast<unsigned long long>(ts.rows[0]) * (4ull * W + sizeof(T) * (W + 4ull)));
    if (lane < ts.rows[0]) *r.at(row, cl) = s;
}

// b_c = sum of the members' residuals in ascending order (eight loads in flight, the
// additions sequential); x_c = omega b_c / diag where the planet smooths on the coarse level.
template <typename T>
__device__ void c_restrict_zero(const LevelView<T>& coarse, int tile, int lane, const std::uint32_t* moff,
                                const std::uint32_t* member, const DistVec<T>& r, const DistVec<T>& bc,
                                const DistVec<T>& xc, T omega, cg::cluster_group& cl) {
    const ph::TileSet<1> ts = ph::tile_set<1>(coarse.tile_meta, coarse.tiles, tile);
    if (ts.rows[0] == 0) return;
    unsigned moved = 0;
    if (lane < ts.rows[0]) {
        const int row = ts.tile[0] * kTile + lane;
        const std::uint32_t k0 = moff[row], k1 = moff[row + 1];
        T s = T(0);
        for (std::uint32_t k = k0; k < k1; k += 8) {
            T v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) v[j] = (k + j < k1) ? *r.at(static_cast<int>(member[k + j]), cl) : T(0);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (k + j < k1) s += v[j];
            }
        }
        *bc.at(row, cl) = s;
        if (ts.sweep[0]) *xc.at(row, cl) = omega * coarse.inv[row] * s;
        moved = 4u + (k1 - k0) * (4u + static_cast<unsigned>(sizeof(T))) + 3u * static_cast<unsigned>(sizeof(T));
    }
    ph::count_bytes_warp(coarse.bytes, moved);
}

template <typename T, int W>
__device__ void c_prolong_smooth(const LevelView<T>& lv, int tile, int lane, const std::int32_t* agg,
                                 const DistVec<T>& e, const DistVec<T>& b, const DistVec<T>& x, const DistVec<T>& y,
                                 T omega, cg::cluster_group& cl) {
    const ph::TileSet<1> ts = ph::tile_set<1>(lv.tile_meta, lv.tiles, tile);
    if (!ts.sweep[0]) return;
    ph::count_bytes(lv.bytes, lane, static_cast<unsigned long long>(ts.rows[0]) * (4ull * W + sizeof(T) * (W + 4ull) + 4ull));
    // padding rows store nothing, and their aggregate index (coarse row 0 of the batch) is
    // not this planet's: they are skipped (a valid row's neighbours and their aggregates are
    // all the planet's own)
    if (lane >= ts.rows[0]) return;
    const std::uint32_t P = lv.rows;
    const int row = ts.tile[0] * kTile + lane;
    T s = *b.at(row, cl);
#pragma unroll
    for (int j = 0; j < W; ++j) {
        const int c = lv.col[j * P + row];
        s -= lv.vd[j * P + row] * (*x.at(c, cl) + ph::prod(lv.correction, *e.at(agg[c], cl)));
    }
    T out;
    if (omega == T(1)) {
        out = lv.inv[row] * s;
    } else {
        const T xo = *x.at(row, cl) + ph::prod(lv.correction, *e.at(agg[row], cl));
        out = xo + omega * (lv.inv[row] * s - xo);
    }
    *y.at(row, cl) = out;
}

template <typename T>
__device__ void c_prolong(const LevelView<T>& lv, int tile, int lane, const std::int32_t* agg, const DistVec<T>& xc,
                          const DistVec<T>& x, cg::cluster_group& cl) {
    const ph::TileSet<1> ts = ph::tile_set<1>(lv.tile_meta, lv.tiles, tile);
    if (lane >= ts.rows[0] || !ts.sweep[0]) return;
    const int row = ts.tile[0] * kTile + lane;
    *x.at(row, cl) += ph::prod(lv.correction, *xc.at(agg[row], cl));
}

template <typename T>
__device__ void c_dense_row(const DenseView& dense, int inst, int rowi, int lane32, const T* inv, const DistVec<T>& b,
                            const DistVec<T>& x, cg::cluster_group& cl) {
    const int n = static_cast<int>(dense.size[inst]);
    const int base = static_cast<int>(dense.row_base[inst]);
    const T* a = inv + dense.offset[inst] + static_cast<std::int64_t>(rowi) * n;
    T s = T(0);
    for (int j = lane32; j < n; j += 32) s += a[j] * *b.at(base + j, cl);
    s = warp_sum(s);
    if (lane32 == 0) *x.at(base + rowi, cl) = s;
}

// ---- the kernel ---------------------------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(1024, 1) k_coarse_cluster(const __grid_constant__ TailArgs<T> a) {
    cg::cluster_group cl = cg::this_cluster();
    const int C = static_cast<int>(a.cluster);
    const int inst = static_cast<int>(blockIdx.x) / C;
    const int rank = static_cast<int>(cl.block_rank());
    const int coarsest = a.dense.level[inst];
    if (coarsest < a.first || !ph::gate_open(a.sc, inst, a.gate)) return;   // the whole cluster
    const int gid = static_cast<int>(threadIdx.x >> 8), lane = static_cast<int>(threadIdx.x & 255);
    extern __shared__ __align__(16) unsigned char cluster_bytes[];
    T* vec = reinterpret_cast<T*>(cluster_bytes);
    // this planet's slices: per level four vectors of `span` rows in every block
    __shared__ DistLevel<T> lv[kMaxLevels];
    __shared__ int total_rows;
    __shared__ T scratch;
    if (threadIdx.x == 0) {
    int total = 0;
    for (int l = a.first; l <= coarsest; ++l) {
        const int t0 = static_cast<int>(a.tile_range[(l * a.instances + inst) * 2]);
        const int nt = static_cast<int>(a.tile_range[(l * a.instances + inst) * 2 + 1]);
        const int q = (nt + C - 1) / C;
        const int span = q * kTile;
        const unsigned inv_q = (65536u + static_cast<unsigned>(q) - 1u) / static_cast<unsigned>(q);
        T* slice = vec + total;
        for (int v = 0; v < 4; ++v) {
            DistVec<T>& dv = v == 0 ? lv[l].x : v == 1 ? lv[l].y : v == 2 ? lv[l].b : lv[l].r;
            dv = DistVec<T>{slice + v * span, &scratch, a.error, t0 * kTile, span, C, inv_q, rank};
        }
        lv[l].tile0 = t0;
        lv[l].tiles = nt;
        lv[l].own0 = t0 + ::min(nt, rank * q);
        lv[l].own1 = t0 + ::min(nt, (rank + 1) * q);
        total += 4 * span;
    }
    total_rows = total;
    }
    __syncthreads();
    for (int i = static_cast<int>(threadIdx.x); i < total_rows; i += static_cast<int>(blockDim.x)) vec[i] = T(0);
    __syncthreads();
    // the tail level's right-hand side and zero-start iterate, this block's tiles
    const int first = a.first;
    const bool first_in_x = a.starts_in_x[first] != 0;
    {
        const T* gx = first_in_x ? a.level[first].x : a.level[first].y;
        const DistLevel<T>& F = lv[first];
        const DistVec<T>& sx = first_in_x ? F.x : F.y;
        for (int row = F.own0 * kTile + static_cast<int>(threadIdx.x); row < F.own1 * kTile;
             row += static_cast<int>(blockDim.x)) {
            F.b.local[row - F.b.base - rank * F.b.span] = a.level[first].b[row];
            sx.local[row - sx.base - rank * sx.span] = gx[row];
        }
    }
    cl.sync();
    const T omega = a.omega;
#define PSGB_OWN_TILES(L) for (int tile = (L).own0 + gid; tile < (L).own1; tile += ph::kGroups)
    // Down: the level's remaining pre-sweeps, residual, restriction fused with the next
    // level's first sweep.
    for (int l = first; l < coarsest; ++l) {
        const LevelView<T>& view = a.level[l].view;
        const DistLevel<T>& L = lv[l];
        DistVec<T> cur = a.starts_in_x[l] ? L.x : L.y, oth = a.starts_in_x[l] ? L.y : L.x;
        for (int k = 1; k < a.pre[l]; ++k) {
            cluster_widths(view.width, [&](auto W) {
                if (a.inner[l] > 1) {
                    PSGB_OWN_TILES(L) c_smooth_block<T, decltype(W)::value>(view, tile, gid, lane, L.b, cur, oth, omega,
                                                                         a.inner[l], cl);
                } else {
                    PSGB_OWN_TILES(L) c_smooth<T, decltype(W)::value>(view, tile, lane, L.b, cur, oth, omega, cl);
                }
            });
            cl.sync();
            const DistVec<T> t = cur; cur = oth; oth = t;
        }
        cluster_widths(view.width, [&](auto W) {
            PSGB_OWN_TILES(L) c_residual<T, decltype(W)::value>(view, tile, lane, L.b, cur, L.r, cl);
        });
        cl.sync();
        const DistLevel<T>& Cn = lv[l + 1];
        const DistVec<T> cn = a.starts_in_x[l + 1] ? Cn.x : Cn.y;
        PSGB_OWN_TILES(Cn)
            c_restrict_zero<T>(a.level[l + 1].view, tile, lane, a.level[l].member_offset, a.level[l].member, L.r, Cn.b,
                               cn, omega, cl);
        cl.sync();
    }
    // The coarsest level: x = A^-1 b, one warp per row over the cluster.
    {
        const int n = static_cast<int>(a.dense.size[inst]);
        for (int row = rank * 32 + static_cast<int>(threadIdx.x >> 5); row < n; row += 32 * C)
            c_dense_row<T>(a.dense, inst, row, static_cast<int>(threadIdx.x & 31), a.dense_inv, lv[coarsest].b,
                           lv[coarsest].x, cl);
        cl.sync();
    }
    // Up: prolongation fused with the first post-sweep, then the remaining post-sweeps.
    for (int l = coarsest - 1; l >= first; --l) {
        const LevelView<T>& view = a.level[l].view;
        const DistLevel<T>& L = lv[l];
        const DistVec<T>& e = lv[l + 1].x;
        DistVec<T> cur = a.starts_in_x[l] ? L.x : L.y, oth = a.starts_in_x[l] ? L.y : L.x;
        if ((a.pre[l] - 1) & 1) { const DistVec<T> t = cur; cur = oth; oth = t; }   // where the down sweeps ended
        if (a.post[l] == 0) {
            PSGB_OWN_TILES(L) c_prolong<T>(view, tile, lane, a.level[l].agg, e, cur, cl);
            cl.sync();
            continue;
        }
        cluster_widths(view.width, [&](auto W) {
            PSGB_OWN_TILES(L)
                c_prolong_smooth<T, decltype(W)::value>(view, tile, lane, a.level[l].agg, e, L.b, cur, oth, omega, cl);
        });
        cl.sync();
        { const DistVec<T> t = cur; cur = oth; oth = t; }
        for (int k = 1; k < a.post[l]; ++k) {
            cluster_widths(view.width, [&](auto W) {
                if (a.inner[l] > 1) {
                    PSGB_OWN_TILES(L) c_smooth_block<T, decltype(W)::value>(view, tile, gid, lane, L.b, cur, oth, omega,
                                                                         a.inner[l], cl);
                } else {
                    PSGB_OWN_TILES(L) c_smooth<T, decltype(W)::value>(view, tile, lane, L.b, cur, oth, omega, cl);
                }
            });
            cl.sync();
            const DistVec<T> t = cur; cur = oth; oth = t;
        }
    }
#undef PSGB_OWN_TILES
    // the tail level's final iterate (in its x) back to global memory, valid rows only
    {
        const DistLevel<T>& F = lv[first];
        for (int t = F.own0; t < F.own1; ++t) {
            const int rows = static_cast<int>((a.level[first].view.tile_meta[t] >> 22) & 0x1FFu);
            const int row = t * kTile + static_cast<int>(threadIdx.x);
            if (static_cast<int>(threadIdx.x) < rows) a.level[first].x[row] = F.x.local[row - F.x.base - rank * F.x.span];
        }
    }
}

}  // namespace

template <typename T>
unsigned cluster_tail_max_bytes() {
    static const unsigned limit = [] {
        int device = 0, optin = 0, cluster = 0;
        cudaFuncAttributes fa{};
        if (cudaGetDevice(&device) != cudaSuccess ||
            cudaDeviceGetAttribute(&cluster, cudaDevAttrClusterLaunch, device) != cudaSuccess || cluster == 0 ||
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess ||
            cudaFuncGetAttributes(&fa, k_coarse_cluster<T>) != cudaSuccess) {
            cudaGetLastError();
            return 0u;
        }
        const long room = static_cast<long>(optin) - static_cast<long>(fa.sharedSizeBytes);
        if (room <= 0 || cudaFuncSetAttribute(k_coarse_cluster<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              static_cast<int>(room)) != cudaSuccess) {
            cudaGetLastError();
            return 0u;
        }
        return static_cast<unsigned>(room);
    }();
    return limit;
}
template unsigned cluster_tail_max_bytes<float>();
template unsigned cluster_tail_max_bytes<double>();

template <typename T>
bool cluster_tail_fits(unsigned cluster, unsigned rows_per_block) {
    const std::size_t bytes = std::size_t(4) * rows_per_block * sizeof(T);
    if (cluster < 2 || cluster > 8 || (cluster & (cluster - 1)) != 0 || bytes > cluster_tail_max_bytes<T>()) return false;
    // can a cluster of that many blocks, each with this shared memory, be resident at all
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(cluster);
    cfg.blockDim = dim3(1024);
    cfg.dynamicSmemBytes = bytes;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, k_coarse_cluster<T>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return clusters > 0;
}
template bool cluster_tail_fits<float>(unsigned, unsigned);
template bool cluster_tail_fits<double>(unsigned, unsigned);

template <typename T>
void launch_coarse_cluster(const TailArgs<T>& args, cudaStream_t st) {
    const std::size_t bytes = std::size_t(4) * args.shared_rows * sizeof(T);
    if (args.cluster < 2 || args.cluster > 8 || (args.cluster & (args.cluster - 1)) != 0 ||
        bytes > cluster_tail_max_bytes<T>())
        throw std::logic_error("coarse tail: the cluster layout does not fit");
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = args.cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(args.instances * args.cluster);
    cfg.blockDim = dim3(1024);
    cfg.dynamicSmemBytes = bytes;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PSGB_LAUNCH(kFamSmoothCoarse, st, {
        const cudaError_t e = cudaLaunchKernelEx(&cfg, k_coarse_cluster<T>, args);
        if (e != cudaSuccess) throw std::runtime_error(std::string("coarse cluster tail launch: ") + cudaGetErrorString(e));
    });
}

template void launch_coarse_cluster<float>(const TailArgs<float>&, cudaStream_t);
template void launch_coarse_cluster<double>(const TailArgs<double>&, cudaStream_t);

}  // namespace psgb

// Aggregation-multigrid kernels for sm_103a (GB300).
//
// Replaces the CPU V-cycle of the reference (sim/planet/surface/heat_transport.cpp:
// coarsen_values :157-171, factor_dense/solve_dense :202-243, gauss_seidel :258-286,
// v_cycle :288-326). The hierarchy's structure is the reference's; the smoother is
// damped Jacobi (both sweeps of a level read only the previous iterate, so every row
// is independent), the coarsest level is solved with an explicit dense inverse.
//
// All kernels are HBM/L2 streaming kernels over ELL slot-major rows: one thread per
// row, 256-row tiles, neighbour gathers served mostly from L2 thanks to the
// reference's space-filling cell order. No tensor cores (sparse stencils).
#include "common.cuh"
#include "kernels.hpp"
#include "phases.cuh"
#include "profile.hpp"

#include <stdexcept>

namespace psgb {
namespace {

// ---- assembly -------------------------------------------------------------

__global__ void k_assemble_transport(LevelView<double> lv, const double* __restrict__ w,
                                     const double* __restrict__ wsum, const double* __restrict__ area,
                                     const double* __restrict__ slope,
                                     const double* __restrict__ conductance,
                                     const double* __restrict__ edge_conductance,
                                     double* __restrict__ vd) {
    pdl_begin();
    const int tile = blockIdx.x;
    const int row = tile * kTile + threadIdx.x;
    const std::uint32_t P = lv.rows, W = lv.width;
    if (threadIdx.x >= lv.tile_rows[tile]) {
        // padding rows: identity, no couplings
        for (std::uint32_t j = 0; j < W; ++j) vd[j * P + row] = 0.0;
        vd[W * P + row] = 1.0;
        return;
    }
    const double K = conductance[lv.tile_inst[tile]];
    const double s = slope[row];
    const bool free_row = s > 0.0;
    double diag;
    if (edge_conductance == nullptr) {
        diag = free_row ? dadd(__ddiv_rn(area[row], s), dmul(K, wsum[row])) : 1.0;
    } else {
        double sum = 0.0;
        for (std::uint32_t j = 0; j < 6; ++j) sum = dadd(sum, dmul(edge_conductance[j * P + row], w[j * P + row]));
        diag = free_row ? dadd(__ddiv_rn(area[row], s), sum) : 1.0;
    }
    vd[W * P + row] = diag;
    for (std::uint32_t j = 0; j < W; ++j) {
        double v = 0.0;
        if (j < 6) {
            const int nb = lv.col[j * P + row];
            const double g = edge_conductance == nullptr ? K : edge_conductance[j * P + row];
            const double wj = w[j * P + row];
            if (free_row && nb != row && slope[nb] > 0.0) v = dmul(-g, wj);
        }
        vd[j * P + row] = v;
    }
}

__global__ void k_set_matrix_csr(std::uint32_t n, std::uint32_t P, std::uint32_t W,
                                 const std::uint32_t* __restrict__ off_begin,
                                 const double* __restrict__ diag, const double* __restrict__ off,
                                 double* __restrict__ vd) {
    pdl_begin();
    const std::uint32_t row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= P) return;
    if (row >= n) {
        for (std::uint32_t j = 0; j < W; ++j) vd[j * P + row] = 0.0;
        vd[W * P + row] = 1.0;
        return;
    }
    const std::uint32_t b = off_begin[row], e = off_begin[row + 1];
    for (std::uint32_t j = 0; j < W; ++j) vd[j * P + row] = (b + j < e) ? off[b + j] : 0.0;
    vd[W * P + row] = diag[row];
}

// Galerkin values: each coarse entry sums its fine sources in the reference's
// order (rows ascending, then the row's entries), from 0.0 - bit-identical to
// coarsen_values.
__global__ void k_galerkin(std::uint32_t lists, const std::uint32_t* __restrict__ offset,
                           const std::uint32_t* __restrict__ source, const double* __restrict__ fine,
                           double* __restrict__ coarse) {
    pdl_begin();
    const std::uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= lists) return;
    double sum = 0.0;
    for (std::uint32_t k = offset[id]; k < offset[id + 1]; ++k) sum = dadd(sum, fine[source[k]]);
    coarse[id] = sum;
}

__global__ void k_finalize_level(std::uint32_t P, std::uint32_t W, double* __restrict__ vd64,
                                 float* __restrict__ vd32, double* __restrict__ inv64,
                                 float* __restrict__ inv32) {
    pdl_begin();
    const std::uint32_t row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= P) return;
    double d = vd64[W * P + row];
    if (d == 0.0) {   // absent rows of a shorter planet: keep them an identity
        d = 1.0;
        vd64[W * P + row] = 1.0;
    }
    for (std::uint32_t j = 0; j < W; ++j) vd32[j * P + row] = static_cast<float>(vd64[j * P + row]);
    vd32[W * P + row] = static_cast<float>(d);
    const double inv = 1.0 / d;
    inv64[row] = inv;
    inv32[row] = static_cast<float>(inv);
}

// Dense inverse of every planet's coarsest level (symmetric positive definite):
// assemble from the ELL values, then in-place Gauss-Jordan without pivoting. One CTA
// per planet; the matrix lives in global memory (<= 400 x 400 doubles).
__global__ void __launch_bounds__(1024) k_dense_invert(DenseView dense, int level, LevelView<double> lv,
                                                       double* __restrict__ work,
                                                       double* __restrict__ inv64,
                                                       float* __restrict__ inv32) {
    pdl_begin();
    const int inst = blockIdx.x;
    if (dense.level[inst] != level) return;
    const int n = static_cast<int>(dense.size[inst]);
    const std::int64_t base = dense.row_base[inst];
    double* a = work + dense.offset[inst];
    const std::uint32_t P = lv.rows, W = lv.width;
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) a[idx] = 0.0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const std::int64_t row = base + i;
        a[i * n + i] = lv.vd[W * P + row];
        for (std::uint32_t j = 0; j < W; ++j) {
            const std::int64_t c = lv.col[j * P + row];
            if (c == row) continue;
            a[i * n + (c - base)] += lv.vd[j * P + row];
        }
    }
    __syncthreads();
    __shared__ double f[400];
    __shared__ double pivot_inv;
    for (int k = 0; k < n; ++k) {
        if (threadIdx.x == 0) pivot_inv = 1.0 / a[k * n + k];
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            a[k * n + j] = (j == k ? 1.0 : a[k * n + j]) * pivot_inv;
        }
        for (int i = threadIdx.x; i < n; i += blockDim.x) f[i] = a[i * n + k];
        __syncthreads();
        for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
            const int i = idx / n, j = idx - i * n;
            if (i == k) continue;
            const double aij = (j == k) ? 0.0 : a[idx];
            a[idx] = aij - f[i] * a[k * n + j];
        }
        __syncthreads();
    }
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
        inv64[dense.offset[inst] + idx] = a[idx];
        inv32[dense.offset[inst] + idx] = static_cast<float>(a[idx]);
    }
}

// ---- V-cycle pieces: one 256-thread block per tile (the shared phases of phases.cuh) ----

template <typename T, int R>
__global__ void k_smooth_zero(LevelView<T> lv, const T* __restrict__ b, T* __restrict__ x, T omega,
                              const InstanceScalars* sc, int gate) {
    ph::prefetch_meta(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    ph::smooth_zero<T, R>(lv, blockIdx.x * R, threadIdx.x, b, x, omega, sc, gate);
}

// Blocks past the level's tile sets carry the dense solves of the planets whose coarsest
// level this is (they do not smooth here).
template <typename T, int W, int R>
__global__ void k_smooth(LevelView<T> lv, const T* __restrict__ b, const T* __restrict__ x, T* __restrict__ y,
                         T omega, const InstanceScalars* sc, int gate, DenseTask<T> dense) {
    ph::prefetch_static<T, W, R>(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    const unsigned sets = ph::tile_sets(lv.tiles, R);
    if (blockIdx.x >= sets) {
        ph::dense_block<T>(dense, blockIdx.x - sets, threadIdx.x, sc, gate);
        return;
    }
    ph::smooth<T, W, R>(lv, blockIdx.x * R, threadIdx.x, b, x, y, omega, sc, gate);
}

template <typename T, int W>
__global__ void k_smooth_block(LevelView<T> lv, const T* __restrict__ b, const T* __restrict__ x, T* __restrict__ y,
                               T omega, int inner, const InstanceScalars* sc, int gate, DenseTask<T> dense) {
    ph::prefetch_static<T, W, 1>(lv, blockIdx.x, threadIdx.x);
    pdl_begin();
    if (blockIdx.x >= lv.tiles) {
        ph::dense_block<T>(dense, blockIdx.x - lv.tiles, threadIdx.x, sc, gate);
        return;
    }
    ph::smooth_block<T, W>(lv, blockIdx.x, 0, threadIdx.x, b, x, y, omega, inner, sc, gate);
}

template <typename T, int W, int R>
__global__ void k_residual(LevelView<T> lv, const T* __restrict__ b, const T* __restrict__ x, T* __restrict__ r,
                           const InstanceScalars* sc, int gate, DenseTask<T> dense) {
    ph::prefetch_static<T, W, R>(lv, blockIdx.x * R, threadIdx.x);
    pdl_begin();
    const unsigned sets = ph::tile_sets(lv.tiles, R);
    if (blockIdx.x >= sets) {
        ph::dense_block<T>(dense, blockIdx.x - sets, threadIdx.x, sc, gate);
        return;
    }
    ph::residual<T, W, R>(lv, blockIdx.x * R, threadIdx.x, b, x, r, sc, gate);
}

template <typename T, int W, int R>
__global__ void k_spmv(LevelView<T> lv, const T* __restrict__ x, T* __restrict__ y) {
    pdl_begin();
    ph::spmv<T, W, R>(lv, blockIdx.x * R, threadIdx.x, x, y);
}

template <typename T>
__global__ void k_restrict(LevelView<T> coarse, const std::uint32_t* __restrict__ moff,
                           const std::uint32_t* __restrict__ member, const T* __restrict__ r, T* __restrict__ bc,
                           const InstanceScalars* sc, int gate) {
    pdl_begin();
    ph::restrict_only<T, ph::kRowsCoarse>(coarse, blockIdx.x * ph::kRowsCoarse, threadIdx.x, moff, member, r, bc, sc, gate);
}

template <typename T>
__global__ void k_restrict_zero(LevelView<T> coarse, const std::uint32_t* __restrict__ moff,
                                const std::uint32_t* __restrict__ member, const T* __restrict__ r,
                                T* __restrict__ bc, T* __restrict__ xc, T omega, const InstanceScalars* sc,
                                int gate) {
#pragma unroll
    for (int k = 0; k < ph::kRowsCoarse; ++k) {
        const unsigned tile = blockIdx.x * ph::kRowsCoarse + k;
        if (tile < coarse.tiles) {
            if (threadIdx.x == 0) ph::prefetch_l1(coarse.tile_meta + tile);
            ph::prefetch_l1(moff + tile * kTile + threadIdx.x);
        }
    }
    pdl_begin();
    ph::restrict_zero<T, ph::kRowsCoarse>(coarse, blockIdx.x * ph::kRowsCoarse, threadIdx.x, moff, member, r, bc, xc, omega,
                                          sc, gate);
}

// A coarse level's residual and the restriction into the next level in one launch: a warp
// per next-level row, lane m forming the residual of the row's member m exactly as
// k_residual does (same terms, same order), then the members' residuals summed in
// ascending order as k_restrict_zero sums them, and the next level's zero-start sweep.
// The residual vector is never stored. Extra blocks past the rows solve the dense
// coarsest levels of planets whose coarsest level is this one, as k_residual's do.
constexpr int kWarpsPerBlock = kTile / 32;

template <typename T, int W>
__global__ void k_residual_restrict(LevelView<T> lv, LevelView<T> coarse, const std::uint32_t* __restrict__ moff,
                                    const std::uint32_t* __restrict__ member, const T* __restrict__ b,
                                    const T* __restrict__ x, T* __restrict__ bc, T* __restrict__ xc, T omega,
                                    const InstanceScalars* sc, int gate, DenseTask<T> dense) {
    const unsigned blocks = (coarse.rows + kWarpsPerBlock - 1) / kWarpsPerBlock;
    const int lane = static_cast<int>(threadIdx.x & 31);
    const int row = static_cast<int>(blockIdx.x) * kWarpsPerBlock + static_cast<int>(threadIdx.x >> 5);
    const std::uint32_t P = lv.rows;
    // Before the wait, what no kernel writes: the row's tile word, its member range, the
    // first 32 members and their columns (rows past 32 members load theirs in the loop).
    ph::TileSet<1> ts{};
    std::uint32_t k0 = 0, k1 = 0;
    int f0 = 0;
    int c0[W];
#pragma unroll
    for (int j = 0; j < W; ++j) c0[j] = 0;
    if (blockIdx.x < blocks) {
        ts = ph::tile_set<1>(coarse.tile_meta, coarse.tiles, row / kTile);
        k0 = moff[row];
        k1 = moff[row + 1];
        if (k0 + static_cast<std::uint32_t>(lane) < k1) {
            f0 = static_cast<int>(member[k0 + lane]);
#pragma unroll
            for (int j = 0; j < W; ++j) c0[j] = lv.col[j * P + f0];
        }
    }
    pdl_begin();
    if (blockIdx.x >= blocks) {
        ph::dense_block<T>(dense, blockIdx.x - blocks, threadIdx.x, sc, gate);
        return;
    }
    if (row % kTile >= ts.rows[0] || !ph::gate_open(sc, ts.inst[0], gate)) return;   // the whole warp
    T s = T(0);
    unsigned moved = 0;
    for (std::uint32_t base = k0; base < k1; base += 32) {
        const std::uint32_t k = base + static_cast<std::uint32_t>(lane);
        T rm = T(0);
        if (k < k1) {
            const bool first = base == k0;
            const int f = first ? f0 : static_cast<int>(member[k]);
            rm = b[f] - lv.vd[W * P + f] * x[f];
#pragma unroll
            for (int j = 0; j < W; ++j) rm -= lv.vd[j * P + f] * x[first ? c0[j] : lv.col[j * P + f]];
            moved += 4u * W + static_cast<unsigned>(sizeof(T)) * (W + 3u) + 4u;
        }
        const int n = static_cast<int>(k1 - base < 32u ? k1 - base : 32u);
        for (int i = 0; i < n; ++i) s += __shfl_sync(0xffffffffu, rm, i);
    }
    if (lane == 0) {
        bc[row] = s;
        if (ts.sweep[0]) xc[row] = omega * coarse.inv[row] * s;
        moved += 4u + 3u * static_cast<unsigned>(sizeof(T));
    }
    ph::count_bytes_warp(coarse.bytes, moved);
}

template <typename T, int W, int R>
__global__ void __launch_bounds__(kTile, 8) k_prolong_smooth(LevelView<T> lv, const std::int32_t* __restrict__ agg,
                                 const T* __restrict__ e, const T* __restrict__ b, const T* __restrict__ x,
                                 T* __restrict__ y, T omega, const InstanceScalars* sc, int gate) {
    ph::prefetch_static<T, W, R>(lv, blockIdx.x * R, threadIdx.x);
#pragma unroll
    for (int k = 0; k < R; ++k)
        if (blockIdx.x * R + k < lv.tiles) ph::prefetch_l1(agg + (blockIdx.x * R + k) * kTile + threadIdx.x);
    pdl_begin();
    ph::prolong_smooth<T, W, R>(lv, blockIdx.x * R, threadIdx.x, agg, e, b, x, y, omega, sc, gate);
}

template <typename T, int R>
__global__ void k_prolong(LevelView<T> lv, const std::int32_t* __restrict__ agg, const T* __restrict__ xc,
                          T* __restrict__ x, const InstanceScalars* sc, int gate) {
    ph::prefetch_meta(lv, blockIdx.x * R, threadIdx.x);
#pragma unroll
    for (int k = 0; k < R; ++k)
        if (blockIdx.x * R + k < lv.tiles) ph::prefetch_l1(agg + (blockIdx.x * R + k) * kTile + threadIdx.x);
    pdl_begin();
    ph::prolong<T, R>(lv, blockIdx.x * R, threadIdx.x, agg, xc, x, sc, gate);
}

// Coarsest level: x = A^-1 b, one warp per row, eight rows per block.
template <typename T>
__global__ void k_dense_solve(DenseTask<T> dense, const InstanceScalars* sc, int gate) {
    if (threadIdx.x == 0) ph::prefetch_l1(dense.blocks + blockIdx.x);
    pdl_begin();
    ph::dense_block<T>(dense, blockIdx.x, threadIdx.x, sc, gate);
}



}  // namespace


// ---- launchers -----------------------------------------------------------------

// Jacobi sweeps, residuals and prolongations are accounted as fine-level or coarse-level
// launches; a restriction by the level it restricts onto (level 1: from the fine level).
template <typename T>
inline int smooth_family(const LevelView<T>& lv) { return lv.level == 0 ? kFamSmooth : kFamSmoothCoarse; }
template <typename T>
inline int residual_family(const LevelView<T>& lv) { return lv.level == 0 ? kFamResidual : kFamResidualCoarse; }
template <typename T>
inline int restrict_family(const LevelView<T>& coarse) { return coarse.level <= 1 ? kFamRestrict : kFamRestrictCoarse; }
template <typename T>
inline int prolong_family(const LevelView<T>& lv) { return lv.level == 0 ? kFamProlong : kFamProlongCoarse; }


void launch_assemble_transport(const LevelView<double>& fine, const double* w, const double* wsum,
                               const double* area, const double* slope, const double* conductance,
                               const double* edge_conductance, double* vd, cudaStream_t stream) {
    PSGB_LAUNCH(kFamSetup, stream, launch_pdl(k_assemble_transport, fine.tiles, kTile, stream, fine, w, wsum, area, slope, conductance,
                                                          edge_conductance, vd));
}

void launch_set_matrix_csr(std::uint32_t n, std::uint32_t rows, std::uint32_t width,
                           const std::uint32_t* csr_offset, const double* diag, const double* off,
                           double* vd, cudaStream_t stream) {
    PSGB_LAUNCH(kFamSetup, stream, launch_pdl(k_set_matrix_csr, (rows + 255) / 256, 256, stream, n, rows, width, csr_offset, diag, off, vd));
}

void launch_galerkin(std::uint32_t lists, const std::uint32_t* offset, const std::uint32_t* source,
                     const double* fine_vd, double* coarse_vd, cudaStream_t stream) {
    PSGB_LAUNCH(kFamSetup, stream, launch_pdl(k_galerkin, (lists + 255) / 256, 256, stream, lists, offset, source, fine_vd, coarse_vd));
}

void launch_finalize_level(std::uint32_t rows, std::uint32_t width, double* vd64, float* vd32,
                           double* inv64, float* inv32, cudaStream_t stream) {
    PSGB_LAUNCH(kFamSetup, stream, launch_pdl(k_finalize_level, (rows + 255) / 256, 256, stream, rows, width, vd64, vd32, inv64, inv32));
}

void launch_dense_invert(const DenseView& dense, int level, const LevelView<double>& lv,
                         double* work, double* inv64, float* inv32, cudaStream_t stream) {
    PSGB_LAUNCH(kFamSetup, stream, launch_pdl(k_dense_invert, dense.instances, 1024, stream, dense, level, lv, work, inv64, inv32));
}

template <typename T>
void launch_smooth_zero(const LevelView<T>& lv, const T* b, T* x, T omega, const InstanceScalars* sc,
                        int gate, cudaStream_t stream) {
    PSGB_LAUNCH(smooth_family(lv), stream,
                PSGB_VECTOR_SETS(lv.sets_vector, launch_pdl(k_smooth_zero<T, R>, ph::tile_sets(lv.tiles, R), kTile, stream,
                                                            counted(lv, smooth_family(lv)), b, x, omega, sc, gate)));
}

template <typename T>
void launch_smooth(const LevelView<T>& lv, const T* b, const T* x, T* y, T omega,
                   const InstanceScalars* sc, int gate, cudaStream_t stream, const DenseTask<T>& dense, int inner) {
    if (inner > 1) {
        PSGB_LAUNCH(smooth_family(lv), stream,
                    PSGB_WIDTHS(lv.width, launch_pdl(k_smooth_block<T, W>, lv.tiles + dense.count, kTile, stream,
                                                     counted(lv, smooth_family(lv)), b, x, y, omega, inner, sc, gate,
                                                     dense)));
        return;
    }
    PSGB_LAUNCH(smooth_family(lv), stream,
                PSGB_STENCIL_SETS(lv.sets_stencil, PSGB_WIDTHS(lv.width,
                    launch_pdl(k_smooth<T, W, R>, ph::tile_sets(lv.tiles, R) + dense.count, kTile, stream,
                               counted(lv, smooth_family(lv)), b, x, y, omega, sc, gate, dense))));
}

template <typename T>
void launch_residual(const LevelView<T>& lv, const T* b, const T* x, T* r, const InstanceScalars* sc,
                     int gate, cudaStream_t stream, const DenseTask<T>& dense) {
    PSGB_LAUNCH(residual_family(lv), stream,
                PSGB_STENCIL_SETS(lv.sets_stencil, PSGB_WIDTHS(lv.width,
                    launch_pdl(k_residual<T, W, R>, ph::tile_sets(lv.tiles, R) + dense.count, kTile, stream,
                               counted(lv, residual_family(lv)), b, x, r, sc, gate, dense))));
}

template <typename T>
void launch_spmv(const LevelView<T>& lv, const T* x, T* y, cudaStream_t stream) {
    PSGB_LAUNCH(kFamKrylovSpmv, stream,
                PSGB_STENCIL_SETS(lv.sets_stencil, PSGB_WIDTHS(lv.width,
                    launch_pdl(k_spmv<T, W, R>, ph::tile_sets(lv.tiles, R), kTile, stream, counted(lv, kFamKrylovSpmv),
                               x, y))));
}

template <typename T>
void launch_restrict(const LevelView<T>& coarse, const std::uint32_t* member_offset,
                     const std::uint32_t* member, const T* r, T* bc, const InstanceScalars* sc,
                     int gate, cudaStream_t stream) {
    PSGB_LAUNCH(restrict_family(coarse), stream,
                launch_pdl(k_restrict<T>, ph::tile_sets(coarse.tiles, ph::kRowsCoarse), kTile, stream,
                           counted(coarse, restrict_family(coarse)), member_offset, member, r, bc, sc, gate));
}

template <typename T>
void launch_restrict_zero(const LevelView<T>& coarse, const std::uint32_t* member_offset,
                          const std::uint32_t* member, const T* r, T* bc, T* xc, T omega,
                          const InstanceScalars* sc, int gate, cudaStream_t stream) {
    PSGB_LAUNCH(restrict_family(coarse), stream,
                launch_pdl(k_restrict_zero<T>, ph::tile_sets(coarse.tiles, ph::kRowsCoarse), kTile, stream,
                           counted(coarse, restrict_family(coarse)), member_offset, member, r, bc, xc, omega, sc, gate));
}

template <typename T>
void launch_residual_restrict(const LevelView<T>& lv, const LevelView<T>& coarse, const std::uint32_t* member_offset,
                              const std::uint32_t* member, const T* b, const T* x, T* bc, T* xc, T omega,
                              const InstanceScalars* sc, int gate, cudaStream_t stream, const DenseTask<T>& dense) {
    const unsigned blocks = (coarse.rows + kWarpsPerBlock - 1) / kWarpsPerBlock;
    PSGB_LAUNCH(kFamRestrictCoarse, stream,
                PSGB_WIDTHS(lv.width,
                    launch_pdl(k_residual_restrict<T, W>, blocks + dense.count, kTile, stream, lv,
                               counted(coarse, kFamRestrictCoarse), member_offset, member, b, x, bc, xc, omega, sc,
                               gate, dense)));
}

template <typename T>
void launch_prolong_smooth(const LevelView<T>& lv, const std::int32_t* agg, const T* e, const T* b, const T* x,
                           T* y, T omega, const InstanceScalars* sc, int gate, cudaStream_t stream) {
    PSGB_LAUNCH(smooth_family(lv), stream,
                PSGB_STENCIL_SETS(lv.sets_stencil, PSGB_WIDTHS(lv.width,
                    launch_pdl(k_prolong_smooth<T, W, R>, ph::tile_sets(lv.tiles, R), kTile, stream,
                               counted(lv, smooth_family(lv)), agg, e, b, x, y, omega, sc, gate))));
}

template <typename T>
void launch_prolong(const LevelView<T>& fine, const std::int32_t* agg, const T* xc, T* x,
                    const InstanceScalars* sc, int gate, cudaStream_t stream) {
    PSGB_LAUNCH(prolong_family(fine), stream,
                PSGB_VECTOR_SETS(fine.sets_vector, launch_pdl(k_prolong<T, R>, ph::tile_sets(fine.tiles, R), kTile, stream,
                                                              counted(fine, prolong_family(fine)), agg, xc, x, sc, gate)));
}

template <typename T>
void launch_dense_solve(const DenseTask<T>& dense, const InstanceScalars* sc, int gate, cudaStream_t stream) {
    if (dense.count == 0) return;
    DenseTask<T> task = dense;
    task.bytes = profile_bytes_for(kFamDense);
    PSGB_LAUNCH(kFamDense, stream, launch_pdl(k_dense_solve<T>, dense.count, 256, stream, task, sc, gate));
}

#define PSGB_INSTANTIATE(T)                                                                           \
    template void launch_smooth_zero<T>(const LevelView<T>&, const T*, T*, T, const InstanceScalars*, \
                                        int, cudaStream_t);                                           \
    template void launch_smooth<T>(const LevelView<T>&, const T*, const T*, T*, T,                     \
                                   const InstanceScalars*, int, cudaStream_t, const DenseTask<T>&, int); \
    template void launch_residual<T>(const LevelView<T>&, const T*, const T*, T*,                      \
                                     const InstanceScalars*, int, cudaStream_t, const DenseTask<T>&); \
    template void launch_spmv<T>(const LevelView<T>&, const T*, T*, cudaStream_t);                     \
    template void launch_restrict<T>(const LevelView<T>&, const std::uint32_t*, const std::uint32_t*,  \
                                     const T*, T*, const InstanceScalars*, int, cudaStream_t);        \
    template void launch_restrict_zero<T>(const LevelView<T>&, const std::uint32_t*, const std::uint32_t*, \
                                          const T*, T*, T*, T, const InstanceScalars*, int, cudaStream_t); \
    template void launch_residual_restrict<T>(const LevelView<T>&, const LevelView<T>&, const std::uint32_t*,   \
                                              const std::uint32_t*, const T*, const T*, T*, T*, T,             \
                                              const InstanceScalars*, int, cudaStream_t, const DenseTask<T>&); \
    template void launch_prolong_smooth<T>(const LevelView<T>&, const std::int32_t*, const T*, const T*,    \
                                           const T*, T*, T, const InstanceScalars*, int, cudaStream_t);    \
    template void launch_prolong<T>(const LevelView<T>&, const std::int32_t*, const T*, T*,            \
                                    const InstanceScalars*, int, cudaStream_t);                       \
    template void launch_dense_solve<T>(const DenseTask<T>&, const InstanceScalars*, int, cudaStream_t);

PSGB_INSTANTIATE(float)
PSGB_INSTANTIATE(double)

}  // namespace psgb

// Kernel-side views and host launchers of the GB300 heat-transport kernels.
// Only POD views cross this boundary; ownership stays with Planet/Batch.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace psgb {

// Per-planet solver scalars, device-resident, FP64 for every precision.
struct InstanceScalars {
    double rho, alpha, omega, beta;
    double b_norm, target, r_norm, s_norm;
    double outer_b_norm, outer_target, outer_r_norm, tolerance;
    int status;          // Status of the current (inner) Krylov solve
    int half_done;       // BiCGSTAB converged at s: finish with x += alpha p_hat
    int iterations;      // Krylov iterations of the current solve
    int max_iterations;
    int outer_status;    // Status of the FP64 refinement
    int refinements;
    int inner_total;     // Krylov iterations summed over refinements
    int first;           // PCG: first iteration
};

// Tile word: planet (bits 0-21), valid rows 0..256 (bits 22-30), smooths here (bit 31).
constexpr std::uint32_t kMaxInstances = 1u << 22;
inline constexpr std::uint32_t pack_tile(std::int32_t inst, std::int32_t rows, bool sweep) {
    return static_cast<std::uint32_t>(inst) | (static_cast<std::uint32_t>(rows) << 22) | (sweep ? 0x80000000u : 0u);
}

enum Status : int { kRunning = 0, kConverged = 1, kBreakdown = 2, kNonFinite = 3, kCap = 4 };

// Gates: which planets a launch works for.
enum Gate : int {
    kGateAlways = 0,       // every planet (stand-alone preconditioner, assembly)
    kGateRunning = 1,      // planets whose current solve is still running
    kGateSecondHalf = 2,   // running and not already converged at BiCGSTAB's s
    kGateOuter = 3,        // planets whose FP64 refinement is still running
};

// One multigrid level of a batch: ELL slot-major values then diagonal in `vd`
// ((width + 1) * rows entries), `inv` = 1 / diagonal.
template <typename T>
struct LevelView {
    std::uint32_t rows;          // padded
    std::uint32_t width;         // 6, 8, 12 or 16
    std::uint32_t tiles;
    const std::int32_t* col;
    const T* vd;
    const T* inv;
    const std::int32_t* tile_inst;
    const std::int32_t* tile_rows;    // valid rows per tile
    const std::uint8_t* tile_sweep;   // 1: the tile's planet smooths on this level
    const std::uint32_t* tile_meta;   // the three above in one word (pack_tile), padded to 4 tiles
    unsigned long long* bytes;        // algorithmic-byte counter while profiling, else null
    std::uint8_t sets_stencil;        // tiles per tile set of the stencil launches (1 or 2)
    std::uint8_t sets_vector;         // tiles per tile set of the vector launches (1 or 4)
    std::uint8_t level;               // multigrid level (0: fine)
    T correction = T(1);              // scale of the coarse-grid correction prolongated into this level
    // Columns shared by the planets of one mesh level (null: `col` holds every planet's own
    // columns). The planets of a mesh level have the same graph, so their planet-local
    // columns are stored once per distinct graph, slot-major with pitch `spitch`; a tile's
    // shift gives its planet's first row (x, added to a local column) and that row minus
    // the graph's first row in `scol` (y, taken from the row index).
    const std::int32_t* scol = nullptr;
    const int2* tile_shift = nullptr;
    std::uint32_t spitch = 0;
};

struct ReduceCtx {
    double* partial;                  // [tiles][8]
    unsigned* ticket;                 // [instances]
    const std::uint32_t* tile_begin;  // [instances + 1] fine-level tile ranges
    InstanceScalars* sc;
    std::uint32_t instances;
};

struct DenseView {
    std::uint32_t instances;
    const std::int32_t* level;        // coarsest level per planet
    const std::uint64_t* offset;      // inverse offset per planet
    const std::uint32_t* size;        // rows per planet
    const std::int64_t* row_base;     // row base per planet at its coarsest level
};

// Coarsest-level solves x = A^-1 b of the planets whose coarsest level is one level:
// `count` blocks of eight rows, (planet, first row) each; one warp per row. A launch on
// that level (smoothing of the other planets) may carry them in extra blocks.
template <typename T>
struct DenseTask {
    DenseView dense;
    const int2* blocks;
    std::uint32_t count;              // 0: no dense work
    const T* inv;
    const T* b;
    T* x;
    unsigned long long* bytes = nullptr;   // algorithmic-byte counter while profiling, else null
};

// ---- multigrid.cu ---------------------------------------------------------
// Fine-level matrix of the implicit heat step (heat_transport.cpp:351-363):
// diag = A/s + K Σw (s > 0) else 1; off = -K w where both ends are free.
// `conductance` holds one K per planet; `edge_conductance` (optional, slot-major
// like w) replaces K per directed entry.
void launch_assemble_transport(const LevelView<double>& fine, const double* w, const double* wsum,
                               const double* area, const double* slope, const double* conductance,
                               const double* edge_conductance, double* vd, cudaStream_t stream);
// set_matrix from a CSR diagonal/off-diagonal pair (one planet, rows = n).
void launch_set_matrix_csr(std::uint32_t n, std::uint32_t rows, std::uint32_t width,
                           const std::uint32_t* csr_offset, const double* diag, const double* off,
                           double* vd, cudaStream_t stream);
void launch_galerkin(std::uint32_t lists, const std::uint32_t* offset, const std::uint32_t* source,
                     const double* fine_vd, double* coarse_vd, cudaStream_t stream);
void launch_finalize_level(std::uint32_t rows, std::uint32_t width, double* vd64, float* vd32,
                           double* inv64, float* inv32, cudaStream_t stream);
void launch_dense_invert(const DenseView& dense, int level, const LevelView<double>& lv,
                         double* work, double* inv64, float* inv32, cudaStream_t stream);

template <typename T>
void launch_smooth_zero(const LevelView<T>& lv, const T* b, T* x, T omega, const InstanceScalars* sc,
                        int gate, cudaStream_t stream);
// `inner` > 1: block-local sweeps (each tile `inner` Jacobi sweeps in one launch).
template <typename T>
void launch_smooth(const LevelView<T>& lv, const T* b, const T* x, T* y, T omega,
                   const InstanceScalars* sc, int gate, cudaStream_t stream, const DenseTask<T>& dense = {},
                   int inner = 1);
template <typename T>
void launch_residual(const LevelView<T>& lv, const T* b, const T* x, T* r, const InstanceScalars* sc,
                     int gate, cudaStream_t stream, const DenseTask<T>& dense = {});
template <typename T>
void launch_restrict(const LevelView<T>& coarse, const std::uint32_t* member_offset,
                     const std::uint32_t* member, const T* r, T* bc, const InstanceScalars* sc,
                     int gate, cudaStream_t stream);
template <typename T>
void launch_restrict_zero(const LevelView<T>& coarse, const std::uint32_t* member_offset,
                          const std::uint32_t* member, const T* r, T* bc, T* xc, T omega,
                          const InstanceScalars* sc, int gate, cudaStream_t stream);
// A coarse level's residual fused with the restriction into the next level and that
// level's zero-start sweep (same bits as launch_residual then launch_restrict_zero; the
// residual is not stored), with the dense blocks of launch_residual.
template <typename T>
void launch_residual_restrict(const LevelView<T>& lv, const LevelView<T>& coarse, const std::uint32_t* member_offset,
                              const std::uint32_t* member, const T* b, const T* x, T* bc, T* xc, T omega,
                              const InstanceScalars* sc, int gate, cudaStream_t stream, const DenseTask<T>& dense);
template <typename T>
void launch_prolong_smooth(const LevelView<T>& lv, const std::int32_t* agg, const T* e, const T* b, const T* x,
                           T* y, T omega, const InstanceScalars* sc, int gate, cudaStream_t stream);
template <typename T>
void launch_prolong(const LevelView<T>& fine, const std::int32_t* agg, const T* xc, T* x,
                    const InstanceScalars* sc, int gate, cudaStream_t stream);
template <typename T>
void launch_dense_solve(const DenseTask<T>& dense, const InstanceScalars* sc, int gate, cudaStream_t stream);
template <typename T>
void launch_spmv(const LevelView<T>& lv, const T* x, T* y, cudaStream_t stream);



}  // namespace psgb

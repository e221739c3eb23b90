// Host driver of the GB300 transport solve: planets, batches, V-cycle, Krylov loops.
#pragma once

#include "operators.hpp"
#include "planet.hpp"

#include <memory>
#include <vector>

namespace psgb {

enum Precision : int { kFP64 = 0, kMixed = 1 };
enum Method : int { kPCG = 0, kBiCGSTAB = 1 };
enum Schedule : int { kScheduleAuto = 0, kScheduleKernels = 1, kSchedulePersistent = 2 };

struct SolveOptions {
    int precision = kFP64;
    int method = kBiCGSTAB;
    double tolerance = 1e-10;          // ||b - A x|| <= tolerance ||b|| (FP64 residual)
    double inner_tolerance = 1e-4;     // mixed: relative reduction per refinement
    int max_iterations = 1000;         // Krylov iterations per inner solve
    int max_refinements = 20;
    int poll = 4;                      // Krylov iterations between status reads
    int schedule = kScheduleAuto;      // persistent kernel or one kernel per phase
};

// Host-side mesh, graph and hierarchy; no device memory is touched.
// `agglomerated`: the transport graph one mesh level coarser (agglomerated_transport_graph).
std::unique_ptr<Planet> make_planet(std::uint32_t level, double radius_m, bool agglomerated = false);
// Uploads the operator geometry to HBM (idempotent).
void upload_planet(Planet& planet);

std::unique_ptr<Batch> make_batch(const std::vector<Planet*>& planets);
// The same batch with every device array placed in caller-provided device memory
// [arena, arena + arena_bytes): no device or pinned allocation, no stream, event or graph
// creation; the solver then runs directly on the caller's stream.
std::unique_ptr<Batch> make_batch_in(const std::vector<Planet*>& planets, void* arena, std::size_t arena_bytes);

// Default tiles per thread of every level's launches (from its tile count).
void default_launch_shapes(Batch& b);

// The fine-level (padded) row base of planet i inside the batch.
inline std::int64_t fine_base(const Batch& b, std::size_t i) { return b.fine_base[i]; }

LevelView<double> view64(const Batch& b, std::size_t level);
LevelView<float> view32(const Batch& b, std::size_t level);

// Matrix of the implicit step on every planet; `slope`, `conductance` and
// `edge_conductance` are device arrays in the batch's fine layout.
void assemble_transport(Batch& b, const double* slope, const double* conductance,
                        const double* edge_conductance, cudaStream_t st);
// One planet's matrix from the reference's CSR diagonal/off-diagonal form (device arrays).
void set_matrix_csr(Batch& b, const double* diag, const double* off, cudaStream_t st);
// Galerkin values on every level, the coarsest inverses, FP32 copies.
void prepare_levels(Batch& b, cudaStream_t st);

template <typename T>
void vcycle(Batch& b, const T* rhs, T* x, int gate, bool first_sweep_done, cudaStream_t st);
template <typename T>
T* vcycle_first_target(Batch& b, T* x);

// Solve A x = rhs for every planet (FP64 device vectors, fine layout). `x` holds
// the initial guess on entry. Host copies of the per-planet scalars land in
// b.host_scalars.
void solve(Batch& b, const SolveOptions& opt, const double* rhs, double* x, cudaStream_t st);

// The fine level of a batch as the transport-step kernels see it.
StepView step_view(const Batch& b);

// The levels from `level` down fit the shared-memory coarse tail in precision T.
template <typename T>
bool tail_fits_shared(const Batch& b, int level);

// Rows of each vector one block of a `cluster`-block cluster holds for the largest planet
// (per level from `level` down, the planet's tiles shared out over the cluster).
unsigned tail_cluster_rows(const Batch& b, int level, unsigned cluster);
// The levels from `level` down fit clusters of `cluster` blocks in precision T.
template <typename T>
bool tail_fits_cluster(const Batch& b, int level, unsigned cluster);

// The form the coarse tail of a solve in precision T takes: the batch's choice where it
// fits, else the next one down (cluster, shared memory, spread, one block per planet).
enum class TailForm { kNone, kBlock, kSpread, kShared, kCluster };
template <typename T>
TailForm tail_form(const Batch& b);

}  // namespace psgb

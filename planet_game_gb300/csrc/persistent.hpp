// The persistent cooperative solver: one launch runs a whole FP64-refined Krylov solve
// (every refinement, every inner iteration, every V-cycle level) for all planets of a
// batch. Arguments are plain device pointers and views, filled by the host driver.
#pragma once

#include "kernels.hpp"

#include <cuda_runtime.h>

#include <cstdint>

namespace psgb {

constexpr int kMaxLevels = 12;

// Grid-barrier state: arrival count, generation, error flag (three device words).
struct PersistentSync {
    unsigned* count;
    unsigned* gen;
    unsigned* error;   // 1: a barrier wait ran past its iteration limit
};

template <typename T>
struct PersistentLevel {
    LevelView<T> view;
    T* x;                               // level iterate (level 0: unused, the solve's vector)
    T* y;                               // ping-pong partner
    T* b;                               // restricted right-hand side (levels >= 1)
    T* r;                               // residual (levels < depth - 1)
    const std::uint32_t* member_offset; // aggregates of the next coarser level
    const std::uint32_t* member;
    const std::int32_t* agg;            // fine row -> aggregate of the next coarser level
};

template <typename T>
struct PersistentArgs {
    PersistentLevel<T> level[kMaxLevels];
    unsigned char dense_at[kMaxLevels]; // some planet's coarsest level is this one
    int depth;
    DenseView dense;
    const T* dense_inv;
    const int2* dense_blocks;           // blocks of eight coarsest rows, (planet, first row)
    unsigned dense_block_offset[kMaxLevels + 1];   // per level, into dense_blocks
    LevelView<double> fine64;           // FP64 fine matrix (refinement residual)
    const double* rhs64;
    double* x64;
    double* r64;
    T* k[10];                           // Krylov vectors; k[8] inner rhs, k[9] inner solution
    ReduceCtx ctx;
    InstanceScalars* sc;
    unsigned instances;
    const std::uint8_t* active;         // planets taking part (null: all)
    double tolerance;                   // outer: ||b - A x|| <= tolerance ||b||
    double inner_tolerance;
    int max_iterations;
    int max_refinements;
    int method;                         // psgb::Method
    int pre[kMaxLevels], post[kMaxLevels];   // sweeps per level
    int inner[kMaxLevels];                   // block-local sweeps per smoothing pass
    unsigned char starts_in_x[kMaxLevels];   // the level's first sweep writes x (sweep parity)
    T omega;
    PersistentSync sync;
};

// Cooperative launch on `st`, one 1024-thread block per SM. Throws if the device cannot
// run it (no cooperative launch, block does not fit). `serialize`: order the launch after
// the previous persistent solve of this process on the device, whatever its stream (an
// event per device, created on first use); callers that create no CUDA objects pass false
// and must not overlap solves themselves.
template <typename T>
void launch_persistent(const PersistentArgs<T>& args, cudaStream_t st, bool serialize);

// True when the persistent kernel fits one block per SM on the current device.
bool persistent_supported();

// The kernel's own entry points (instantiated for float and double, one translation
// unit each): co-resident 1024-thread blocks per SM, and the cooperative launch of
// `blocks` blocks on `st`.
template <typename T>
int persistent_kernel_blocks_per_sm();
template <typename T>
void persistent_kernel_launch(const PersistentArgs<T>& args, unsigned blocks, cudaStream_t st);

}  // namespace psgb

// The coarse tail of the V-cycle: from a level down to every planet's coarsest level and
// back up. Below the tail level every planet's level holds few rows, where a launch per
// phase costs more than the phase: the planet's blocks run all of its sweeps, residuals,
// restrictions, the dense coarsest solve and the prolongations with barriers in between.
// Either one 1024-thread block per planet (block barriers; the vectors in global or in
// shared memory), a cooperative launch in which each planet owns 1 to 16 co-resident
// blocks in proportion to its rows at the tail level, meeting at a per-planet barrier in
// global memory (bounded waits), or a thread-block cluster of 2, 4 or 8 blocks per planet
// holding the vectors in the cluster's distributed shared memory (hardware cluster
// barriers). Each phase is the same per-tile arithmetic as the grid-wide V-cycle, so the
// result is identical.
#pragma once

#include "coarse_tail_blocks.hpp"
#include "kernels.hpp"
#include "persistent.hpp"

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace psgb {

template <typename T>
struct TailArgs {
    PersistentLevel<T> level[kMaxLevels];   // vectors and transitions per level (x, y, b, r, agg, members)
    const std::uint32_t* tile_range;         // [levels][instances][2]: first tile, tile count
    int first;                               // the tail level (>= 1)
    int depth;
    unsigned instances;
    DenseView dense;
    const T* dense_inv;
    int pre[kMaxLevels], post[kMaxLevels], inner[kMaxLevels];
    unsigned char starts_in_x[kMaxLevels];
    T omega;
    const InstanceScalars* sc;
    int gate;
    // per-planet blocks (null: one block per planet)
    const std::uint32_t* cta;   // per block: planet | rank << 16 | size << 24
    unsigned ctas;
    unsigned* barrier;          // [2][instances]: arrivals, generation
    unsigned* error;            // set when a barrier wait runs past its limit
    // one block per planet with the tail levels' vectors in shared memory: the largest
    // planet's padded rows summed over the tail levels (0: vectors in global memory); with
    // a cluster, the largest planet's rows per block
    unsigned shared_rows;
    // blocks of the thread-block cluster of each planet (0: no cluster), the vectors spread
    // over the cluster's shared memory
    unsigned cluster;
};

// Co-resident 1024-thread tail blocks on this device (0: no cooperative launch).
unsigned tail_block_budget();
// Dynamic shared memory a shared-memory tail block may take on this device (0: none).
template <typename T>
unsigned tail_shared_max_bytes();

template <typename T>
void launch_coarse_tail(const TailArgs<T>& args, cudaStream_t st);

// Dynamic shared memory a block of the cluster tail may take (0: no cluster launch).
template <typename T>
unsigned cluster_tail_max_bytes();
// Clusters of `cluster` blocks (2, 4 or 8) holding `rows_per_block` rows of each of the
// four vectors per block fit in shared memory and can be resident on this device.
template <typename T>
bool cluster_tail_fits(unsigned cluster, unsigned rows_per_block);
template <typename T>
void launch_coarse_cluster(const TailArgs<T>& args, cudaStream_t st);

}  // namespace psgb

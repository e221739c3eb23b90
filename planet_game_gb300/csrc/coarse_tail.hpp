// The coarse tail of the V-cycle: from a level down to every planet's coarsest level and
// back up, one 1024-thread block per planet. Below the tail level every planet's level
// holds a few thousand rows at most, where a launch per phase costs more than the phase:
// the block runs all of its planet's sweeps, residuals, restrictions, the dense coarsest
// solve and the prolongations with block barriers in between. Each phase is the same
// per-tile code as the grid-wide V-cycle, so the result is identical.
#pragma once

#include "kernels.hpp"
#include "persistent.hpp"

#include <cuda_runtime.h>

#include <cstdint>

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
};

template <typename T>
void launch_coarse_tail(const TailArgs<T>& args, cudaStream_t st);

}  // namespace psgb

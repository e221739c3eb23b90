// Per-level autotuner of a batch: launch shapes (tiles per thread of the stencil and
// vector launches, which never change a result) and damped-Jacobi sweeps per level
// (which change the preconditioner, so they are chosen by timing whole solves that must
// still meet their tolerance).
#pragma once

#include "solver.hpp"

#include <vector>

namespace psgb {

struct Tuning {
    std::vector<int> pre, post;                    // sweeps per level
    std::vector<int> inner;                        // block-local sweeps per smoothing launch, per level
    std::vector<std::uint8_t> sets_stencil;        // per level: 1 or 2
    std::vector<std::uint8_t> sets_vector;         // per level: 1 or 4
    double omega = 0.8;
    double correction = 1.0;                       // coarse-grid correction scale
    int tail_level = 0;                            // coarse tail from this level (0: none)
    bool tail_spread = true;                       // several blocks per large planet in the tail
    bool tail_shared = false;                      // one block per planet, the tail levels' vectors in shared memory
    unsigned tail_cluster = 0;                     // blocks of a cluster per planet (2, 4, 8; 0: none), vectors in
                                                   // the cluster's distributed shared memory
    unsigned tail_blocks = 0;                      // blocks of the tail launch (out; 0: no tail)
    double tuned_ms = 0.0;                         // trial solve with the chosen settings
    double default_ms = 0.0;                       // trial solve with the settings before tuning
    int trials = 0;                                // trial solves timed
};

// Tunes `b` on the system its matrix holds with right-hand side `rhs` (device, fine
// layout), every trial solve starting from `x0` (the step's own initial guess, the
// temperature before the step; null: zero); `x` is device scratch of the fine layout.
// Leaves the chosen settings applied (b.tuned) and returns them.
Tuning autotune(Batch& b, const SolveOptions& opt, const double* rhs, const double* x0, double* x, cudaStream_t st);

// The batch's current settings.
Tuning current_tuning(const Batch& b);

// Applies settings (from autotune, possibly cached from an earlier run); the sizes must
// match the batch's depth.
void apply_tuning(Batch& b, const Tuning& t);

// Back to uniform sweeps from the solve options and default launch shapes.
void clear_tuning(Batch& b);

}  // namespace psgb

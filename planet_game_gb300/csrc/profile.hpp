// Launch accounting and opt-in per-kernel timing.
//
// Every launcher calls launch_begin/launch_end around its kernel: launches are counted
// per kernel family, and while a profile is active for one family, a CUDA event pair is
// recorded on the launching stream around each of its launches. The host reads the
// summed device time after synchronising (psgb_profile_end in the C-ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace psgb {

enum KernelFamily : int {
    kFamSmooth = 0,      // fine-level Jacobi sweeps (k_smooth, k_smooth_zero, k_prolong_smooth)
    kFamResidual,        // V-cycle residual
    kFamRestrict,        // restriction
    kFamProlong,         // prolongation
    kFamDense,           // coarsest dense solve
    kFamKrylovSpmv,      // Krylov products with fused dots (bicg_v, bicg_t, pcg_q)
    kFamKrylovVector,    // Krylov vector updates with fused dots
    kFamRefine,          // FP64 refinement residual / update
    kFamSetup,           // assembly, Galerkin, dense inverse, level finalisation
    kFamStep,            // transport-step right-hand side and flux form
    kFamOperator,        // finite-volume operators
    kFamColumn,          // column radiation
    kFamPersistent,      // the persistent cooperative solve (one launch per solve)
    kFamSmoothCoarse,    // Jacobi sweeps of the coarse levels
    kFamResidualCoarse,  // V-cycle residual of the coarse levels
    kFamRestrictCoarse,  // restriction onto a level below the first coarse one
    kFamProlongCoarse,   // prolongation onto a coarse level
    kFamCount
};

const char* family_name(int family);
int family_of(const char* name);

void launch_begin(int family, cudaStream_t st);
void launch_end(int family, cudaStream_t st);

std::uint64_t launches_total();
std::uint64_t launches_of(int family);

// True while a profile is recording (launches then bypass CUDA graphs so that every
// launch of the profiled family gets its own event pair).
bool profile_active();
// Stream capture: launches are not counted while a graph is being recorded; each replay
// of a graph adds its kernel nodes instead.
void set_capturing(bool on);
void count_graph_kernels(std::uint64_t kernels);

// Device counter of the algorithmic bytes that the kernels of `family` move (each vector a
// kernel touches counted once per active row), while a profile of that family records;
// null otherwise. Allocated on the first profile_begin. Launchers pass it in the views of
// their launches.
unsigned long long* profile_bytes_for(int family);
std::uint64_t profile_bytes_exchange();

bool profile_begin(int family);
// Synchronises the recorded events; returns false if no profile was active.
bool profile_end(double* total_ms, std::uint64_t* launches);

}  // namespace psgb

#define PSGB_LAUNCH(family, stream, ...)           \
    do {                                           \
        ::psgb::launch_begin((family), (stream));  \
        __VA_ARGS__;                               \
        ::psgb::launch_end((family), (stream));    \
    } while (0)

// Host launchers of the finite-volume operator and transport-step kernels (operators.cu).
#pragma once

#include "host/insolation.hpp"
#include "planet.hpp"

namespace psgb {

// Sub-step-mean insolation per cell (insolation.cu), FP32 out.
void launch_substep_insolation(const DevMesh& m, const InsolationNodes& nodes, float* out, cudaStream_t st);

template <typename T>
void launch_laplacian(const DevMesh& m, const T* in, T* out, cudaStream_t st);
template <typename T>
void launch_gradient(const DevMesh& m, const T* in, T* east, T* north, cudaStream_t st);
template <typename T>
void launch_divergence(const DevMesh& m, const T* flux, T* out, cudaStream_t st);
// Agglomerated planets: node means of fine-cell fields (b, mean_b may be null) and fine
// cells taking their node's value.
void launch_group_mean(const DevMesh& m, const double* a, const double* b, double* mean_a, double* mean_b,
                       cudaStream_t st);
void launch_group_scatter(const DevMesh& m, const double* node_value, double* out, cudaStream_t st);
void launch_diffusion_source(const DevMesh& m, double conductance, const double* t, double* out,
                             cudaStream_t st);

// The fine level of a batch as the transport step sees it.
struct StepView {
    std::uint32_t rows, tiles, instances;
    const std::int32_t* tile_inst;
    const std::int32_t* tile_rows;
    const std::uint32_t* tile_begin;
    const std::int32_t* nbr;            // the fine level's ELL columns
    const double* w;
    const double* area;
    const double* conductance;          // [instances]
    const double* edge_conductance;     // [6][P] or null
    const double* slope_of;             // [instances] dt / C
    unsigned long long* bytes;          // algorithmic-byte counter while the step family is profiled
};

// Held rows (slope <= 0) solve x = 0, as the reference masks their residual
// (heat_transport.cpp:396-398).
void launch_mask_rhs(std::size_t n, const double* slope, double* rhs, cudaStream_t st);

void launch_step_rhs(const StepView& v, const double* t0, const double* src, double* rhs, double* slope,
                     double* x0, cudaStream_t st);
// sums: [instances][8] = sum A H, sum A|H|, sum A H T, sum A S, sum A|S|, sum A dT/s
void launch_step_finish(const StepView& v, const double* t, const double* t0, const double* src,
                        double* h, double* t_new, double* partial, double* sums, cudaStream_t st);

}  // namespace psgb

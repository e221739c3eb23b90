// Sub-step-mean insolation of the Earth-like development planet (input generation).
#pragma once

#include "mesh.hpp"

#include <cstdint>

namespace psgb {

// The sub-step's 16 Gauss-Legendre time nodes (substep_forcing.cpp:75-100): quadrature
// weight, sin and cos of the solar declination, incident flux (W/m^2).
struct InsolationNode {
    double weight, sin_dec, cos_dec, flux;
};
struct InsolationNodes {
    InsolationNode node[16];
};
InsolationNodes substep_forcing_nodes(std::int64_t substep);

void substep_mean_insolation(const HostMesh& mesh, std::int64_t substep, float* out);

}  // namespace psgb

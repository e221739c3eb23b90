// Sub-step-mean insolation of the Earth-like development planet (input generation).
#pragma once

#include "mesh.hpp"

#include <cstdint>

namespace psgb {

void substep_mean_insolation(const HostMesh& mesh, std::int64_t substep, float* out);

}  // namespace psgb

// Sub-step-mean top-of-atmosphere insolation per cell on the GPU (the source term's
// forcing input): compute_substep_mean_insolation (sim/planet/orbit/substep_forcing.cpp:
// 102-127) with daily_mean_insolation_W_m2 (:35-56) at the sub-step's 16 time nodes. The
// nodes (orbit, declination, flux) are the host's (host/insolation.cpp); each thread
// sums one cell's quadrature in node order, rounding as the reference (no FMA), and
// stores FP32. CUDA's acos and sin differ from the host library's by an ulp or two, so
// the stored values agree with the reference's to within one FP32 ulp.
#include "operators.hpp"
#include "profile.hpp"

#include <cuda_runtime.h>

namespace psgb {
namespace {

constexpr double kPi = 3.14159265358979323846;

__global__ void k_substep_insolation(std::uint32_t n, std::uint32_t P, const double* __restrict__ latitude,
                                     const __grid_constant__ InsolationNodes nodes, float* __restrict__ out) {
    const std::uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double sl = latitude[c], cl = latitude[P + c];
    double mean = 0.0;
#pragma unroll 4
    for (int k = 0; k < 16; ++k) {
        const InsolationNode& node = nodes.node[k];
        const double a = sl * node.sin_dec;
        const double b = cl * node.cos_dec;
        double h0 = 0.0;
        if (b <= 0.0) {
            h0 = a > 0.0 ? kPi : 0.0;
        } else {
            const double cosine = -a / b;
            if (cosine <= -1.0) h0 = kPi;
            else if (cosine < 1.0) h0 = acos(cosine);
        }
        const double value = node.flux / kPi * (h0 * a + b * sin(h0));
        mean += node.weight * (0.0 < value ? value : 0.0);
    }
    out[c] = static_cast<float>(mean);
}

}  // namespace

void launch_substep_insolation(const DevMesh& m, const InsolationNodes& nodes, float* out, cudaStream_t st) {
    PSGB_LAUNCH(kFamOperator, st, k_substep_insolation<<<(m.n + 255) / 256, 256, 0, st>>>(m.n, m.p, m.latitude, nodes, out));
}

}  // namespace psgb

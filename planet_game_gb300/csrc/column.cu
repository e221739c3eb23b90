// K12: per-cell grey column radiation for sm_103a.
//
// For every cell, N equal-mass sigma layers (N <= 16; the reference caps N at 8,
// sim/planet/atmosphere/atmosphere.hpp:85, the same formulas hold for any N):
//   emissivity   eps_k = -expm1(-(tau_d dp/p0 + kappa_v q_k dp/g))   (atmosphere_column.hpp:85-104)
//   cloud optics f_k, tau_k, R_k, kappa_l LWP_k, transmission, column fraction
//                                                                     (atmosphere_column.hpp:599-623)
//   cloud LW     eps_k' = -expm1(log1p(-eps_k) - kappa_l LWP_k)       (atmosphere_column.hpp:627-634)
//   two-stream   absorbed_k, downward surface LW, OLR                 (atmosphere_column.hpp:125-143)
// with layer emission eps_k sigma T_k^4 (atmosphere_column.hpp:918) and a black surface
// sigma Ts^4 below. FP64 throughout, in the reference's operation order; this file is
// compiled without FMA contraction, so only the math-library results of expm1/log1p can
// differ from the host's (by an ulp or so).
//
// Layout: layer-major [N][cells] arrays, one thread per cell, the column in registers.
#include "column.hpp"
#include "common.cuh"
#include "profile.hpp"

#include <stdexcept>

namespace psgb {
namespace {

template <int L>
__global__ void __launch_bounds__(128) k_column(std::uint32_t cells, ColumnConstants k,
                                                const double* __restrict__ temp, const double* __restrict__ hum,
                                                const double* __restrict__ cloud, const double* __restrict__ ts,
                                                const double* __restrict__ ps, double* __restrict__ emissivity,
                                                double* __restrict__ absorbed, double* __restrict__ fraction,
                                                double* __restrict__ reflectance, double* __restrict__ scalars) {
    const std::uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    const double p_s = ps[c];
    const double layer_pa = p_s / static_cast<double>(L);
    const double dry = k.dry_optical_depth * layer_pa / k.reference_pressure;
    const double mass = p_s / (k.gravity * static_cast<double>(L));
    const double omg = 1.0 - k.cloud_asymmetry;
    double eps[L], emis[L];
    double clear = 1.0, transmission = 1.0, col_tau = 0.0;
#pragma unroll
    for (int l = 0; l < L; ++l) {
        const std::size_t i = static_cast<std::size_t>(l) * cells + c;
        const double q = hum[i];
        const double vapour = (q > 0.0 ? q : 0.0) * layer_pa / k.gravity;
        double e = -expm1(-(dry + k.vapour_absorption * vapour));
        const double ql = cloud[i];
        const double path = (ql > 0.0 ? ql : 0.0) * mass;
        double f = 0.0, r = 0.0;
        if (path > 0.0) {
            const double ratio = path / k.in_cloud_water_path;
            f = ratio < 1.0 ? ratio : 1.0;
            const double tau = 3.0 * (path / f) / (2.0 * 1000.0 * k.effective_radius);
            clear *= 1.0 - f;
            r = f * omg * tau / (2.0 + omg * tau);
            transmission *= 1.0 - r;
            col_tau += f * tau;
            const double lw = k.cloud_longwave_absorption * path;
            if (lw > 0.0) e = -expm1(log1p(-e) - lw);
        }
        fraction[i] = f;
        reflectance[i] = r;
        eps[l] = e;
        emissivity[i] = e;
        const double t = temp[i];
        const double t2 = t * t;
        emis[l] = e * k.stefan_boltzmann * t2 * t2;
    }
    double above[L];
    double down = 0.0;
#pragma unroll
    for (int l = L - 1; l >= 0; --l) {
        above[l] = down;
        down = (1.0 - eps[l]) * down + emis[l];
    }
    const double tsc = ts[c];
    const double ts2 = tsc * tsc;
    double up = k.stefan_boltzmann * ts2 * ts2;
#pragma unroll
    for (int l = 0; l < L; ++l) {
        absorbed[static_cast<std::size_t>(l) * cells + c] = eps[l] * (up + above[l]);
        up = (1.0 - eps[l]) * up + emis[l];
    }
    scalars[c] = down;
    scalars[cells + c] = up;
    scalars[2 * static_cast<std::size_t>(cells) + c] = transmission;
    scalars[3 * static_cast<std::size_t>(cells) + c] = 1.0 - clear;
    scalars[4 * static_cast<std::size_t>(cells) + c] = col_tau;
}

}  // namespace

void launch_column_radiation(std::uint32_t cells, std::uint32_t layers, const ColumnConstants& k,
                             const double* temp, const double* hum, const double* cloud, const double* ts,
                             const double* ps, double* emissivity, double* absorbed, double* fraction,
                             double* reflectance, double* scalars, cudaStream_t st) {
    const dim3 grid((cells + 127) / 128), block(128);
#define PSGB_COLUMN_CASE(N) \
    case N: PSGB_LAUNCH(kFamColumn, st, (k_column<N><<<grid, block, 0, st>>>(cells, k, temp, hum, cloud, ts, ps, emissivity, absorbed, fraction, reflectance, scalars))); break;
    switch (layers) {
        PSGB_COLUMN_CASE(1) PSGB_COLUMN_CASE(2) PSGB_COLUMN_CASE(3) PSGB_COLUMN_CASE(4)
        PSGB_COLUMN_CASE(5) PSGB_COLUMN_CASE(6) PSGB_COLUMN_CASE(7) PSGB_COLUMN_CASE(8)
        PSGB_COLUMN_CASE(9) PSGB_COLUMN_CASE(10) PSGB_COLUMN_CASE(11) PSGB_COLUMN_CASE(12)
        PSGB_COLUMN_CASE(13) PSGB_COLUMN_CASE(14) PSGB_COLUMN_CASE(15) PSGB_COLUMN_CASE(16)
        default: throw std::invalid_argument("column radiation supports 1 to 16 layers");
    }
#undef PSGB_COLUMN_CASE
}

}  // namespace psgb

// Host launcher of the column-radiation kernel (column.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace psgb {

// Optical and physical constants of the column (the reference's AtmosphereParameters
// fields, sim/planet/atmosphere/atmosphere.hpp:22-83, plus g and sigma).
struct ColumnConstants {
    double dry_optical_depth;            // tau_d
    double vapour_absorption;            // kappa_v, m^2/kg
    double in_cloud_water_path;          // W_c, kg/m^2
    double effective_radius;             // r_e, m
    double cloud_asymmetry;              // g
    double cloud_longwave_absorption;    // kappa_l, m^2/kg
    double reference_pressure;           // p0, Pa
    double gravity;                      // m/s^2
    double stefan_boltzmann;             // W/m^2/K^4
};

void launch_column_radiation(std::uint32_t cells, std::uint32_t layers, const ColumnConstants& k,
                             const double* temp, const double* hum, const double* cloud, const double* ts,
                             const double* ps, double* emissivity, double* absorbed, double* fraction,
                             double* reflectance, double* scalars, cudaStream_t st);

}  // namespace psgb

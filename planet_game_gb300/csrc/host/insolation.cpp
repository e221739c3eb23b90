// Sub-step-mean top-of-atmosphere insolation (the source term's forcing input).
//
// Restates compute_substep_mean_insolation (sim/planet/orbit/substep_forcing.cpp:35-127):
// the climate sub-step [begin, end) of the orbital calendar
// (sim/core/scheduler/orbital_calendar.cpp), 16 Gauss-Legendre nodes in time, at each
// node the Kepler orbit (sim/planet/orbit/orbit_state.cpp: eccentric anomaly by 64
// bisection steps, true anomaly, solar longitude, declination, incident flux), and
// per cell the analytic daily mean Q = (S/pi)(h0 sin(lat) sin(dec) + cos(lat) cos(dec)
// sin h0). The Gauss-Legendre nodes and weights are computed here by Newton iteration
// on the Legendre polynomial, and the planet is the Earth-like development planet.
#include "insolation.hpp"

#include <algorithm>
#include <array>
#include <cmath>

namespace psgb {
namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kTwoPi = 2.0 * kPi;

struct Orbit {
    double orbital_period_s = 31'556'925.216;
    double sidereal_rotation_period_s = 86'164.0905;
    double axial_tilt_rad = 0.4090926006005829;
    double semi_major_axis_m = 149'597'870'700.0;
    double eccentricity = 0.0167086;
    double longitude_periapsis_rad = 3.14159265358979323846;
    double star_luminosity_W = 3.827531850364947e26;
    double initial_orbital_phase_rad = 0.0;
};

double wrap(double a) {
    double w = std::fmod(a, kTwoPi);
    if (w < 0.0) w += kTwoPi;
    return w;
}

// Gauss-Legendre nodes/weights on [-1, 1], n = 16, ascending.
void gauss_legendre(std::array<double, 16>& x, std::array<double, 16>& w) {
    const int n = 16;
    for (int i = 0; i < n; ++i) {
        double z = std::cos(kPi * (i + 0.75) / (n + 0.5));
        double dp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; ++k) {
                const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            const double dz = p1 / dp;
            z -= dz;
            if (std::abs(dz) < 1e-17) break;
        }
        x[n - 1 - i] = z;
        w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
    for (int i = 0; i < n / 2; ++i) {   // exact symmetry
        x[i] = -x[n - 1 - i];
        w[i] = w[n - 1 - i];
    }
}

using Node = InsolationNode;

Node orbit_at(const Orbit& o, double t, double weight) {
    const double mean = wrap(o.initial_orbital_phase_rad + kTwoPi * std::fmod(t, o.orbital_period_s) / o.orbital_period_s);
    double E = mean;
    if (!(mean == 0.0 || o.eccentricity == 0.0)) {
        double lo = 0.0, hi = kTwoPi;
        for (int i = 0; i < 64; ++i) {
            const double mid = 0.5 * (lo + hi);
            if (mid - o.eccentricity * std::sin(mid) - mean > 0.0) hi = mid; else lo = mid;
        }
        E = 0.5 * (lo + hi);
    }
    const double ce = std::cos(E), se = std::sin(E);
    const double radial = 1.0 - o.eccentricity * ce;
    const double distance = o.semi_major_axis_m * radial;
    const double cos_nu = (ce - o.eccentricity) / radial;
    const double sin_nu = std::sqrt(1.0 - o.eccentricity * o.eccentricity) * se / radial;
    const double nu = wrap(std::atan2(sin_nu, cos_nu));
    const double lambda = wrap(o.longitude_periapsis_rad + nu + kPi);
    const double cl = std::cos(lambda), sl = std::sin(lambda);
    const double ct = std::cos(o.axial_tilt_rad), st = std::sin(o.axial_tilt_rad);
    double sx = cl, sy = ct * sl, sz = st * sl;
    const double m = std::sqrt(sx * sx + sy * sy + sz * sz);
    sx /= m; sy /= m; sz /= m;
    const double dec = std::asin(std::clamp(sz, -1.0, 1.0));
    Node n;
    n.weight = weight;
    n.sin_dec = std::sin(dec);
    n.cos_dec = std::cos(dec);
    n.flux = o.star_luminosity_W / (4.0 * kPi * distance * distance);
    return n;
}

double daily_mean(double sl, double cl, double sd, double cd, double flux) {
    const double a = sl * sd;
    const double b = cl * cd;
    double h0 = 0.0;
    if (b <= 0.0) {
        h0 = a > 0.0 ? kPi : 0.0;
    } else {
        const double c = -a / b;
        if (c <= -1.0) h0 = kPi;
        else if (c < 1.0) h0 = std::acos(c);
    }
    const double v = flux / kPi * (h0 * a + b * std::sin(h0));
    return std::max(0.0, v);
}

}  // namespace

InsolationNodes substep_forcing_nodes(std::int64_t substep) {
    const Orbit o;
    const double per_year = 12.0;
    auto begin_tick = [&](std::int64_t k) {
        const double crossing = o.orbital_period_s * (static_cast<double>(k) / per_year - o.initial_orbital_phase_rad / kTwoPi);
        return std::ceil(crossing / 60.0);
    };
    const double t0 = begin_tick(substep) * 60.0;
    const double t1 = begin_tick(substep + 1) * 60.0;
    const double span = t1 - t0;
    std::array<double, 16> gx{}, gw{};
    gauss_legendre(gx, gw);
    InsolationNodes nodes{};
    for (int i = 0; i < 16; ++i) nodes.node[i] = orbit_at(o, t0 + 0.5 * span * (1.0 + gx[i]), 0.5 * gw[i]);
    return nodes;
}

void substep_mean_insolation(const HostMesh& mesh, std::int64_t substep, float* out) {
    const InsolationNodes nodes = substep_forcing_nodes(substep);
    for (std::size_t c = 0; c < mesh.cells; ++c) {
        const double x = mesh.center[3 * c], y = mesh.center[3 * c + 1], z = mesh.center[3 * c + 2];
        const double sl = z;
        const double cl = std::sqrt(x * x + y * y);
        double mean = 0.0;
        for (const Node& n : nodes.node) mean += n.weight * daily_mean(sl, cl, n.sin_dec, n.cos_dec, n.flux);
        out[c] = static_cast<float>(mean);
    }
}

}  // namespace psgb

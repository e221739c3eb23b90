// psgb_solve_implicit_transport: the implicit transport solve with a general tile response
// (sim/planet/surface/heat_transport.cpp:595-772, ImplicitTransportSettings and
// ImplicitTransportResult in heat_transport.hpp:82-119).
//
// Find sources h with F(h) = h - K lap(T(h)) (+ latent) = 0, where T(h) and its slope dT/dh
// come from the caller's response. The response stays on the host (one call per
// evaluation, host arrays); the GPU does the two-point Laplacians and every linear Newton
// system (A/s - K Q) dT = -A F, a multigrid-preconditioned Krylov solve. The outer loop
// follows the reference: a backtracking line search on the merit sum A F^2 with the
// iterate kept at or above the floor, a bounded number of full steps across kinks when
// no descent is found above the rounding floor, and the conservative flux form of the
// last iterate's temperatures as the transport applied. Reductions run over the mesh's
// 256-cell blocks in block order, as the reference's deterministic reductions do.
#include "../../include/planetsim_gb300.h"
#include "capi_internal.hpp"

#include <algorithm>
#include <cmath>
#include <limits>
#include <stdexcept>
#include <utility>
#include <vector>

namespace {

using psgb::capi::guarded;

constexpr std::size_t kBlock = 256;

void require(bool ok, const char* what) {
    if (!ok) throw std::invalid_argument(what);
}

// Block-ordered sum: per 256-cell block in cell order, then the blocks in order.
template <typename F>
double block_sum(std::size_t n, F&& term) {
    double total = 0.0;
    for (std::size_t begin = 0; begin < n; begin += kBlock) {
        const std::size_t end = std::min(n, begin + kBlock);
        double part = 0.0;
        for (std::size_t i = begin; i < end; ++i) part += term(i);
        total += part;
    }
    return total;
}

double max_abs(const std::vector<double>& v) {
    double m = 0.0;
    for (double x : v) m = std::max(m, std::abs(x));
    return m;
}

struct Solver {
    psgb_planet* planet;
    std::size_t n;
    double K;
    const std::vector<double>& area;
    const double* floor;
    const double* latent;
    psgb_transport_response response;
    void* user;
    psgb_solve_options inner;
    std::vector<double> diffusion;

    // K lap(t) on the GPU (reference op order, bit-identical to diffusion_source).
    void laplacian(const std::vector<double>& t, std::vector<double>& out) {
        const int code = psgb_diffusion_source(planet, K, t.data(), out.data(), PSGB_MEMORY_HOST, nullptr);
        if (code != PSGB_OK) throw std::runtime_error(psgb_last_error());
    }

    // The response at h, F(h) and the merit sum A F^2.
    double evaluate(const std::vector<double>& h, std::vector<double>& mean, std::vector<double>& slope,
                    std::vector<double>& residual) {
        if (response(user, n, h.data(), mean.data(), slope.data()) != 0)
            throw std::runtime_error("the transport response callback failed");
        laplacian(mean, diffusion);
        for (std::size_t i = 0; i < n; ++i) {
            residual[i] = h[i] - diffusion[i];
            if (latent != nullptr) residual[i] += latent[i];
        }
        return block_sum(n, [&](std::size_t i) { return area[i] * residual[i] * residual[i]; });
    }

    // (A/s + K L) dT = -A F, held cells (s = 0) pinned at zero; returns Krylov iterations.
    int newton_system(const std::vector<double>& slope, const std::vector<double>& residual, std::vector<double>& dt) {
        std::vector<double> rhs(n);
        for (std::size_t i = 0; i < n; ++i) rhs[i] = -residual[i] * area[i];
        std::fill(dt.begin(), dt.end(), 0.0);
        psgb_solve_report rep{};
        const int code = psgb_solve_newton_system(planet, &inner, K, slope.data(), rhs.data(), dt.data(), &rep,
                                                  PSGB_MEMORY_HOST, nullptr);
        // An inexact inner solve is fine (the outer loop converges regardless); only a
        // failure that leaves no usable direction ends the solve.
        if (code != PSGB_OK && code != PSGB_ERR_NOT_CONVERGED) throw std::runtime_error(psgb_last_error());
        return rep.iterations;
    }
};

}  // namespace

extern "C" {

void psgb_transport_settings_default(psgb_transport_settings* out) {
    if (out == nullptr) return;
    out->max_newton_iterations = 30;
    out->max_line_search_halvings = 12;
    out->rounding_floor_W_m2 = 1e-3;
    out->max_non_monotone_steps = 4;
    out->max_non_monotone_growth = 100.0;
    out->newton_tolerance_W_m2 = 1e-6;
    out->cg_relative_tolerance = 1e-6;
    out->max_cg_iterations = 2000;
}

int psgb_solve_implicit_transport(psgb_planet* planet, double conductance_W_K, const double* source_floor_W_m2,
                                  psgb_transport_response response, void* user,
                                  const psgb_transport_settings* settings_in, const psgb_solve_options* options,
                                  const double* latent_W_m2, double* source_out_W_m2, double* mean_out_K,
                                  psgb_transport_result* result) {
    return guarded([&] {
        require(planet != nullptr && source_floor_W_m2 != nullptr && response != nullptr &&
                    source_out_W_m2 != nullptr && mean_out_K != nullptr,
                "null argument");
        require(std::isfinite(conductance_W_K) && conductance_W_K > 0.0,
                "transport conductance must be finite and positive");
        psgb_transport_settings settings;
        psgb_transport_settings_default(&settings);
        if (settings_in != nullptr) settings = *settings_in;
        require(settings.max_newton_iterations >= 0 && settings.max_line_search_halvings >= 0 &&
                    settings.max_non_monotone_steps >= 0 && settings.max_cg_iterations > 0,
                "iteration limits must not be negative");
        require(settings.cg_relative_tolerance > 0.0 && settings.cg_relative_tolerance < 1.0,
                "the inner tolerance must be in (0, 1)");

        psgb_planet_info info{};
        if (psgb_planet_info_get(planet, &info) != PSGB_OK) throw std::runtime_error(psgb_last_error());
        const std::size_t n = info.cells;
        std::vector<double> area(n);
        {   // the transport graph's node areas (an agglomeration's summed fine areas)
            psgb_graph_view view{};
            if (psgb_planet_graph_view(planet, &view) != PSGB_OK) throw std::runtime_error(psgb_last_error());
            std::copy(view.area_m2, view.area_m2 + n, area.begin());
        }
        Solver s{planet, n, conductance_W_K, area, source_floor_W_m2, latent_W_m2, response, user, {}, std::vector<double>(n)};
        psgb_solve_options_default(&s.inner);
        if (options != nullptr) s.inner = *options;
        s.inner.tolerance = settings.cg_relative_tolerance;
        s.inner.max_iterations = settings.max_cg_iterations;

        std::vector<double> source(n), mean(n), slope(n), residual(n), delta_mean(n), delta_source(n), trial(n),
            trial_mean(n), trial_slope(n), trial_residual(n);
        for (std::size_t i = 0; i < n; ++i) source[i] = std::max(0.0, source_floor_W_m2[i]);
        psgb_transport_result out{};
        double merit = s.evaluate(source, mean, slope, residual);
        int non_monotone = 0;
        for (int iteration = 0; iteration < settings.max_newton_iterations; ++iteration) {
            if (max_abs(residual) <= settings.newton_tolerance_W_m2) break;
            // Newton direction: dT from the linear system, dh = -F + K lap(dT).
            out.cg_iterations += s.newton_system(slope, residual, delta_mean);
            s.laplacian(delta_mean, delta_source);
            for (std::size_t i = 0; i < n; ++i) delta_source[i] -= residual[i];
            // Backtracking on the merit; the iterate never drops below the floor.
            double step = 1.0, trial_merit = 0.0;
            for (int halving = 0;; ++halving) {
                for (std::size_t i = 0; i < n; ++i)
                    trial[i] = std::max(source[i] + step * delta_source[i], source_floor_W_m2[i]);
                trial_merit = s.evaluate(trial, trial_mean, trial_slope, trial_residual);
                if (trial_merit < merit) break;
                if (halving == settings.max_line_search_halvings) {
                    // No descent: at the rounding floor stop; farther out (a kink of the
                    // response) take the full step a bounded number of times, unless it
                    // is not finite or raises the merit too much.
                    if (max_abs(residual) <= settings.rounding_floor_W_m2 || non_monotone == settings.max_non_monotone_steps) {
                        step = 0.0;
                    } else {
                        ++non_monotone;
                        step = 1.0;
                        for (std::size_t i = 0; i < n; ++i)
                            trial[i] = std::max(source[i] + delta_source[i], source_floor_W_m2[i]);
                        trial_merit = s.evaluate(trial, trial_mean, trial_slope, trial_residual);
                        if (!(std::isfinite(trial_merit) && trial_merit <= settings.max_non_monotone_growth * merit))
                            step = 0.0;
                    }
                    break;
                }
                step *= 0.5;
            }
            if (step == 0.0) break;
            std::swap(source, trial);
            std::swap(mean, trial_mean);
            std::swap(slope, trial_slope);
            std::swap(residual, trial_residual);
            merit = trial_merit;
            ++out.newton_iterations;
        }
        // The transport applied: the conservative flux form of the last temperatures.
        std::vector<double> applied(n);
        s.laplacian(mean, applied);
        if (latent_W_m2 != nullptr)
            for (std::size_t i = 0; i < n; ++i) applied[i] -= latent_W_m2[i];
        out.consistency_residual_W_m2 = max_abs(residual);
        out.sum_W = block_sum(n, [&](std::size_t i) { return area[i] * applied[i]; });
        out.absolute_sum_W = block_sum(n, [&](std::size_t i) { return std::abs(area[i] * applied[i]); });
        out.dissipation_W_K = block_sum(n, [&](std::size_t i) { return area[i] * applied[i] * mean[i]; });
        std::copy(applied.begin(), applied.end(), source_out_W_m2);
        std::copy(mean.begin(), mean.end(), mean_out_K);
        if (result != nullptr) *result = out;
        return PSGB_OK;
    });
}

}  // extern "C"

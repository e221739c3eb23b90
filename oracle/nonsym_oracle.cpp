// CPU ORACLE - test infrastructure only. Not part of the product and never called by it.
//
// A plain C++ restatement of the reference's non-symmetric transport pieces, compiled into
// the oracle library with planetsim_oracle.cpp:
//   block ILU(0)                   sim/core/math/incomplete_lu.cpp:33-152
//   advection_diffusion_source     sim/planet/surface/heat_transport.cpp:774-815
//   right-preconditioned BiCGSTAB  sim/planet/surface/heat_transport.cpp:823-897
//   solve_implicit_tracer          sim/planet/surface/heat_transport.cpp:901-1081
//   solve_implicit_advection_diffusion  sim/planet/surface/heat_transport.cpp:1083-1318, with the
//                                  column of tests/unit/test_advection_diffusion.cpp:73-104
// Same operations in the same order, sums over the reference's deterministic blocks
// (sequential inside a block, then the blocks in order), -ffp-contract=off: the results
// are the reference's bits. Parity pinning: tests/test_oracle_golden.py checks each entry
// point against the reference's own outputs (tests/golden/nonsym.npz).
#include "oracle_abi.hpp"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <utility>
#include <vector>

namespace {

// ---- block ILU(0) -----------------------------------------------------------------

struct Ilu {
    std::vector<std::size_t> block_start;
    std::vector<std::size_t> start, column, diagonal;
    std::vector<double> value;
    bool zero_pivot = false;

    Ilu(std::size_t rows, const std::uint32_t* offset, const std::uint32_t* neighbour, const double* diag,
        const double* off, const std::uint32_t* blocks, std::size_t block_count, double scale)
        : block_start(blocks, blocks + block_count + 1) {
        std::vector<std::size_t> block_of(rows);
        for (std::size_t b = 0; b + 1 < block_start.size(); ++b)
            for (std::size_t i = block_start[b]; i < block_start[b + 1]; ++i) block_of[i] = b;
        start.assign(rows + 1, 0);
        diagonal.resize(rows);
        std::vector<std::pair<std::size_t, double>> row;
        for (std::size_t i = 0; i < rows; ++i) {
            row.clear();
            row.emplace_back(i, diag[i] * scale);
            for (std::size_t k = offset[i]; k < offset[i + 1]; ++k)
                if (block_of[neighbour[k]] == block_of[i]) row.emplace_back(neighbour[k], off[k]);
            std::sort(row.begin(), row.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
            start[i + 1] = start[i] + row.size();
            for (std::size_t q = 0; q < row.size(); ++q) {
                column.push_back(row[q].first);
                value.push_back(row[q].second);
                if (row[q].first == i) diagonal[i] = start[i] + q;
            }
        }
        for (std::size_t b = 0; b + 1 < block_start.size(); ++b) factor(block_start[b], block_start[b + 1]);
    }

    // IKJ elimination restricted to the pattern, rows [first, last).
    void factor(std::size_t first, std::size_t last) {
        const std::size_t absent = std::numeric_limits<std::size_t>::max();
        std::vector<std::size_t> position(last - first, absent);
        for (std::size_t i = first; i < last; ++i) {
            for (std::size_t q = start[i]; q < start[i + 1]; ++q) position[column[q] - first] = q;
            for (std::size_t q = start[i]; q < diagonal[i]; ++q) {
                const std::size_t j = column[q];
                const double pivot = value[diagonal[j]];
                if (pivot == 0.0) zero_pivot = true;
                value[q] /= pivot;
                for (std::size_t t = diagonal[j] + 1; t < start[j + 1]; ++t) {
                    const std::size_t at = position[column[t] - first];
                    if (at != absent) value[at] -= value[q] * value[t];
                }
            }
            for (std::size_t q = start[i]; q < start[i + 1]; ++q) position[column[q] - first] = absent;
        }
    }

    void solve(std::vector<double>& x) const {
        for (std::size_t b = 0; b + 1 < block_start.size(); ++b) {
            const std::size_t first = block_start[b], last = block_start[b + 1];
            for (std::size_t i = first; i < last; ++i) {
                double sum = x[i];
                for (std::size_t q = start[i]; q < diagonal[i]; ++q) sum -= value[q] * x[column[q]];
                x[i] = sum;
            }
            for (std::size_t i = last; i-- > first;) {
                double sum = x[i];
                for (std::size_t q = diagonal[i] + 1; q < start[i + 1]; ++q) sum -= value[q] * x[column[q]];
                x[i] = sum / value[diagonal[i]];
            }
        }
    }
};

// Dot product over fixed blocks of `block` rows: sequential inside a block, blocks in order.
double block_dot(const std::vector<double>& u, const std::vector<double>& v, std::size_t block) {
    double total = 0.0;
    for (std::size_t b = 0; b < u.size(); b += block) {
        double part = 0.0;
        const std::size_t e = std::min(u.size(), b + block);
        for (std::size_t i = b; i < e; ++i) part += u[i] * v[i];
        total = total + part;
    }
    return total;
}

// BiCGSTAB from x = 0 with right preconditioning (heat_transport.cpp:823-897).
template <typename Apply, typename Precondition>
int bicgstab(std::size_t n, std::size_t block, const Apply& apply, const Precondition& precondition,
             const std::vector<double>& b, std::vector<double>& x, double tolerance, int max_iterations) {
    const auto dot = [&](const std::vector<double>& u, const std::vector<double>& v) { return block_dot(u, v, block); };
    x.assign(n, 0.0);
    std::vector<double> r = b;
    const std::vector<double> shadow = r;
    std::vector<double> p(n, 0.0), v(n, 0.0), p_hat(n, 0.0), s(n, 0.0), s_hat(n, 0.0), t(n, 0.0);
    const double b_norm = std::sqrt(dot(b, b));
    if (!(b_norm > 0.0)) return 0;
    double rho = 1.0, alpha = 1.0, omega = 1.0;
    int iteration = 0;
    while (iteration < max_iterations) {
        const double rho_next = dot(shadow, r);
        if (rho_next == 0.0 || omega == 0.0) break;
        const double beta = rho_next / rho * (alpha / omega);
        rho = rho_next;
        for (std::size_t i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
        precondition(p, p_hat);
        apply(p_hat, v);
        const double shadow_v = dot(shadow, v);
        if (shadow_v == 0.0) break;
        alpha = rho / shadow_v;
        for (std::size_t i = 0; i < n; ++i) s[i] = r[i] - alpha * v[i];
        ++iteration;
        if (std::sqrt(dot(s, s)) <= tolerance * b_norm) {
            for (std::size_t i = 0; i < n; ++i) x[i] += alpha * p_hat[i];
            break;
        }
        precondition(s, s_hat);
        apply(s_hat, t);
        const double t_t = dot(t, t);
        omega = t_t > 0.0 ? dot(t, s) / t_t : 0.0;
        for (std::size_t i = 0; i < n; ++i) {
            x[i] += alpha * p_hat[i] + omega * s_hat[i];
            r[i] = s[i] - omega * t[i];
        }
        if (std::sqrt(dot(r, r)) <= tolerance * b_norm) break;
    }
    return iteration;
}

}  // namespace

extern "C" {

void* orc_ilu_new(std::uint64_t rows, const std::uint32_t* offset, const std::uint32_t* neighbour,
                  const double* diag, const double* off, const std::uint32_t* block_start, std::uint64_t blocks,
                  double scale) {
    return new Ilu(rows, offset, neighbour, diag, off, block_start, blocks, scale);
}
int orc_ilu_zero_pivot(void* h) { return static_cast<Ilu*>(h)->zero_pivot ? 1 : 0; }
void orc_ilu_solve(void* h, std::uint64_t rows, double* x) {
    std::vector<double> v(x, x + rows);
    static_cast<Ilu*>(h)->solve(v);
    std::copy(v.begin(), v.end(), x);
}
void orc_ilu_free(void* h) { delete static_cast<Ilu*>(h); }

// advection_diffusion_source: per node H_eddy and H_advective.
void orc_advection_source(std::uint64_t nodes, const std::uint32_t* offset, const std::uint32_t* neighbour,
                          const double* area, std::uint64_t layers, const double* conductance,
                          const double* outflow, const double* latent, const double* mean, const double* energy,
                          double* eddy_out, double* advective_out) {
    const std::size_t entries = offset[nodes];
    for (std::size_t a = 0; a < nodes; ++a) {
        double eddy = 0.0, advective = 0.0;
        for (std::size_t k = offset[a]; k < offset[a + 1]; ++k) {
            const std::size_t b = neighbour[k];
            eddy += conductance[k] * (mean[b] - mean[a]);
            for (std::size_t l = 0; l < layers; ++l) {
                const double out = outflow[l * entries + k];
                const std::size_t upwind = out > 0.0 ? a : b;
                advective -= out * energy[l * nodes + upwind];
            }
        }
        eddy_out[a] = eddy / area[a];
        if (latent != nullptr) eddy_out[a] -= latent[a];
        advective_out[a] = advective / area[a];
    }
}

// solve_implicit_tracer; stats: iterations, relative residual, clipped kg, column divergence.
void orc_solve_implicit_tracer(std::uint64_t nodes, const std::uint32_t* offset, const std::uint32_t* neighbour,
                               std::uint64_t layers, const double* conductance, const double* outflow,
                               double heat_capacity, const double* layer_mass, const double* tracer, double dt,
                               double tolerance, int max_iterations, double* tracer_out, double* stats) {
    const std::size_t entries = offset[nodes], L = layers, rows = nodes * L;
    const double exchange_scale = 1.0 / (heat_capacity * static_cast<double>(L));
    std::vector<double> vertical(rows, 0.0);
    double column_divergence = 0.0;
    for (std::size_t a = 0; a < nodes; ++a) {
        double w = 0.0;
        for (std::size_t l = 0; l < L; ++l) {
            for (std::size_t k = offset[a]; k < offset[a + 1]; ++k) w -= outflow[l * entries + k];
            vertical[a * L + l] = l + 1 < L ? w : 0.0;
        }
        column_divergence = std::max(column_divergence, std::abs(w));
    }
    // the stacked system: row a L + l, the graph row's entries in this layer, below, above
    std::vector<std::uint32_t> s_offset(rows + 1, 0), s_neighbour;
    for (std::size_t a = 0; a < nodes; ++a) {
        for (std::size_t l = 0; l < L; ++l) {
            const std::size_t row = a * L + l;
            for (std::size_t k = offset[a]; k < offset[a + 1]; ++k)
                s_neighbour.push_back(static_cast<std::uint32_t>(neighbour[k] * L + l));
            if (l > 0) s_neighbour.push_back(static_cast<std::uint32_t>(row - 1));
            if (l + 1 < L) s_neighbour.push_back(static_cast<std::uint32_t>(row + 1));
            s_offset[row + 1] = static_cast<std::uint32_t>(s_neighbour.size());
        }
    }
    std::vector<double> diagonal(rows, 0.0), off(s_neighbour.size(), 0.0), rhs(rows, 0.0);
    for (std::size_t a = 0; a < nodes; ++a) {
        const double rate = layer_mass[a] / dt;
        for (std::size_t l = 0; l < L; ++l) {
            const std::size_t row = a * L + l;
            double own = rate;
            std::size_t at = s_offset[row];
            for (std::size_t k = offset[a]; k < offset[a + 1]; ++k, ++at) {
                const double flow = outflow[l * entries + k];
                const double eddy = conductance[k] * exchange_scale;
                own += std::max(flow, 0.0) + eddy;
                off[at] = -std::max(-flow, 0.0) - eddy;
            }
            const double below = l > 0 ? vertical[a * L + l - 1] : 0.0;
            const double above = vertical[row];
            if (l > 0) {
                own += std::max(-below, 0.0);
                off[at++] = -std::max(below, 0.0);
            }
            if (l + 1 < L) {
                own += std::max(above, 0.0);
                off[at++] = -std::max(-above, 0.0);
            }
            diagonal[row] = own;
            rhs[row] = rate * tracer[l * nodes + a];
        }
    }
    std::vector<std::uint32_t> blocks{0};
    for (std::size_t b = 0; b < nodes; b += 256) blocks.push_back(static_cast<std::uint32_t>(std::min(nodes, b + 256) * L));
    const Ilu factor(rows, s_offset.data(), s_neighbour.data(), diagonal.data(), off.data(), blocks.data(),
                     blocks.size() - 1, 1.0);
    const auto apply = [&](const std::vector<double>& x, std::vector<double>& y) {
        for (std::size_t row = 0; row < rows; ++row) {
            double sum = diagonal[row] * x[row];
            for (std::size_t k = s_offset[row]; k < s_offset[row + 1]; ++k) sum += off[k] * x[s_neighbour[k]];
            y[row] = sum;
        }
    };
    const auto precondition = [&](const std::vector<double>& x, std::vector<double>& y) {
        y = x;
        factor.solve(y);
    };
    std::vector<double> start(rows, 0.0);
    for (std::size_t a = 0; a < nodes; ++a)
        for (std::size_t l = 0; l < L; ++l) start[a * L + l] = tracer[l * nodes + a];
    std::vector<double> applied(rows, 0.0), residual(rows, 0.0), delta;
    apply(start, applied);
    for (std::size_t row = 0; row < rows; ++row) residual[row] = rhs[row] - applied[row];
    const int iterations = bicgstab(rows, 256 * L, apply, precondition, residual, delta, tolerance, max_iterations);
    std::vector<double> solved(rows, 0.0);
    for (std::size_t row = 0; row < rows; ++row) solved[row] = std::max(0.0, start[row] + (delta.empty() ? 0.0 : delta[row]));
    apply(solved, applied);
    double residual_norm = 0.0, rhs_norm = 0.0;
    for (std::size_t row = 0; row < rows; ++row) {
        residual_norm += (rhs[row] - applied[row]) * (rhs[row] - applied[row]);
        rhs_norm += rhs[row] * rhs[row];
    }
    // the flux form of the solution, each face once from its lower node
    std::vector<double> change(rows, 0.0);
    for (std::size_t a = 0; a < nodes; ++a) {
        for (std::size_t l = 0; l < L; ++l) {
            const std::size_t row = a * L + l;
            for (std::size_t k = offset[a]; k < offset[a + 1]; ++k) {
                const std::size_t b = neighbour[k];
                if (b < a) continue;
                const std::size_t other = b * L + l;
                const double flow = outflow[l * entries + k];
                const double eddy = conductance[k] * exchange_scale;
                const double flux = (flow > 0.0 ? flow * solved[row] : flow * solved[other]) +
                                    eddy * (solved[row] - solved[other]);
                change[row] -= flux;
                change[other] += flux;
            }
            if (l + 1 < L) {
                const double w = vertical[row];
                const double flux = w > 0.0 ? w * solved[row] : w * solved[row + 1];
                change[row] -= flux;
                change[row + 1] += flux;
            }
        }
    }
    double clipped = 0.0;
    for (std::size_t a = 0; a < nodes; ++a) {
        for (std::size_t l = 0; l < L; ++l) {
            const std::size_t row = a * L + l;
            double value = tracer[l * nodes + a] + dt * change[row] / layer_mass[a];
            if (value < 0.0) {
                clipped -= value * layer_mass[a];
                value = 0.0;
            }
            tracer_out[l * nodes + a] = value;
        }
    }
    stats[0] = iterations;
    stats[1] = rhs_norm > 0.0 ? std::sqrt(residual_norm / rhs_norm) : 0.0;
    stats[2] = clipped;
    stats[3] = column_divergence;
}


// solve_implicit_advection_diffusion with the reference test's column: a x + r x^4 = b + h
// (solve_column_surface's dry Newton, column_step.cpp:254-276), s_l = c_p x (1 + eps_l) +
// phi_l. stats: newton, linear iterations, consistency, sum, absolute, eddy absolute,
// advective absolute.
void orc_solve_implicit_advection_diffusion(const orc_graph* gp, std::uint64_t layers, const double* conductance,
                                            const double* outflow, const double* latent, double heat_capacity,
                                            double a, const double* b, const double* epsilon,
                                            const double* geopotential, const double* floor, double cg_tolerance,
                                            double newton_tolerance, double* source_out, double* mean_out,
                                            double* energy_out, double* stats) {
    const std::size_t n = gp->n, entries = gp->offset[n], L = layers;
    const std::uint32_t* offset = gp->offset;
    const std::uint32_t* neighbour = gp->neighbour;
    const double* area = gp->area;
    const double radiative = 0.75 * 0.97 * 5.670374419e-8;
    struct Iterate {
        std::vector<double> source, mean, slope, energy, energy_slope, residual;
        double merit = 0.0;
    };
    const auto respond = [&](Iterate& at) {
        at.mean.assign(n, 0.0);
        at.slope.assign(n, 0.0);
        at.energy.assign(L * n, 0.0);
        at.energy_slope.assign(L * n, 0.0);
        for (std::size_t i = 0; i < n; ++i) {
            const double rhs = b[i] + at.source[i];
            double x = std::min(rhs / a, std::sqrt(std::sqrt(rhs / radiative)));
            for (int it = 0; it < 10; ++it) {
                const double x3 = x * x * x;
                const double value = a * x + radiative * x3 * x - rhs;
                const double slope = a + 4.0 * radiative * x3;
                const double step = value / slope;
                x -= step;
                if (std::abs(step) <= 4.0 * std::numeric_limits<double>::epsilon() * x) break;
            }
            at.mean[i] = x;
            at.slope[i] = 1.0 / (a + 4.0 * radiative * x * x * x + 0.0);
            for (std::size_t l = 0; l < L; ++l) {
                at.energy[l * n + i] = heat_capacity * x * (1.0 + epsilon[l]) + geopotential[l];
                at.energy_slope[l * n + i] = heat_capacity * at.slope[i] * (1.0 + epsilon[l]);
            }
        }
    };
    std::vector<double> eddy(n, 0.0), advective(n, 0.0);
    const auto source_of = [&](const Iterate& at) {
        orc_advection_source(n, offset, neighbour, area, L, conductance, outflow, latent, at.mean.data(),
                             at.energy.data(), eddy.data(), advective.data());
    };
    const auto evaluate = [&](Iterate& at) {
        respond(at);
        source_of(at);
        at.residual.assign(n, 0.0);
        double merit = 0.0;
        for (std::size_t begin = 0; begin < n; begin += 256) {
            double part = 0.0;
            for (std::size_t i = begin; i < std::min(n, begin + 256); ++i) {
                at.residual[i] = at.source[i] - (eddy[i] + advective[i]);
                part += area[i] * at.residual[i] * at.residual[i];
            }
            merit = merit + part;
        }
        at.merit = merit;
    };
    const auto max_abs = [&](const std::vector<double>& v) {
        double largest = 0.0;
        for (const double x : v) largest = std::max(largest, std::abs(x));
        return largest;
    };
    Iterate current, trial;
    current.source.assign(n, 0.0);
    for (std::size_t i = 0; i < n; ++i) current.source[i] = std::max(0.0, floor[i]);
    evaluate(current);
    std::vector<std::uint32_t> blocks{0};
    for (std::size_t begin = 0; begin < n; begin += 256) blocks.push_back(static_cast<std::uint32_t>(std::min(n, begin + 256)));
    std::vector<double> diagonal(n, 0.0), off(entries, 0.0), sym_diag(n, 0.0), sym_off(entries, 0.0), rhs(n, 0.0),
        delta(n, 0.0), scaled(n, 0.0), leftover(n, 0.0);
    void* multigrid = orc_hierarchy_new(gp);
    int newton = 0, linear = 0, non_monotone = 0;
    const int max_newton = 30, max_halvings = 12, max_non_monotone = 4, max_cg = 2000;
    const double rounding_floor = 1e-3, max_growth = 100.0;
    for (int iteration = 0; iteration < max_newton; ++iteration) {
        if (max_abs(current.residual) <= newton_tolerance) break;
        for (std::size_t i = 0; i < n; ++i) {
            const double inverse_area = 1.0 / area[i];
            double own = 0.0;
            for (std::size_t k = offset[i]; k < offset[i + 1]; ++k) {
                const std::size_t j = neighbour[k];
                const double g = conductance[k];
                own -= g * current.slope[i];
                double nb = g * current.slope[j];
                for (std::size_t l = 0; l < L; ++l) {
                    const double out = outflow[l * entries + k];
                    if (out > 0.0) {
                        own -= out * current.energy_slope[l * n + i];
                    } else {
                        nb -= out * current.energy_slope[l * n + j];
                    }
                }
                off[k] = -nb * inverse_area;
            }
            diagonal[i] = 1.0 - own * inverse_area;
            rhs[i] = -current.residual[i];
        }
        const Ilu factor(n, offset, neighbour, diagonal.data(), off.data(), blocks.data(), blocks.size() - 1, 1.0);
        const auto apply = [&](const std::vector<double>& x, std::vector<double>& y) {
            for (std::size_t i = 0; i < n; ++i) {
                double sum = diagonal[i] * x[i];
                for (std::size_t k = offset[i]; k < offset[i + 1]; ++k) sum += off[k] * x[neighbour[k]];
                y[i] = sum;
            }
        };
        for (std::size_t i = 0; i < n; ++i) {
            double sum = 0.0;
            for (std::size_t k = offset[i]; k < offset[i + 1]; ++k) {
                sum += conductance[k];
                sym_off[k] = -conductance[k];
            }
            sym_diag[i] = area[i] / std::max(current.slope[i], 1.0e-12) + sum;
        }
        orc_hierarchy_set_matrix(multigrid, sym_diag.data(), sym_off.data());
        const auto precondition = [&](const std::vector<double>& x, std::vector<double>& y) {
            for (std::size_t i = 0; i < n; ++i) scaled[i] = area[i] * x[i];
            y.assign(n, 0.0);
            orc_vcycle_sgs(multigrid, scaled.data(), y.data());
            for (std::size_t i = 0; i < n; ++i) y[i] /= std::max(current.slope[i], 1.0e-12);
            apply(y, leftover);
            for (std::size_t i = 0; i < n; ++i) leftover[i] = x[i] - leftover[i];
            factor.solve(leftover);
            for (std::size_t i = 0; i < n; ++i) y[i] += leftover[i];
        };
        linear += bicgstab(n, 256, apply, precondition, rhs, delta, cg_tolerance, max_cg);
        double step = 1.0;
        bool accepted = false;
        for (int halving = 0;; ++halving) {
            trial.source.assign(n, 0.0);
            for (std::size_t i = 0; i < n; ++i) trial.source[i] = std::max(current.source[i] + step * delta[i], floor[i]);
            evaluate(trial);
            if (trial.merit < current.merit) {
                accepted = true;
                break;
            }
            if (halving == max_halvings) {
                if (max_abs(current.residual) > rounding_floor && non_monotone < max_non_monotone) {
                    ++non_monotone;
                    for (std::size_t i = 0; i < n; ++i) trial.source[i] = std::max(current.source[i] + delta[i], floor[i]);
                    evaluate(trial);
                    accepted = std::isfinite(trial.merit) && trial.merit <= max_growth * current.merit;
                }
                break;
            }
            step *= 0.5;
        }
        if (!accepted) break;
        std::swap(current, trial);
        ++newton;
    }
    orc_hierarchy_free(multigrid);
    source_of(current);
    double sum = 0.0, absolute = 0.0, eddy_absolute = 0.0, advective_absolute = 0.0;
    for (std::size_t i = 0; i < n; ++i) {
        source_out[i] = eddy[i] + advective[i];
        sum += area[i] * source_out[i];
        absolute += area[i] * std::abs(source_out[i]);
        eddy_absolute += area[i] * std::abs(eddy[i]);
        advective_absolute += area[i] * std::abs(advective[i]);
    }
    std::copy(current.mean.begin(), current.mean.end(), mean_out);
    std::copy(current.energy.begin(), current.energy.end(), energy_out);
    stats[0] = newton;
    stats[1] = linear;
    stats[2] = max_abs(current.residual);
    stats[3] = sum;
    stats[4] = absolute;
    stats[5] = eddy_absolute;
    stats[6] = advective_absolute;
}

}  // extern "C"

// CPU ORACLE - test infrastructure only. Not part of the product and never called by it.
//
// A plain C++ restatement of the reference's non-symmetric transport pieces, compiled into
// the oracle library with planetsim_oracle.cpp:
//   block ILU(0)                   sim/core/math/incomplete_lu.cpp:33-152
//   advection_diffusion_source     sim/planet/surface/heat_transport.cpp:774-815
//   right-preconditioned BiCGSTAB  sim/planet/surface/heat_transport.cpp:823-897
//   solve_implicit_tracer          sim/planet/surface/heat_transport.cpp:901-1081
// Same operations in the same order, sums over the reference's deterministic blocks
// (sequential inside a block, then the blocks in order), -ffp-contract=off: the results
// are the reference's bits. Parity pinning: tests/test_oracle_golden.py checks each entry
// point against the reference's own outputs (tests/golden/nonsym.npz).
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

}  // extern "C"

// CPU ORACLE - test infrastructure only. Not part of the product and never called by it.
//
// A plain C++ restatement of the reference PlanetSim algorithms on the heat-transport
// path, used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
// checker and the timed CPU baseline. It takes the mesh and transport graph as flat
// arrays (the GB300 library's host mesh builder produces them; that builder is itself
// pinned bit-for-bit against the reference's make_icosphere by the golden fixtures).
//
// Parity pinning: tests/test_oracle_golden.py checks every entry point below against
// golden vectors produced by the reference's own code (tests/golden/make_golden.py,
// built from the reference sources by oracle/Makefile.ref). The FP64 PCG, V-cycle,
// Galerkin values, hierarchy structure and operators match the reference bit for bit
// (same operation order, deterministic 256-cell block reductions, -ffp-contract=off);
// the column radiation matches to the last few ulps of libm.
//
// Reference files (paths inside fgianni/planet_game):
//   finite-volume operators      sim/planet/operators/finite_volume.cpp:34-111
//   diffusion source             sim/planet/surface/heat_transport.cpp:28-36, 579-593
//   aggregation hierarchy        sim/planet/surface/heat_transport.cpp:73-200
//   dense coarse solve           sim/planet/surface/heat_transport.cpp:202-243
//   SGS V-cycle                  sim/planet/surface/heat_transport.cpp:258-326
//   PCG (solve_newton_system)    sim/planet/surface/heat_transport.cpp:337-429
//   Newton driver                sim/planet/surface/heat_transport.cpp:595-772
//   BiCGSTAB                     sim/planet/surface/heat_transport.cpp:823-897
//   column radiation             sim/planet/atmosphere/atmosphere_column.hpp:39-143, 589-634
//   saturation                   sim/planet/atmosphere/saturation.cpp:9-54
#include "oracle_abi.hpp"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <vector>

namespace {

constexpr std::size_t kBlock = 256;   // the reference's deterministic cell blocks

struct Graph {
    std::size_t n;
    const std::uint32_t* offset;      // n + 1
    const std::uint32_t* neighbour;
    const double* weight;             // l / d
    const double* weight_sum;
    const double* area;
};

// Block-ordered sum: sequential inside each 256-cell block, then over blocks in order
// (reduce_deterministic_blocks, sim/core/scheduler/deterministic_executor.hpp:42-57).
template <typename F>
double block_sum(std::size_t n, F&& term) {
    double total = 0.0;
    for (std::size_t b = 0; b < n; b += kBlock) {
        double part = 0.0;
        const std::size_t e = std::min(n, b + kBlock);
        for (std::size_t i = b; i < e; ++i) part += term(i);
        total = total + part;
    }
    return total;
}

double dot(const std::vector<double>& a, const std::vector<double>& b) {
    return block_sum(a.size(), [&](std::size_t i) { return a[i] * b[i]; });
}

// ---- hierarchy ----------------------------------------------------------------------

constexpr std::size_t kNone = std::numeric_limits<std::size_t>::max();

struct Level {
    std::size_t size = 0;
    std::vector<double> diag;
    std::vector<std::size_t> off;     // CSR row starts (size + 1)
    std::vector<std::size_t> col;
    std::vector<double> val;
    std::vector<std::size_t> agg;     // empty on the coarsest level
    std::vector<std::size_t> tgt;     // kNone: lands on the aggregate's diagonal
    std::vector<double> chol;         // coarsest only
};

struct Hierarchy {
    std::vector<Level> levels;
    // per-level scratch of the SGS V-cycle (one solve at a time per hierarchy)
    mutable std::vector<std::vector<double>> prev, rhs, sol;
    // exported copies for the C ABI
    std::vector<std::vector<std::uint32_t>> x_off, x_col, x_agg;
    std::vector<std::vector<std::int64_t>> x_tgt;
};

std::vector<std::size_t> aggregates(const Level& L, std::size_t& count) {
    std::vector<std::size_t> a(L.size, kNone);
    count = 0;
    for (std::size_t r = 0; r < L.size; ++r) {
        if (a[r] != kNone) continue;
        bool all_free = true;
        for (std::size_t k = L.off[r]; k < L.off[r + 1] && all_free; ++k) all_free = a[L.col[k]] == kNone;
        if (!all_free) continue;
        a[r] = count;
        for (std::size_t k = L.off[r]; k < L.off[r + 1]; ++k) a[L.col[k]] = count;
        ++count;
    }
    for (std::size_t r = 0; r < L.size; ++r) {
        if (a[r] != kNone) continue;
        double best = 0.0;
        for (std::size_t k = L.off[r]; k < L.off[r + 1]; ++k) {
            if (a[L.col[k]] != kNone && -L.val[k] > best) {
                best = -L.val[k];
                a[r] = a[L.col[k]];
            }
        }
        if (a[r] == kNone) a[r] = count++;
    }
    return a;
}

Level coarse_pattern(Level& F) {
    std::size_t count = 0;
    F.agg = aggregates(F, count);
    Level Cc;
    Cc.size = count;
    std::vector<std::vector<std::size_t>> cols(count);
    for (std::size_t r = 0; r < F.size; ++r)
        for (std::size_t k = F.off[r]; k < F.off[r + 1]; ++k)
            if (F.agg[F.col[k]] != F.agg[r]) cols[F.agg[r]].push_back(F.agg[F.col[k]]);
    Cc.off.assign(count + 1, 0);
    for (std::size_t a = 0; a < count; ++a) {
        std::sort(cols[a].begin(), cols[a].end());
        cols[a].erase(std::unique(cols[a].begin(), cols[a].end()), cols[a].end());
        Cc.col.insert(Cc.col.end(), cols[a].begin(), cols[a].end());
        Cc.off[a + 1] = Cc.col.size();
    }
    Cc.diag.assign(count, 0.0);
    Cc.val.assign(Cc.col.size(), 0.0);
    F.tgt.assign(F.col.size(), kNone);
    for (std::size_t r = 0; r < F.size; ++r) {
        const std::size_t a = F.agg[r];
        for (std::size_t k = F.off[r]; k < F.off[r + 1]; ++k) {
            const std::size_t b = F.agg[F.col[k]];
            if (b == a) continue;
            const auto first = Cc.col.begin() + static_cast<std::ptrdiff_t>(Cc.off[a]);
            const auto last = Cc.col.begin() + static_cast<std::ptrdiff_t>(Cc.off[a + 1]);
            F.tgt[k] = static_cast<std::size_t>(std::lower_bound(first, last, b) - Cc.col.begin());
        }
    }
    return Cc;
}

void galerkin(const Level& F, Level& Cc) {
    std::fill(Cc.diag.begin(), Cc.diag.end(), 0.0);
    std::fill(Cc.val.begin(), Cc.val.end(), 0.0);
    for (std::size_t r = 0; r < F.size; ++r) {
        const std::size_t a = F.agg[r];
        Cc.diag[a] += F.diag[r];
        for (std::size_t k = F.off[r]; k < F.off[r + 1]; ++k) {
            if (F.tgt[k] == kNone) Cc.diag[a] += F.val[k];
            else Cc.val[F.tgt[k]] += F.val[k];
        }
    }
}

void cholesky(Level& L) {
    const std::size_t n = L.size;
    L.chol.assign(n * n, 0.0);
    for (std::size_t r = 0; r < n; ++r) {
        L.chol[r * n + r] = L.diag[r];
        for (std::size_t k = L.off[r]; k < L.off[r + 1]; ++k) L.chol[r * n + L.col[k]] = L.val[k];
    }
    for (std::size_t j = 0; j < n; ++j) {
        double p = L.chol[j * n + j];
        for (std::size_t k = 0; k < j; ++k) p -= L.chol[j * n + k] * L.chol[j * n + k];
        p = std::sqrt(p);
        L.chol[j * n + j] = p;
        for (std::size_t i = j + 1; i < n; ++i) {
            double s = L.chol[i * n + j];
            for (std::size_t k = 0; k < j; ++k) s -= L.chol[i * n + k] * L.chol[j * n + k];
            L.chol[i * n + j] = s / p;
        }
    }
}

void chol_solve(const Level& L, const std::vector<double>& b, std::vector<double>& x) {
    const std::size_t n = L.size;
    x = b;
    for (std::size_t i = 0; i < n; ++i) {
        for (std::size_t k = 0; k < i; ++k) x[i] -= L.chol[i * n + k] * x[k];
        x[i] /= L.chol[i * n + i];
    }
    for (std::size_t i = n; i-- > 0;) {
        for (std::size_t k = i + 1; k < n; ++k) x[i] -= L.chol[k * n + i] * x[k];
        x[i] /= L.chol[i * n + i];
    }
}

Hierarchy build(const Graph& g) {
    Hierarchy h;
    h.levels.resize(1);
    Level& F = h.levels[0];
    F.size = g.n;
    F.diag.assign(g.weight_sum, g.weight_sum + g.n);
    F.off.assign(g.offset, g.offset + g.n + 1);
    F.col.assign(g.neighbour, g.neighbour + g.offset[g.n]);
    F.val.resize(g.offset[g.n]);
    for (std::size_t k = 0; k < F.val.size(); ++k) F.val[k] = -g.weight[k];
    while (h.levels.back().size > 400) {
        Level Cc = coarse_pattern(h.levels.back());
        galerkin(h.levels.back(), Cc);
        if (Cc.size >= h.levels.back().size) {
            h.levels.back().agg.clear();
            h.levels.back().tgt.clear();
            break;
        }
        h.levels.push_back(std::move(Cc));
    }
    for (const Level& L : h.levels) {
        h.x_off.emplace_back(L.off.begin(), L.off.end());
        h.x_col.emplace_back(L.col.begin(), L.col.end());
        h.x_agg.emplace_back(L.agg.begin(), L.agg.end());
        std::vector<std::int64_t> t(L.tgt.size());
        for (std::size_t k = 0; k < t.size(); ++k) t[k] = L.tgt[k] == kNone ? -1 : static_cast<std::int64_t>(L.tgt[k]);
        h.x_tgt.push_back(std::move(t));
    }
    return h;
}

void set_values(Hierarchy& h) {
    for (std::size_t l = 0; l + 1 < h.levels.size(); ++l) galerkin(h.levels[l], h.levels[l + 1]);
    cholesky(h.levels.back());
}

// Symmetric block-hybrid Gauss-Seidel half sweep (heat_transport.cpp:258-286).
void gauss_seidel(const Level& L, const std::vector<double>& b, std::vector<double>& x, bool forward, bool blocked,
                  std::vector<double>& prev) {
    if (!blocked) {
        for (std::size_t s = 0; s < L.size; ++s) {
            const std::size_t r = forward ? s : L.size - 1 - s;
            double sum = b[r];
            for (std::size_t k = L.off[r]; k < L.off[r + 1]; ++k) sum -= L.val[k] * x[L.col[k]];
            x[r] = sum / L.diag[r];
        }
        return;
    }
    prev.assign(x.begin(), x.end());
    for (std::size_t b0 = 0; b0 < L.size; b0 += kBlock) {
        const std::size_t b1 = std::min(L.size, b0 + kBlock);
        for (std::size_t s = 0; s < b1 - b0; ++s) {
            const std::size_t r = forward ? b0 + s : b1 - 1 - s;
            double sum = b[r];
            for (std::size_t k = L.off[r]; k < L.off[r + 1]; ++k) {
                const std::size_t c = L.col[k];
                sum -= L.val[k] * ((c >= b0 && c < b1) ? x[c] : prev[c]);
            }
            x[r] = sum / L.diag[r];
        }
    }
}

void vcycle_sgs(const Hierarchy& h, std::size_t l, const std::vector<double>& b, std::vector<double>& x) {
    const Level& L = h.levels[l];
    if (l + 1 == h.levels.size()) {
        chol_solve(L, b, x);
        return;
    }
    if (h.prev.size() != h.levels.size()) {
        h.prev.resize(h.levels.size());
        h.rhs.resize(h.levels.size());
        h.sol.resize(h.levels.size());
    }
    x.assign(L.size, 0.0);
    gauss_seidel(L, b, x, true, l == 0, h.prev[l]);
    // residual and restriction: the coarse sums take the residuals in ascending row order
    std::vector<double>& bc = h.rhs[l + 1];
    bc.assign(h.levels[l + 1].size, 0.0);
    for (std::size_t i = 0; i < L.size; ++i) {
        double v = b[i] - L.diag[i] * x[i];
        for (std::size_t k = L.off[i]; k < L.off[i + 1]; ++k) v -= L.val[k] * x[L.col[k]];
        bc[L.agg[i]] += v;
    }
    std::vector<double>& xc = h.sol[l + 1];
    vcycle_sgs(h, l + 1, bc, xc);
    for (std::size_t i = 0; i < L.size; ++i) x[i] += xc[L.agg[i]];
    gauss_seidel(L, b, x, false, l == 0, h.prev[l]);
}

// The GB300 V-cycle's algorithm: damped Jacobi (pre sweeps from zero, post sweeps),
// residual, restriction in ascending fine-row order, prolongation scaled by `correction`
// (the product rounded, then added), dense coarsest solve.
void vcycle_jacobi(const Hierarchy& h, std::size_t l, int pre, int post, double omega, double correction,
                   const std::vector<double>& b, std::vector<double>& x) {
    const Level& L = h.levels[l];
    if (l + 1 == h.levels.size()) {
        chol_solve(L, b, x);
        return;
    }
    auto sweep = [&](std::vector<double>& v) {
        std::vector<double> y(L.size);
        for (std::size_t i = 0; i < L.size; ++i) {
            double s = b[i];
            for (std::size_t k = L.off[i]; k < L.off[i + 1]; ++k) s -= L.val[k] * v[L.col[k]];
            y[i] = v[i] + omega * (s / L.diag[i] - v[i]);
        }
        v.swap(y);
    };
    x.assign(L.size, 0.0);
    for (std::size_t i = 0; i < L.size; ++i) x[i] = omega * b[i] / L.diag[i];
    for (int k = 1; k < pre; ++k) sweep(x);
    std::vector<double> bc(h.levels[l + 1].size, 0.0);
    for (std::size_t i = 0; i < L.size; ++i) {
        double v = b[i] - L.diag[i] * x[i];
        for (std::size_t k = L.off[i]; k < L.off[i + 1]; ++k) v -= L.val[k] * x[L.col[k]];
        bc[L.agg[i]] += v;
    }
    std::vector<double> xc;
    vcycle_jacobi(h, l + 1, pre, post, omega, correction, bc, xc);
    for (std::size_t i = 0; i < L.size; ++i) {
        const double e = correction * xc[L.agg[i]];
        x[i] += e;
    }
    for (int k = 0; k < post; ++k) sweep(x);
}

// Fine matrix of the implicit step (heat_transport.cpp:351-363); `edge_g` (optional,
// per CSR entry) replaces the scalar conductance.
void assemble(Hierarchy& h, const Graph& g, double K, const double* edge_g, const std::vector<double>& slope) {
    Level& F = h.levels[0];
    for (std::size_t c = 0; c < g.n; ++c) {
        const bool free_row = slope[c] > 0.0;
        double coupling = 0.0;
        if (edge_g != nullptr) {
            for (std::size_t k = g.offset[c]; k < g.offset[c + 1]; ++k) coupling += edge_g[k] * g.weight[k];
        } else {
            coupling = K * g.weight_sum[c];
        }
        F.diag[c] = free_row ? g.area[c] / slope[c] + coupling : 1.0;
        for (std::size_t k = g.offset[c]; k < g.offset[c + 1]; ++k) {
            const double kk = edge_g != nullptr ? edge_g[k] : K;
            F.val[k] = free_row && slope[g.neighbour[k]] > 0.0 ? -kk * g.weight[k] : 0.0;
        }
    }
    set_values(h);
}

void apply(const Level& F, const std::vector<double>& x, std::vector<double>& y) {
    for (std::size_t i = 0; i < F.size; ++i) {
        double s = F.diag[i] * x[i];
        for (std::size_t k = F.off[i]; k < F.off[i + 1]; ++k) s += F.val[k] * x[F.col[k]];
        y[i] = s;
    }
}

// PCG of solve_newton_system (heat_transport.cpp:394-429) on the assembled matrix.
int pcg(const Hierarchy& h, const std::vector<double>& slope, const std::vector<double>& rhs, double tol, int max_it,
        std::vector<double>& x) {
    const Level& F = h.levels[0];
    const std::size_t n = F.size;
    x.assign(n, 0.0);
    std::vector<double> r(n), z, p, q(n, 0.0);
    for (std::size_t i = 0; i < n; ++i) r[i] = slope[i] > 0.0 ? rhs[i] : 0.0;
    vcycle_sgs(h, 0, r, z);
    p = z;
    double rho = dot(r, z);
    const double target = tol * std::sqrt(dot(r, r));
    int it = 0;
    while (it < max_it && std::sqrt(dot(r, r)) > target && rho > 0.0) {
        apply(F, p, q);
        const double alpha = rho / dot(p, q);
        for (std::size_t i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        vcycle_sgs(h, 0, r, z);
        const double next = dot(r, z);
        const double beta = next / rho;
        rho = next;
        for (std::size_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        ++it;
    }
    return it;
}

// Right-preconditioned BiCGSTAB (heat_transport.cpp:823-897) with the SGS V-cycle.
int bicgstab(const Hierarchy& h, const std::vector<double>& b, double tol, int max_it, std::vector<double>& x) {
    const Level& F = h.levels[0];
    const std::size_t n = F.size;
    x.assign(n, 0.0);
    std::vector<double> r = b, shadow = b, p(n, 0.0), v(n, 0.0), ph, s(n, 0.0), sh, t(n, 0.0);
    const double bn = std::sqrt(dot(b, b));
    if (!(bn > 0.0)) return 0;
    double rho = 1.0, alpha = 1.0, omega = 1.0;
    int it = 0;
    while (it < max_it) {
        const double rn = dot(shadow, r);
        if (rn == 0.0 || omega == 0.0) break;
        const double beta = rn / rho * (alpha / omega);
        rho = rn;
        for (std::size_t i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
        vcycle_sgs(h, 0, p, ph);
        apply(F, ph, v);
        const double sv = dot(shadow, v);
        if (sv == 0.0) break;
        alpha = rho / sv;
        for (std::size_t i = 0; i < n; ++i) s[i] = r[i] - alpha * v[i];
        ++it;
        if (std::sqrt(dot(s, s)) <= tol * bn) {
            for (std::size_t i = 0; i < n; ++i) x[i] += alpha * ph[i];
            break;
        }
        vcycle_sgs(h, 0, s, sh);
        apply(F, sh, t);
        const double tt = dot(t, t);
        omega = tt > 0.0 ? dot(t, s) / tt : 0.0;
        for (std::size_t i = 0; i < n; ++i) {
            x[i] += alpha * ph[i] + omega * sh[i];
            r[i] = s[i] - omega * t[i];
        }
        if (std::sqrt(dot(r, r)) <= tol * bn) break;
    }
    return it;
}

void diffusion(const Graph& g, double K, const double* t, double* out) {
    for (std::size_t c = 0; c < g.n; ++c) {
        const double own = t[c];
        double sum = 0.0;
        for (std::size_t k = g.offset[c]; k < g.offset[c + 1]; ++k) sum += (t[g.neighbour[k]] - own) * g.weight[k];
        out[c] = K * sum / g.area[c];
    }
}

// ---- column radiation -------------------------------------------------------------

struct ColumnConstants {
    double tau_d, kappa_v, w_c, r_e, g_asym, kappa_l, p0, gravity, sigma;
};

// Bolton (1980) over water, Murphy and Koop (2005) over ice scaled to meet at 0 C.
double murphy_koop(double t) { return std::exp(9.550426 - 5723.265 / t + 3.53068 * std::log(t) - 0.00728332 * t); }

double saturation_vapour_pressure(double t) {
    if (t >= 273.15) return 611.2 * std::exp(17.67 * (t - 273.15) / (t - 29.65));
    return 611.2 / murphy_koop(273.15) * murphy_koop(t);
}

}  // namespace

extern "C" {

struct orc_mesh {
    std::uint64_t cells, edges;
    const std::uint32_t* edge_offset;
    const std::uint8_t* edge_count;
    const std::uint32_t* neighbor;
    const std::uint32_t* edge;
    const float* normal_east;
    const float* normal_north;
    const std::uint32_t* edge_first;
    const double* edge_length;
    const double* edge_distance;
    const double* area;
};

static Graph graph_of(const orc_graph* g) {
    return Graph{static_cast<std::size_t>(g->n), g->offset, g->neighbour, g->weight, g->weight_sum, g->area};
}

// laplacian<T> (finite_volume.cpp:91-111): (1/A) sum (phi_j - phi_i) l / d
void orc_laplacian_f64(const orc_mesh* m, const double* in, double* out) {
    for (std::size_t c = 0; c < m->cells; ++c) {
        double sum = 0.0;
        for (std::uint32_t k = 0; k < m->edge_count[c]; ++k) {
            const std::size_t d = m->edge_offset[c] + k, e = m->edge[d];
            sum += (in[m->neighbor[d]] - in[c]) * m->edge_length[e] / m->edge_distance[e];
        }
        out[c] = sum / m->area[c];
    }
}

void orc_laplacian_f32(const orc_mesh* m, const float* in, float* out) {
    for (std::size_t c = 0; c < m->cells; ++c) {
        const double own = static_cast<double>(in[c]);
        double sum = 0.0;
        for (std::uint32_t k = 0; k < m->edge_count[c]; ++k) {
            const std::size_t d = m->edge_offset[c] + k, e = m->edge[d];
            sum += (static_cast<double>(in[m->neighbor[d]]) - own) * m->edge_length[e] / m->edge_distance[e];
        }
        out[c] = static_cast<float>(sum / m->area[c]);
    }
}

}  // extern "C"

// gradient<T> (finite_volume.cpp:55-89): least squares over the edge normals.
template <typename T>
static void gradient_impl(const orc_mesh* m, const T* in, T* east, T* north) {
    for (std::size_t c = 0; c < m->cells; ++c) {
        const double own = static_cast<double>(in[c]);
        double mee = 0.0, men = 0.0, mnn = 0.0, re = 0.0, rn = 0.0;
        for (std::uint32_t k = 0; k < m->edge_count[c]; ++k) {
            const std::size_t d = m->edge_offset[c] + k;
            const double a = static_cast<double>(m->normal_east[d]);
            const double b = static_cast<double>(m->normal_north[d]);
            const double slope = (static_cast<double>(in[m->neighbor[d]]) - own) / m->edge_distance[m->edge[d]];
            mee += a * a;
            men += a * b;
            mnn += b * b;
            re += slope * a;
            rn += slope * b;
        }
        const double det = mee * mnn - men * men;
        east[c] = static_cast<T>((mnn * re - men * rn) / det);
        north[c] = static_cast<T>((mee * rn - men * re) / det);
    }
}
extern "C" {
void orc_gradient_f64(const orc_mesh* m, const double* in, double* e, double* n) { gradient_impl(m, in, e, n); }
void orc_gradient_f32(const orc_mesh* m, const float* in, float* e, float* n) { gradient_impl(m, in, e, n); }

}  // extern "C"

// divergence<T> (finite_volume.cpp:34-53): (1/A) sum s F l
template <typename T>
static void divergence_impl(const orc_mesh* m, const T* flux, T* out) {
    for (std::size_t c = 0; c < m->cells; ++c) {
        double net = 0.0;
        for (std::uint32_t k = 0; k < m->edge_count[c]; ++k) {
            const std::size_t e = m->edge[m->edge_offset[c] + k];
            const double orient = m->edge_first[e] == c ? 1.0 : -1.0;
            net += orient * static_cast<double>(flux[e]) * m->edge_length[e];
        }
        out[c] = static_cast<T>(net / m->area[c]);
    }
}
extern "C" {
void orc_divergence_f64(const orc_mesh* m, const double* f, double* o) { divergence_impl(m, f, o); }
void orc_divergence_f32(const orc_mesh* m, const float* f, float* o) { divergence_impl(m, f, o); }

void orc_diffusion_source(const orc_graph* g, double K, const double* t, double* out) {
    diffusion(graph_of(g), K, t, out);
}

// ---- hierarchy -----------------------------------------------------------------------
void* orc_hierarchy_new(const orc_graph* g) { return new Hierarchy(build(graph_of(g))); }
void orc_hierarchy_free(void* h) { delete static_cast<Hierarchy*>(h); }
std::uint64_t orc_hierarchy_levels(void* h) { return static_cast<Hierarchy*>(h)->levels.size(); }

// sizes = {rows, off-diagonals, aggregate length, target length}; pointers stay valid
// while the hierarchy lives.
void orc_hierarchy_level(void* hp, std::uint64_t l, std::uint64_t* sizes, const std::uint32_t** off,
                         const std::uint32_t** col, const std::uint32_t** agg, const std::int64_t** tgt) {
    Hierarchy& h = *static_cast<Hierarchy*>(hp);
    sizes[0] = h.levels[l].size;
    sizes[1] = h.x_col[l].size();
    sizes[2] = h.x_agg[l].size();
    sizes[3] = h.x_tgt[l].size();
    *off = h.x_off[l].data();
    *col = h.x_col[l].data();
    *agg = h.x_agg[l].data();
    *tgt = h.x_tgt[l].data();
}

// GraphMultigrid::set_matrix (heat_transport.cpp:559-571)
void orc_hierarchy_set_matrix(void* hp, const double* diag, const double* off) {
    Hierarchy& h = *static_cast<Hierarchy*>(hp);
    Level& F = h.levels[0];
    std::copy(diag, diag + F.size, F.diag.begin());
    std::copy(off, off + F.val.size(), F.val.begin());
    set_values(h);
}

// Galerkin values of level l: diagonal [rows], off-diagonals [CSR order].
void orc_hierarchy_values(void* hp, std::uint64_t l, double* diag, double* off) {
    const Level& L = static_cast<Hierarchy*>(hp)->levels[l];
    std::copy(L.diag.begin(), L.diag.end(), diag);
    std::copy(L.val.begin(), L.val.end(), off);
}

void orc_vcycle_sgs(void* hp, const double* rhs, double* out) {
    const Hierarchy& h = *static_cast<Hierarchy*>(hp);
    std::vector<double> b(rhs, rhs + h.levels[0].size), x;
    vcycle_sgs(h, 0, b, x);
    std::copy(x.begin(), x.end(), out);
}

void orc_vcycle_jacobi(void* hp, int pre, int post, double omega, double correction, const double* rhs,
                       double* out) {
    const Hierarchy& h = *static_cast<Hierarchy*>(hp);
    std::vector<double> b(rhs, rhs + h.levels[0].size), x;
    vcycle_jacobi(h, 0, pre, post, omega, correction, b, x);
    std::copy(x.begin(), x.end(), out);
}

// solve_newton_system: assemble (A/s + K L), Galerkin, Cholesky, PCG; returns iterations.
int orc_pcg(void* hp, const orc_graph* g, double K, const double* edge_g, const double* slope, const double* rhs,
            double tol, int max_it, double* x_out) {
    Hierarchy& h = *static_cast<Hierarchy*>(hp);
    const Graph gr = graph_of(g);
    std::vector<double> s(slope, slope + gr.n), b(rhs, rhs + gr.n), x;
    assemble(h, gr, K, edge_g, s);
    const int it = pcg(h, s, b, tol, max_it, x);
    std::copy(x.begin(), x.end(), x_out);
    return it;
}

int orc_bicgstab(void* hp, const orc_graph* g, double K, const double* slope, const double* rhs, double tol,
                 int max_it, double* x_out) {
    Hierarchy& h = *static_cast<Hierarchy*>(hp);
    const Graph gr = graph_of(g);
    std::vector<double> s(slope, slope + gr.n), b(rhs, rhs + gr.n), x;
    assemble(h, gr, K, nullptr, s);
    const int it = bicgstab(h, b, tol, max_it, x);
    std::copy(x.begin(), x.end(), x_out);
    return it;
}

}  // extern "C"

namespace {

// solve_implicit_transport (heat_transport.cpp:595-772) for a response(at, mean, slope)
// and a per-cell floor. stats = {newton, cg, consistency, sum, abs, dissipation}.
template <typename Response>
void implicit_transport(const Graph& g, double K, Response&& response, const double* floor, double cg_tol,
                        double newton_tol, double* mean_out, double* source_out, double* stats) {
    const std::size_t n = g.n;
    Hierarchy h = build(g);
    const int max_newton = 30, max_halvings = 12, max_non_monotone = 4;
    const double rounding_floor = 1e-3, max_growth = 100.0;
    std::vector<double> source(n, 0.0), mean(n), slope(n), diff(n), resid(n), rhs(n), dmean, dsource(n), trial(n),
        tmean(n), tslope(n);
    for (std::size_t c = 0; c < n; ++c) source[c] = std::max(0.0, floor[c]);
    auto evaluate = [&](const std::vector<double>& at, std::vector<double>& at_mean, std::vector<double>& at_slope,
                        std::vector<double>& at_resid) {
        response(at, at_mean, at_slope);
        diffusion(g, K, at_mean.data(), diff.data());
        return block_sum(n, [&](std::size_t c) {
            at_resid[c] = at[c] - diff[c];
            return g.area[c] * at_resid[c] * at_resid[c];
        });
    };
    auto max_abs = [&](const std::vector<double>& v) {
        double m = 0.0;
        for (std::size_t b = 0; b < n; b += kBlock) {
            double part = 0.0;
            for (std::size_t i = b; i < std::min(n, b + kBlock); ++i) part = std::max(part, std::abs(v[i]));
            m = std::max(m, part);
        }
        return m;
    };
    double merit = evaluate(source, mean, slope, resid);
    int newton = 0, cg = 0, non_monotone = 0;
    for (int iteration = 0; iteration < max_newton; ++iteration) {
        if (max_abs(resid) <= newton_tol) break;
        for (std::size_t c = 0; c < n; ++c) rhs[c] = -resid[c] * g.area[c];
        assemble(h, g, K, nullptr, slope);
        cg += pcg(h, slope, rhs, cg_tol, 2000, dmean);
        diffusion(g, K, dmean.data(), dsource.data());
        for (std::size_t c = 0; c < n; ++c) dsource[c] -= resid[c];
        double step = 1.0, trial_merit = 0.0;
        for (int halving = 0;; ++halving) {
            for (std::size_t c = 0; c < n; ++c) trial[c] = std::max(source[c] + step * dsource[c], floor[c]);
            std::vector<double> tresid(n, 0.0);
            trial_merit = evaluate(trial, tmean, tslope, tresid);
            if (trial_merit < merit) {
                resid = std::move(tresid);
                break;
            }
            if (halving == max_halvings) {
                if (max_abs(resid) <= rounding_floor || non_monotone == max_non_monotone) {
                    step = 0.0;
                } else {
                    ++non_monotone;
                    step = 1.0;
                    for (std::size_t c = 0; c < n; ++c) trial[c] = std::max(source[c] + dsource[c], floor[c]);
                    trial_merit = evaluate(trial, tmean, tslope, tresid);
                    if (std::isfinite(trial_merit) && trial_merit <= max_growth * merit) resid = std::move(tresid);
                    else step = 0.0;
                }
                break;
            }
            step *= 0.5;
        }
        if (step == 0.0) break;
        std::swap(source, trial);
        std::swap(mean, tmean);
        std::swap(slope, tslope);
        merit = trial_merit;
        ++newton;
    }
    diffusion(g, K, mean.data(), source_out);
    std::copy(mean.begin(), mean.end(), mean_out);
    double s = 0.0, a = 0.0, d = 0.0;
    for (std::size_t b = 0; b < n; b += kBlock) {
        double ps = 0.0, pa = 0.0, pd = 0.0;
        for (std::size_t c = b; c < std::min(n, b + kBlock); ++c) {
            const double flux = g.area[c] * source_out[c];
            ps += flux;
            pa += std::abs(flux);
            pd += flux * mean[c];
        }
        s += ps;
        a += pa;
        d += pd;
    }
    stats[0] = newton;
    stats[1] = cg;
    stats[2] = max_abs(resid);
    stats[3] = s;
    stats[4] = a;
    stats[5] = d;
}

// The quartic tile response of tests/unit/test_heat_transport.cpp:30-76: a x + r x^4 = b + h
// per cell, r = 0.75 * 0.97 * sigma, root by the dry Newton of solve_column_surface
// (sim/planet/surface/column_step.cpp:255-270: start at the smaller single-term root, at
// most column_newton_iterations = 10 steps, stop once a step is within 4 eps of x); slope
// dx/dh = 1 / (a + 4 r x^3) (column_step.cpp:273-276). Cells whose index is a multiple of
// seven hold at 273.15 K with slope 0 when they would warm past it.
void quartic_response(std::size_t n, double a, const double* b, const double* source, double* mean, double* slope) {
    const double r = 0.75 * 0.97 * 5.670374419e-8;
    for (std::size_t c = 0; c < n; ++c) {
        const double rhs = b[c] + source[c];
        double x = std::min(rhs / a, std::sqrt(std::sqrt(rhs / r)));
        for (int it = 0; it < 10; ++it) {
            const double x3 = x * x * x;
            const double value = a * x + r * x3 * x - rhs;
            const double d = a + 4.0 * r * x3;
            const double step = value / d;
            x -= step;
            if (std::abs(step) <= 4.0 * std::numeric_limits<double>::epsilon() * x) break;
        }
        if (c % 7U == 0U && x > 273.15) {
            mean[c] = 273.15;
            slope[c] = 0.0;
            continue;
        }
        mean[c] = x;
        slope[c] = 1.0 / (a + 4.0 * r * x * x * x + 0.0);
    }
}

}  // namespace

extern "C" {

// The linear response mean = base + slope h with floor = -inf.
void orc_solve_implicit_transport_linear(const orc_graph* gp, double K, const double* base, const double* slope_in,
                                         double cg_tol, double newton_tol, double* mean_out, double* source_out,
                                         double* stats) {
    const Graph g = graph_of(gp);
    const std::vector<double> floor(g.n, -std::numeric_limits<double>::infinity());
    implicit_transport(
        g, K,
        [&](const std::vector<double>& at, std::vector<double>& mean, std::vector<double>& slope) {
            for (std::size_t c = 0; c < g.n; ++c) {
                mean[c] = base[c] + slope_in[c] * at[c];
                slope[c] = slope_in[c];
            }
        },
        floor.data(), cg_tol, newton_tol, mean_out, source_out, stats);
}

void orc_quartic_response(std::uint64_t n, double a, const double* b, const double* source, double* mean,
                          double* slope) {
    quartic_response(n, a, b, source, mean, slope);
}

// The quartic response with the test's floor (the source that puts a column at 100 K).
void orc_solve_implicit_transport_quartic(const orc_graph* gp, double K, double a, const double* b, double cg_tol,
                                          double newton_tol, double* floor_out, double* mean_out, double* source_out,
                                          double* stats) {
    const Graph g = graph_of(gp);
    const double r = 0.75 * 0.97 * 5.670374419e-8;
    for (std::size_t c = 0; c < g.n; ++c) {
        const double x = 100.0;
        floor_out[c] = a * x + r * x * x * x * x - b[c];
    }
    implicit_transport(
        g, K,
        [&](const std::vector<double>& at, std::vector<double>& mean, std::vector<double>& slope) {
            quartic_response(g.n, a, b, at.data(), mean.data(), slope.data());
        },
        floor_out, cg_tol, newton_tol, mean_out, source_out, stats);
}

// The same solve on an agglomerated graph with the production group response
// (surface_energy.cpp:1240-1296): every fine cell answers the quartic at its group's source
// (the hold rule on the fine cell's index), a group takes the area-weighted means of its
// cells (summed in cell order) over the group's area. `floor` per group.
void orc_solve_implicit_transport_group_quartic(const orc_graph* gp, std::uint64_t fine_cells,
                                                const std::uint32_t* group_of_cell, const double* fine_area,
                                                double K, double a, const double* b_fine, const double* floor,
                                                double cg_tol, double newton_tol, double* mean_out,
                                                double* source_out, double* stats) {
    const Graph g = graph_of(gp);
    std::vector<double> floor_v(floor, floor + g.n), h_fine(fine_cells), mean_f(fine_cells), slope_f(fine_cells),
        air(g.n), air_slope(g.n);
    implicit_transport(
        g, K,
        [&](const std::vector<double>& at, std::vector<double>& mean, std::vector<double>& slope) {
            for (std::size_t c = 0; c < fine_cells; ++c) h_fine[c] = at[group_of_cell[c]];
            quartic_response(fine_cells, a, b_fine, h_fine.data(), mean_f.data(), slope_f.data());
            std::fill(air.begin(), air.end(), 0.0);
            std::fill(air_slope.begin(), air_slope.end(), 0.0);
            for (std::size_t c = 0; c < fine_cells; ++c) {
                air[group_of_cell[c]] += fine_area[c] * mean_f[c];
                air_slope[group_of_cell[c]] += fine_area[c] * slope_f[c];
            }
            for (std::size_t n = 0; n < g.n; ++n) {
                mean[n] = air[n] / g.area[n];
                slope[n] = air_slope[n] / g.area[n];
            }
        },
        floor_v.data(), cg_tol, newton_tol, mean_out, source_out, stats);
}

// The implicit sub-step with the linear column response, solved directly with the
// reference PCG: (A/s + K L) T = (A/s) T0 + A S, s = dt/C; then H = flux form of T and
// T_new = T0 + s (S + H). sums = {sum A H, sum A|H|, sum A H T, sum A S, sum A|S|,
// sum A (T_new - T0)/s}. edge_g: optional per-CSR-entry conductance. Returns PCG iterations.
int orc_transport_step(void* hp, const orc_graph* gp, double K, const double* edge_g, double C, double dt,
                       const double* t0, const double* src, double tol, int max_it, double* t_solved, double* h_out,
                       double* t_new, double* sums) {
    Hierarchy& h = *static_cast<Hierarchy*>(hp);
    const Graph g = graph_of(gp);
    const std::size_t n = g.n;
    const double s = dt / C;
    std::vector<double> slope(n, s), b(n), x;
    for (std::size_t c = 0; c < n; ++c) b[c] = g.area[c] / s * t0[c] + g.area[c] * src[c];
    assemble(h, g, K, edge_g, slope);
    const int it = pcg(h, slope, b, tol, max_it, x);
    for (std::size_t c = 0; c < n; ++c) {
        double sum = 0.0;
        for (std::size_t k = g.offset[c]; k < g.offset[c + 1]; ++k) {
            sum += edge_g != nullptr ? (edge_g[k] * g.weight[k]) * (x[g.neighbour[k]] - x[c])
                                     : (x[g.neighbour[k]] - x[c]) * g.weight[k];
        }
        h_out[c] = edge_g != nullptr ? sum / g.area[c] : K * sum / g.area[c];
        t_new[c] = t0[c] + s * (src[c] + h_out[c]);
        t_solved[c] = x[c];
    }
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (std::size_t b0 = 0; b0 < n; b0 += kBlock) {
        double p[6] = {0, 0, 0, 0, 0, 0};
        for (std::size_t c = b0; c < std::min(n, b0 + kBlock); ++c) {
            const double flux = g.area[c] * h_out[c];
            p[0] += flux;
            p[1] += std::abs(flux);
            p[2] += flux * x[c];
            p[3] += g.area[c] * src[c];
            p[4] += std::abs(g.area[c] * src[c]);
            p[5] += g.area[c] * ((t_new[c] - t0[c]) / s);
        }
        for (int q = 0; q < 6; ++q) acc[q] += p[q];
    }
    std::copy(acc, acc + 6, sums);
    return it;
}

// ---- column radiation: N equal-mass layers, layer-major arrays -------------------------
void orc_column_radiation(std::uint64_t cells, std::uint32_t layers, const double* kk, const double* temp,
                          const double* hum, const double* cloud, const double* ts, const double* ps, double* emissivity,
                          double* absorbed, double* fraction, double* reflectance, double* scalars) {
    const ColumnConstants k{kk[0], kk[1], kk[2], kk[3], kk[4], kk[5], kk[6], kk[7], kk[8]};
    const std::size_t L = layers;
    std::vector<double> eps(L), em(L), above(L);
    for (std::size_t c = 0; c < cells; ++c) {
        const double layer_pa = ps[c] / static_cast<double>(L);
        const double dry = k.tau_d * layer_pa / k.p0;
        const double mass = ps[c] / (k.gravity * static_cast<double>(L));
        const double omg = 1.0 - k.g_asym;
        double clear = 1.0, trans = 1.0, col_tau = 0.0;
        for (std::size_t l = 0; l < L; ++l) {
            const std::size_t i = l * cells + c;
            const double vapour = std::max(0.0, hum[i]) * layer_pa / k.gravity;
            eps[l] = -std::expm1(-(dry + k.kappa_v * vapour));
            fraction[i] = 0.0;
            reflectance[i] = 0.0;
            const double path = std::max(0.0, cloud[i]) * mass;
            if (!(path > 0.0)) continue;
            const double f = std::min(1.0, path / k.w_c);
            const double tau = 3.0 * (path / f) / (2.0 * 1000.0 * k.r_e);
            fraction[i] = f;
            clear *= 1.0 - f;
            reflectance[i] = f * omg * tau / (2.0 + omg * tau);
            trans *= 1.0 - reflectance[i];
            col_tau += f * tau;
            const double lw = k.kappa_l * path;
            if (lw > 0.0) eps[l] = -std::expm1(std::log1p(-eps[l]) - lw);
        }
        for (std::size_t l = 0; l < L; ++l) {
            const double t2 = temp[l * cells + c] * temp[l * cells + c];
            em[l] = eps[l] * k.sigma * t2 * t2;
            emissivity[l * cells + c] = eps[l];
        }
        double down = 0.0;
        for (std::size_t l = L; l-- > 0;) {
            above[l] = down;
            down = (1.0 - eps[l]) * down + em[l];
        }
        const double ts2 = ts[c] * ts[c];
        double up = k.sigma * ts2 * ts2;
        for (std::size_t l = 0; l < L; ++l) {
            absorbed[l * cells + c] = eps[l] * (up + above[l]);
            up = (1.0 - eps[l]) * up + em[l];
        }
        scalars[c] = down;
        scalars[cells + c] = up;
        scalars[2 * cells + c] = trans;
        scalars[3 * cells + c] = 1.0 - clear;
        scalars[4 * cells + c] = col_tau;
    }
}

// q_sat = eps e / (p - (1 - eps) e), capped at 1 (saturation.cpp:43-50).
double orc_saturation_specific_humidity(double t, double p) {
    const double eps = 287.04 / 461.5;
    const double e = saturation_vapour_pressure(t);
    const double den = p - (1.0 - eps) * e;
    if (!(den > eps * e)) return 1.0;
    return eps * e / den;
}

}  // extern "C"

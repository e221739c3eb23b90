// Test-only C-ABI driver over the reference PlanetSim library, compiled from the
// reference sources by oracle/Makefile.ref into oracle/_ref/libref_driver.so.
//
// This is oracle infrastructure: it is loaded only by tests/golden/make_golden.py
// (to write the golden fixtures) and by the pinning tests that compare the
// restated oracle (oracle/planetsim_oracle.cpp) with the reference itself. No
// product code loads it. It adds no arithmetic of its own: every number it returns
// is computed by the reference's functions named beside each entry point.
//
// heat_transport.cpp is included textually so that the anonymous-namespace
// multigrid pieces (Level, build_hierarchy, coarsen_values, v_cycle,
// solve_newton_system) can be driven directly, which is how the aggregates,
// coarse patterns and Galerkin scatter targets are checked bit for bit.

#include "sim/planet/surface/heat_transport.cpp"

#include "sim/core/math/incomplete_lu.hpp"
#include "sim/planet/atmosphere/atmosphere.hpp"
#include "sim/planet/atmosphere/atmosphere_column.hpp"
#include "sim/planet/atmosphere/saturation.hpp"
#include "sim/planet/mesh/icosphere.hpp"
#include "sim/planet/operators/finite_volume.hpp"
#include "sim/planet/orbit/climate_calendar.hpp"
#include "sim/planet/orbit/substep_forcing.hpp"
#include "sim/planet/planet_parameters.hpp"
#include "sim/planet/surface/column_step.hpp"

#include <chrono>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <vector>

using namespace planetsim;

namespace {

struct RefHierarchy {
    std::vector<Level> levels;
};

std::vector<double> copy_in(const double* values, std::size_t n) {
    return std::vector<double>(values, values + n);
}

}  // namespace

extern "C" {

// ---- mesh: make_icosphere (sim/planet/mesh/icosphere.cpp:200-419) ----------
void* refd_mesh_new(std::uint32_t level, double radius_m) {
    return new PlanetMesh(make_icosphere(level, radius_m));
}

void refd_mesh_free(void* mesh) { delete static_cast<PlanetMesh*>(mesh); }

void refd_mesh_counts(void* handle, std::uint64_t* counts) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    counts[0] = mesh.cell_count();
    counts[1] = mesh.edge_count();
    counts[2] = mesh.directed_edge_count();
    counts[3] = mesh.corner_count();
}

// Per cell: centre/east/north (xyz each), area, source vertex, edge offset, edge count.
void refd_mesh_cells(void* handle, double* center, double* east, double* north, double* area,
                     std::uint32_t* source, std::uint32_t* edge_offset, std::uint8_t* edge_count) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    std::size_t i = 0;
    for (const auto& cell : mesh.cells()) {
        center[3 * i] = cell.center_unit.x;
        center[3 * i + 1] = cell.center_unit.y;
        center[3 * i + 2] = cell.center_unit.z;
        east[3 * i] = cell.east_unit.x;
        east[3 * i + 1] = cell.east_unit.y;
        east[3 * i + 2] = cell.east_unit.z;
        north[3 * i] = cell.north_unit.x;
        north[3 * i + 1] = cell.north_unit.y;
        north[3 * i + 2] = cell.north_unit.z;
        area[i] = cell.area_m2;
        source[i] = cell.source_vertex_index;
        edge_offset[i] = cell.edge_offset;
        edge_count[i] = cell.edge_count;
        ++i;
    }
}

void refd_mesh_cell_edges(void* handle, std::uint32_t* neighbor, std::uint32_t* edge,
                          float* normal_east, float* normal_north) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    std::size_t k = 0;
    for (const auto& cell : mesh.cells()) {
        for (const auto& ce : mesh.cell_edges(cell.id)) {
            neighbor[k] = ce.neighbor.value();
            edge[k] = ce.edge.value();
            normal_east[k] = ce.outward_normal_east;
            normal_north[k] = ce.outward_normal_north;
            ++k;
        }
    }
}

void refd_mesh_edges(void* handle, std::uint32_t* first, std::uint32_t* second, double* length,
                     double* distance) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    std::size_t e = 0;
    for (const auto& edge : mesh.edges()) {
        first[e] = edge.first_cell.value();
        second[e] = edge.second_cell.value();
        length[e] = edge.length_m;
        distance[e] = edge.centroid_distance_m;
        ++e;
    }
}

void refd_mesh_corners(void* handle, double* corners, std::uint32_t* cell_corner) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    std::size_t c = 0;
    for (const auto& corner : mesh.corners_unit()) {
        corners[3 * c] = corner.x;
        corners[3 * c + 1] = corner.y;
        corners[3 * c + 2] = corner.z;
        ++c;
    }
    std::size_t k = 0;
    for (const auto& cell : mesh.cells()) {
        for (const auto index : mesh.cell_corners(cell.id)) {
            cell_corner[k++] = index;
        }
    }
}

// ---- transport graph: mesh_transport_graph (heat_transport.cpp:433-452) ----
void refd_graph(void* handle, double* area, std::uint64_t* offset, std::uint64_t* neighbour,
                double* weight, double* weight_sum) {
    const auto graph = mesh_transport_graph(*static_cast<PlanetMesh*>(handle));
    for (std::size_t i = 0; i < graph.size(); ++i) {
        area[i] = graph.area_m2[i];
        weight_sum[i] = graph.weight_sum[i];
    }
    for (std::size_t i = 0; i < graph.offset.size(); ++i) {
        offset[i] = graph.offset[i];
    }
    for (std::size_t k = 0; k < graph.neighbour.size(); ++k) {
        neighbour[k] = graph.neighbour[k];
        weight[k] = graph.weight[k];
    }
}

// ---- agglomerated graph: agglomerated_transport_graph (heat_transport.cpp:467-539) ----
void refd_agglomeration_counts(void* handle, std::uint64_t* counts) {
    const std::vector<std::size_t>* groups = nullptr;
    const auto& graph = agglomerated_transport_graph(*static_cast<PlanetMesh*>(handle), groups);
    counts[0] = graph.size();
    counts[1] = graph.neighbour.size();
    counts[2] = groups->size();
}

void refd_agglomeration(void* handle, double* area, std::uint64_t* offset, std::uint64_t* neighbour,
                        double* weight, double* weight_sum, std::uint64_t* group_of_cell) {
    const std::vector<std::size_t>* groups = nullptr;
    const auto& graph = agglomerated_transport_graph(*static_cast<PlanetMesh*>(handle), groups);
    for (std::size_t i = 0; i < graph.size(); ++i) {
        area[i] = graph.area_m2[i];
        weight_sum[i] = graph.weight_sum[i];
    }
    for (std::size_t i = 0; i < graph.offset.size(); ++i) offset[i] = graph.offset[i];
    for (std::size_t k = 0; k < graph.neighbour.size(); ++k) {
        neighbour[k] = graph.neighbour[k];
        weight[k] = graph.weight[k];
    }
    for (std::size_t c = 0; c < groups->size(); ++c) group_of_cell[c] = (*groups)[c];
}

// ---- hierarchy: build_hierarchy (heat_transport.cpp:175-200) --------------
void* refd_hierarchy_new(void* handle) {
    const auto graph = mesh_transport_graph(*static_cast<PlanetMesh*>(handle));
    auto* h = new RefHierarchy;
    h->levels = build_hierarchy(graph, graph.size());
    return h;
}

void refd_hierarchy_free(void* h) { delete static_cast<RefHierarchy*>(h); }

std::uint64_t refd_hierarchy_level_count(void* h) {
    return static_cast<RefHierarchy*>(h)->levels.size();
}

// sizes[0] = rows, sizes[1] = off-diagonal entries, sizes[2] = aggregate length,
// sizes[3] = target length.
void refd_hierarchy_level_sizes(void* h, std::uint64_t index, std::uint64_t* sizes) {
    const Level& level = static_cast<RefHierarchy*>(h)->levels[index];
    sizes[0] = level.size;
    sizes[1] = level.column.size();
    sizes[2] = level.aggregate.size();
    sizes[3] = level.target.size();
}

// Integer structure of one level; `target` uses -1 for the aggregate's diagonal.
void refd_hierarchy_level(void* h, std::uint64_t index, std::int64_t* offset,
                          std::int64_t* column, std::int64_t* aggregate, std::int64_t* target,
                          double* diagonal, double* value) {
    const Level& level = static_cast<RefHierarchy*>(h)->levels[index];
    for (std::size_t i = 0; i < level.offset.size(); ++i) offset[i] = static_cast<std::int64_t>(level.offset[i]);
    for (std::size_t i = 0; i < level.column.size(); ++i) column[i] = static_cast<std::int64_t>(level.column[i]);
    for (std::size_t i = 0; i < level.aggregate.size(); ++i) aggregate[i] = static_cast<std::int64_t>(level.aggregate[i]);
    for (std::size_t i = 0; i < level.target.size(); ++i) {
        target[i] = level.target[i] == diagonal_target ? -1 : static_cast<std::int64_t>(level.target[i]);
    }
    for (std::size_t i = 0; i < level.diagonal.size(); ++i) diagonal[i] = level.diagonal[i];
    for (std::size_t i = 0; i < level.value.size(); ++i) value[i] = level.value[i];
}

// set_matrix on the hierarchy: fine values in, Galerkin values on every level
// (coarsen_values, heat_transport.cpp:157-171) and the coarsest Cholesky
// factor (factor_dense, :202-226).
void refd_hierarchy_set_matrix(void* h, const double* diagonal, const double* off) {
    auto& levels = static_cast<RefHierarchy*>(h)->levels;
    Level& fine = levels.front();
    std::copy(diagonal, diagonal + fine.size, fine.diagonal.begin());
    std::copy(off, off + fine.value.size(), fine.value.begin());
    for (std::size_t index = 0; index + 1U < levels.size(); ++index) {
        coarsen_values(levels[index], levels[index + 1U]);
    }
    factor_dense(levels.back());
}

void refd_hierarchy_factor(void* h, double* factor) {
    const auto& level = static_cast<RefHierarchy*>(h)->levels.back();
    std::copy(level.factor.begin(), level.factor.end(), factor);
}

// One V-cycle (v_cycle, heat_transport.cpp:288-326) with the mesh's 256-cell blocks.
void refd_hierarchy_vcycle(void* h, void* mesh_handle, const double* rhs, double* out) {
    const auto& levels = static_cast<RefHierarchy*>(h)->levels;
    const auto& mesh = *static_cast<PlanetMesh*>(mesh_handle);
    const Parallel parallel{mesh.blocks(), 1U};
    std::vector<double> b = copy_in(rhs, levels.front().size);
    std::vector<double> x;
    v_cycle(levels, 0U, b, x, parallel);
    std::copy(x.begin(), x.end(), out);
}

// ---- FV operators (finite_volume.cpp:34-111) --------------------------------
void refd_laplacian_f64(void* handle, const double* in, double* out) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    Field2D<double> scalar(copy_in(in, mesh.cell_count()));
    Field2D<double> result(mesh.cell_count(), 0.0);
    laplacian(mesh, scalar, result, 1U);
    std::copy(result.values().begin(), result.values().end(), out);
}

void refd_laplacian_f32(void* handle, const float* in, float* out) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    Field2D<float> scalar(std::vector<float>(in, in + mesh.cell_count()));
    Field2D<float> result(mesh.cell_count(), 0.0F);
    laplacian(mesh, scalar, result, 1U);
    std::copy(result.values().begin(), result.values().end(), out);
}

void refd_gradient_f64(void* handle, const double* in, double* east, double* north) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    Field2D<double> scalar(copy_in(in, mesh.cell_count()));
    Field2D<double> e(mesh.cell_count(), 0.0);
    Field2D<double> n(mesh.cell_count(), 0.0);
    gradient(mesh, scalar, e, n, 1U);
    std::copy(e.values().begin(), e.values().end(), east);
    std::copy(n.values().begin(), n.values().end(), north);
}

void refd_gradient_f32(void* handle, const float* in, float* east, float* north) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    Field2D<float> scalar(std::vector<float>(in, in + mesh.cell_count()));
    Field2D<float> e(mesh.cell_count(), 0.0F);
    Field2D<float> n(mesh.cell_count(), 0.0F);
    gradient(mesh, scalar, e, n, 1U);
    std::copy(e.values().begin(), e.values().end(), east);
    std::copy(n.values().begin(), n.values().end(), north);
}

void refd_divergence_f64(void* handle, const double* flux, double* out) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    EdgeField<double> edge_flux(mesh.edge_count(), 0.0);
    for (std::size_t e = 0; e < mesh.edge_count(); ++e) {
        edge_flux[EdgeId{static_cast<std::uint32_t>(e)}] = flux[e];
    }
    Field2D<double> result(mesh.cell_count(), 0.0);
    divergence(mesh, edge_flux, result, 1U);
    std::copy(result.values().begin(), result.values().end(), out);
}

void refd_divergence_f32(void* handle, const float* flux, float* out) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    EdgeField<float> edge_flux(mesh.edge_count(), 0.0F);
    for (std::size_t e = 0; e < mesh.edge_count(); ++e) {
        edge_flux[EdgeId{static_cast<std::uint32_t>(e)}] = flux[e];
    }
    Field2D<float> result(mesh.cell_count(), 0.0F);
    divergence(mesh, edge_flux, result, 1U);
    std::copy(result.values().begin(), result.values().end(), out);
}

// ---- diffusion_source (heat_transport.cpp:579-593) --------------------------
void refd_diffusion_source(void* handle, double conductance, const double* temperature,
                           double* source) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    const auto graph = mesh_transport_graph(mesh);
    Field2D<double> t(copy_in(temperature, mesh.cell_count()));
    Field2D<double> s;
    diffusion_source(graph, conductance, t, s, 1U);
    std::copy(s.values().begin(), s.values().end(), source);
}

// ---- solve_implicit_transport with a linear response (heat_transport.cpp:595-772)
// mean = base + slope * h. stats: [newton, cg, consistency, sum, abs_sum, dissipation].
void refd_solve_linear(void* handle, double conductance, const double* base, const double* slope,
                       double cg_tolerance, double newton_tolerance, std::uint64_t workers,
                       double* mean_out, double* source_out, double* stats) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    const auto graph = mesh_transport_graph(mesh);
    const std::size_t n = mesh.cell_count();
    const TransportResponse response = [&](const Field2D<double>& source, Field2D<double>& mean,
                                           Field2D<double>& slope_out) {
        for (std::size_t cell = 0; cell < n; ++cell) {
            mean[cell] = base[cell] + slope[cell] * source[cell];
            slope_out[cell] = slope[cell];
        }
    };
    const Field2D<double> floor(n, -std::numeric_limits<double>::infinity());
    ImplicitTransportSettings settings;
    settings.cg_relative_tolerance = cg_tolerance;
    settings.newton_tolerance_W_m2 = newton_tolerance;
    const auto result = solve_implicit_transport(graph, conductance, floor, response, settings,
                                                 static_cast<std::size_t>(workers));
    std::copy(result.mean_K.values().begin(), result.mean_K.values().end(), mean_out);
    std::copy(result.source_W_m2.values().begin(), result.source_W_m2.values().end(), source_out);
    stats[0] = result.newton_iterations;
    stats[1] = result.cg_iterations;
    stats[2] = result.consistency_residual_W_m2;
    stats[3] = result.sum_W;
    stats[4] = result.absolute_sum_W;
    stats[5] = result.dissipation_W_K;
}

// ---- the nonlinear transport solve with the reference test's quartic response -----
// The tile-like response of tests/unit/test_heat_transport.cpp:30-76: a x + r x^4 = b + h
// per cell, solved by the reference's solve_column_surface; cells whose index is a
// multiple of seven hold at 273.15 K (slope 0) when they would warm past it.
static void quartic_response(std::size_t n, double a, const double* b, const Field2D<double>& source,
                             Field2D<double>& mean, Field2D<double>& slope) {
    const double radiative = 0.75 * 0.97 * stefan_boltzmann_W_m2_K4;
    for (std::size_t cell = 0; cell < n; ++cell) {
        ColumnSystem system;
        system.a = a;
        system.b = b[cell] + source[cell];
        system.radiative = radiative;
        const double x = solve_column_surface(system);
        if (cell % 7U == 0U && x > 273.15) {
            mean[cell] = 273.15;
            slope[cell] = 0.0;
            continue;
        }
        mean[cell] = x;
        slope[cell] = system.slope_K_m2_W(x);
    }
}

void refd_quartic_response(std::uint64_t n, double a, const double* b, const double* source, double* mean_out,
                           double* slope_out) {
    Field2D<double> h(copy_in(source, n)), mean(n, 0.0), slope(n, 0.0);
    quartic_response(n, a, b, h, mean, slope);
    std::copy(mean.values().begin(), mean.values().end(), mean_out);
    std::copy(slope.values().begin(), slope.values().end(), slope_out);
}

// solve_implicit_transport with that response; the floor is the test's floor(): the
// source that puts every column at 100 K.
void refd_solve_quartic(void* handle, double a, double conductance, const double* b, double cg_tolerance,
                        double newton_tolerance, std::uint64_t workers, double* floor_out, double* mean_out,
                        double* source_out, double* stats) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    const auto graph = mesh_transport_graph(mesh);
    const std::size_t n = mesh.cell_count();
    const double radiative = 0.75 * 0.97 * stefan_boltzmann_W_m2_K4;
    Field2D<double> floor(n, 0.0);
    for (std::size_t cell = 0; cell < n; ++cell) {
        const double x = 100.0;
        floor[cell] = a * x + radiative * x * x * x * x - b[cell];
    }
    const TransportResponse response = [&](const Field2D<double>& source, Field2D<double>& mean,
                                           Field2D<double>& slope) { quartic_response(n, a, b, source, mean, slope); };
    ImplicitTransportSettings settings;
    settings.cg_relative_tolerance = cg_tolerance;
    settings.newton_tolerance_W_m2 = newton_tolerance;
    const auto result = solve_implicit_transport(graph, conductance, floor, response, settings,
                                                 static_cast<std::size_t>(workers));
    std::copy(floor.values().begin(), floor.values().end(), floor_out);
    std::copy(result.mean_K.values().begin(), result.mean_K.values().end(), mean_out);
    std::copy(result.source_W_m2.values().begin(), result.source_W_m2.values().end(), source_out);
    stats[0] = result.newton_iterations;
    stats[1] = result.cg_iterations;
    stats[2] = result.consistency_residual_W_m2;
    stats[3] = result.sum_W;
    stats[4] = result.absolute_sum_W;
    stats[5] = result.dissipation_W_K;
}

// The same solve on the agglomerated graph of a fine mesh, as the production step runs it
// (surface_energy.cpp:1219-1300, 1589-1597): each fine cell answers the quartic at its
// group's source, a group's mean and slope are the area-weighted means of its cells'
// (summed in cell order, over the group's area); the floor of a group is the largest of
// its cells' floors. Outputs per group.
void refd_solve_quartic_agglomerated(void* handle, double a, double conductance, const double* b_fine,
                                     double cg_tolerance, double newton_tolerance, std::uint64_t workers,
                                     double* floor_out, double* mean_out, double* source_out, double* stats) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    const std::vector<std::size_t>* group_map = nullptr;
    const TransportGraph& graph = agglomerated_transport_graph(mesh, group_map);
    const std::vector<std::size_t>& group_of_cell = *group_map;
    const std::size_t cells = mesh.cell_count(), groups = graph.size();
    const double radiative = 0.75 * 0.97 * stefan_boltzmann_W_m2_K4;
    Field2D<double> floor(groups, -std::numeric_limits<double>::infinity());
    for (std::size_t cell = 0; cell < cells; ++cell) {
        const double x = 100.0;
        double& f = floor[group_of_cell[cell]];
        f = std::max(f, a * x + radiative * x * x * x * x - b_fine[cell]);
    }
    std::vector<std::vector<std::size_t>> members(groups);
    for (std::size_t cell = 0; cell < cells; ++cell) members[group_of_cell[cell]].push_back(cell);
    Field2D<double> cell_source(cells, 0.0), cell_mean(cells, 0.0), cell_slope(cells, 0.0);
    const TransportResponse response = [&](const Field2D<double>& source, Field2D<double>& mean,
                                           Field2D<double>& slope) {
        for (std::size_t cell = 0; cell < cells; ++cell) cell_source[cell] = source[group_of_cell[cell]];
        quartic_response(cells, a, b_fine, cell_source, cell_mean, cell_slope);
        for (std::size_t group = 0; group < groups; ++group) {
            double air = 0.0, air_slope = 0.0;
            for (const std::size_t cell : members[group]) {
                const double area = mesh.cells()[cell].area_m2;
                air += area * cell_mean[cell];
                air_slope += area * cell_slope[cell];
            }
            mean[group] = air / graph.area_m2[group];
            slope[group] = air_slope / graph.area_m2[group];
        }
    };
    ImplicitTransportSettings settings;
    settings.cg_relative_tolerance = cg_tolerance;
    settings.newton_tolerance_W_m2 = newton_tolerance;
    const auto result = solve_implicit_transport(graph, conductance, floor, response, settings,
                                                 static_cast<std::size_t>(workers));
    std::copy(floor.values().begin(), floor.values().end(), floor_out);
    std::copy(result.mean_K.values().begin(), result.mean_K.values().end(), mean_out);
    std::copy(result.source_W_m2.values().begin(), result.source_W_m2.values().end(), source_out);
    stats[0] = result.newton_iterations;
    stats[1] = result.cg_iterations;
    stats[2] = result.consistency_residual_W_m2;
    stats[3] = result.sum_W;
    stats[4] = result.absolute_sum_W;
    stats[5] = result.dissipation_W_K;
}

// ---- non-symmetric solves (heat_transport.cpp:774-1318, incomplete_lu.cpp) --------
namespace {

const TransportGraph& graph_of(void* handle, int agglomerated, TransportGraph& own) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    if (agglomerated != 0) {
        const std::vector<std::size_t>* groups = nullptr;
        return agglomerated_transport_graph(mesh, groups);
    }
    own = mesh_transport_graph(mesh);
    return own;
}

AdvectionDiffusion transport_of(const TransportGraph& graph, std::uint64_t layers, const double* conductance,
                                const double* outflow, const double* latent, double heat_capacity) {
    AdvectionDiffusion t;
    t.layers = layers;
    t.conductance_W_K.assign(conductance, conductance + graph.neighbour.size());
    t.outflow_kg_s.assign(outflow, outflow + layers * graph.neighbour.size());
    t.heat_capacity_J_kg_K = heat_capacity;
    if (latent != nullptr) t.eddy_latent_W_m2.assign(latent, latent + graph.size());
    return t;
}

}  // namespace

// solve_implicit_transport with the linear response mean = base + slope h on the mesh's
// agglomerated graph (heat_transport.cpp:456-539, 595-772); nodes of the coarser mesh.
void refd_solve_linear_agglomerated(void* handle, double conductance, const double* base, const double* slope,
                                    double cg_tolerance, double newton_tolerance, std::uint64_t workers,
                                    double* mean_out, double* source_out, double* stats) {
    TransportGraph own;
    const TransportGraph& graph = graph_of(handle, 1, own);
    const std::size_t n = graph.size();
    const TransportResponse response = [&](const Field2D<double>& source, Field2D<double>& mean,
                                           Field2D<double>& slope_out) {
        for (std::size_t cell = 0; cell < n; ++cell) {
            mean[cell] = base[cell] + slope[cell] * source[cell];
            slope_out[cell] = slope[cell];
        }
    };
    const Field2D<double> floor(n, -std::numeric_limits<double>::infinity());
    ImplicitTransportSettings settings;
    settings.cg_relative_tolerance = cg_tolerance;
    settings.newton_tolerance_W_m2 = newton_tolerance;
    const auto result = solve_implicit_transport(graph, conductance, floor, response, settings,
                                                 static_cast<std::size_t>(workers));
    std::copy(result.mean_K.values().begin(), result.mean_K.values().end(), mean_out);
    std::copy(result.source_W_m2.values().begin(), result.source_W_m2.values().end(), source_out);
    stats[0] = result.newton_iterations;
    stats[1] = result.cg_iterations;
    stats[2] = result.consistency_residual_W_m2;
}

// IncompleteLU with blocks, then solve(x) in place.
void refd_incomplete_lu(std::uint64_t rows, const std::uint64_t* offset, const std::uint64_t* neighbour,
                        const double* diagonal, const double* off, const std::uint64_t* block_start,
                        std::uint64_t blocks, double scale, double* x) {
    std::vector<std::size_t> o(offset, offset + rows + 1), nb(neighbour, neighbour + offset[rows]),
        bs(block_start, block_start + blocks + 1);
    const IncompleteLU lu(o, nb, std::vector<double>(diagonal, diagonal + rows),
                          std::vector<double>(off, off + offset[rows]), bs, scale, 1U);
    std::vector<double> v(x, x + rows);
    lu.solve(v);
    std::copy(v.begin(), v.end(), x);
}

void refd_advection_source(void* handle, int agglomerated, std::uint64_t layers, const double* conductance,
                           const double* outflow, const double* latent, double heat_capacity, const double* mean,
                           const double* energy, double* eddy_out, double* advective_out) {
    TransportGraph own;
    const TransportGraph& graph = graph_of(handle, agglomerated, own);
    const auto t = transport_of(graph, layers, conductance, outflow, latent, heat_capacity);
    Field2D<double> m(copy_in(mean, graph.size())), eddy, advective;
    advection_diffusion_source(graph, t, m, copy_in(energy, layers * graph.size()), eddy, advective);
    std::copy(eddy.values().begin(), eddy.values().end(), eddy_out);
    std::copy(advective.values().begin(), advective.values().end(), advective_out);
}

// solve_implicit_tracer; stats: iterations, relative residual, clipped, column divergence.
void refd_tracer(void* handle, int agglomerated, std::uint64_t layers, const double* conductance,
                 const double* outflow, double heat_capacity, const double* mass, const double* tracer, double dt,
                 double tolerance, std::uint64_t workers, double* tracer_out, double* stats) {
    TransportGraph own;
    const TransportGraph& graph = graph_of(handle, agglomerated, own);
    const auto t = transport_of(graph, layers, conductance, outflow, nullptr, heat_capacity);
    const auto r = solve_implicit_tracer(graph, t, std::span<const double>(mass, graph.size()),
                                         copy_in(tracer, layers * graph.size()), dt, tolerance, 2'000,
                                         static_cast<std::size_t>(workers));
    std::copy(r.tracer.begin(), r.tracer.end(), tracer_out);
    stats[0] = r.iterations;
    stats[1] = r.relative_residual;
    stats[2] = r.clipped_kg;
    stats[3] = r.column_divergence_kg_s;
}

// solve_implicit_advection_diffusion with the column of test_advection_diffusion.cpp:
// a x + r x^4 = b + h (solve_column_surface), s_l = c_p x (1 + eps_l) + phi_l. Stats:
// newton, linear iterations, consistency, sum, absolute, eddy absolute, advective absolute.
void refd_advection_solve(void* handle, int agglomerated, std::uint64_t layers, const double* conductance,
                          const double* outflow, const double* latent, double heat_capacity, double a,
                          const double* b, const double* epsilon, const double* geopotential, const double* floor,
                          double cg_tolerance, double newton_tolerance, std::uint64_t workers, double* source_out,
                          double* mean_out, double* energy_out, double* stats) {
    TransportGraph own;
    const TransportGraph& graph = graph_of(handle, agglomerated, own);
    const auto t = transport_of(graph, layers, conductance, outflow, latent, heat_capacity);
    const std::size_t nodes = graph.size();
    const double radiative = 0.75 * 0.97 * stefan_boltzmann_W_m2_K4;
    const AdvectionResponse column = [&](const Field2D<double>& source, Field2D<double>& mean,
                                         Field2D<double>& slope, std::vector<double>& energy,
                                         std::vector<double>& energy_slope) {
        mean = Field2D<double>(nodes, 0.0);
        slope = Field2D<double>(nodes, 0.0);
        energy.assign(layers * nodes, 0.0);
        energy_slope.assign(layers * nodes, 0.0);
        for (std::size_t i = 0; i < nodes; ++i) {
            ColumnSystem system;
            system.a = a;
            system.b = b[i] + source[i];
            system.radiative = radiative;
            const double x = solve_column_surface(system);
            mean[i] = x;
            slope[i] = system.slope_K_m2_W(x);
            for (std::size_t l = 0; l < layers; ++l) {
                energy[l * nodes + i] = heat_capacity * x * (1.0 + epsilon[l]) + geopotential[l];
                energy_slope[l * nodes + i] = heat_capacity * slope[i] * (1.0 + epsilon[l]);
            }
        }
    };
    ImplicitTransportSettings settings;
    settings.cg_relative_tolerance = cg_tolerance;
    settings.newton_tolerance_W_m2 = newton_tolerance;
    const auto r = solve_implicit_advection_diffusion(graph, t, Field2D<double>(copy_in(floor, nodes)), column,
                                                      settings, static_cast<std::size_t>(workers));
    std::copy(r.source_W_m2.values().begin(), r.source_W_m2.values().end(), source_out);
    std::copy(r.mean_K.values().begin(), r.mean_K.values().end(), mean_out);
    std::copy(r.energy_J_kg.begin(), r.energy_J_kg.end(), energy_out);
    stats[0] = r.newton_iterations;
    stats[1] = r.linear_iterations;
    stats[2] = r.consistency_residual_W_m2;
    stats[3] = r.sum_W;
    stats[4] = r.absolute_sum_W;
    stats[5] = r.eddy_absolute_sum_W;
    stats[6] = r.advective_absolute_sum_W;
}

// ---- the assembled SPD system by the reference's own PCG + SGS V-cycle ------
// solve_newton_system (heat_transport.cpp:337-429): (A/s) x + K L x = rhs.
int refd_pcg(void* handle, double conductance, const double* slope, const double* rhs,
             double relative_tolerance, int max_iterations, std::uint64_t workers, double* x_out) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    const auto graph = mesh_transport_graph(mesh);
    const std::size_t n = mesh.cell_count();
    std::vector<Level> levels = build_hierarchy(graph, n);
    Field2D<double> s(copy_in(slope, n));
    Field2D<double> b(copy_in(rhs, n));
    Field2D<double> x;
    ImplicitTransportSettings settings;
    settings.cg_relative_tolerance = relative_tolerance;
    settings.max_cg_iterations = max_iterations;
    const int iterations = solve_newton_system(graph, conductance, s, b, levels, x, settings,
                                               static_cast<std::size_t>(workers));
    std::copy(x.values().begin(), x.values().end(), x_out);
    return iterations;
}

// The same solve with the graph and hierarchy built before the clock starts: seconds of
// solve_newton_system alone (matrix values, Galerkin coarsening, coarse factor and PCG).
double refd_pcg_seconds(void* handle, double conductance, const double* slope, const double* rhs,
                        double relative_tolerance, int max_iterations, std::uint64_t workers, double* x_out,
                        int* iterations) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    const auto graph = mesh_transport_graph(mesh);
    const std::size_t n = mesh.cell_count();
    std::vector<Level> levels = build_hierarchy(graph, n);
    Field2D<double> s(copy_in(slope, n));
    Field2D<double> b(copy_in(rhs, n));
    Field2D<double> x;
    ImplicitTransportSettings settings;
    settings.cg_relative_tolerance = relative_tolerance;
    settings.max_cg_iterations = max_iterations;
    const auto start = std::chrono::steady_clock::now();
    *iterations = solve_newton_system(graph, conductance, s, b, levels, x, settings, static_cast<std::size_t>(workers));
    const double seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    std::copy(x.values().begin(), x.values().end(), x_out);
    return seconds;
}

// ---- column radiation (atmosphere_column.hpp:85-143, 599-634) ---------------
// One column of `layers` <= 8 equal-mass layers. Inputs: layer temperature,
// humidity, cloud water (kg/kg); surface T and pressure; gravity; optical
// constants [tau_d, kappa_v, W_c, r_e, g, kappa_l]. Outputs per layer:
// emissivity (with clouds), absorbed longwave, cloud fraction, reflectance;
// scalars: [downward surface LW, OLR, SW transmission, column fraction,
// column optical depth].
int refd_column_radiation(std::uint32_t layers, const double* temperature, const double* humidity,
                          const double* cloud_water, double surface_temperature,
                          double surface_pressure, double gravity, const double* constants,
                          double* emissivity, double* absorbed, double* fraction,
                          double* reflectance, double* scalars) {
    if (layers == 0U || layers > max_column_layers) {
        return -1;
    }
    AtmosphereParameters parameters;
    parameters.layer_count = layers;
    parameters.dry_optical_depth = constants[0];
    parameters.vapour_absorption_m2_kg = constants[1];
    parameters.cloud_in_cloud_water_path_kg_m2 = constants[2];
    parameters.cloud_effective_radius_m = constants[3];
    parameters.cloud_asymmetry = constants[4];
    parameters.cloud_longwave_absorption_m2_kg = constants[5];
    ColumnRadiation column = column_radiation(parameters, surface_pressure, gravity,
                                              std::span<const double>(humidity, layers));
    ColumnMoisture moisture;
    moisture.layer_mass_kg_m2 = surface_pressure / (gravity * static_cast<double>(layers));
    for (std::size_t k = 0; k < layers; ++k) {
        moisture.humidity_kg_kg[k] = humidity[k];
        moisture.cloud_water_kg_kg[k] = cloud_water[k];
        moisture.pressure_Pa[k] = layer_sigma(k, layers) * surface_pressure;
    }
    const CloudOptics optics = cloud_optics(parameters, column, moisture);
    add_cloud_longwave(column, optics);
    LayerArray emission{};
    for (std::size_t k = 0; k < layers; ++k) {
        const double t2 = temperature[k] * temperature[k];
        emission[k] = column.emissivity[k] * column_stefan_boltzmann_W_m2_K4 * t2 * t2;
    }
    const double ts2 = surface_temperature * surface_temperature;
    const LongwaveFluxes fluxes =
        longwave_fluxes(column, emission, column_stefan_boltzmann_W_m2_K4 * ts2 * ts2);
    for (std::size_t k = 0; k < layers; ++k) {
        emissivity[k] = column.emissivity[k];
        absorbed[k] = fluxes.absorbed_in[k];
        fraction[k] = optics.fraction[k];
        reflectance[k] = optics.reflectance[k];
    }
    scalars[0] = fluxes.downward_surface_W_m2;
    scalars[1] = fluxes.outgoing_W_m2;
    scalars[2] = optics.transmission;
    scalars[3] = optics.column_fraction;
    scalars[4] = optics.column_optical_depth;
    return 0;
}

double refd_layer_sigma(std::uint64_t layer, std::uint64_t layers) {
    return layer_sigma(layer, layers);
}

double refd_saturation_specific_humidity(double temperature, double pressure) {
    return saturation_specific_humidity(temperature, pressure);
}

double refd_surface_gravity_earth() {
    return surface_gravity_m_s2(PlanetParameters::earth_development());
}

// Earth-like optical constants (atmosphere.hpp:79-82,120-121).
void refd_earth_like_constants(double* constants) {
    AtmosphereParameters p;
    constants[0] = earth_like_dry_optical_depth;
    constants[1] = earth_like_vapour_absorption_m2_kg;
    constants[2] = p.cloud_in_cloud_water_path_kg_m2;
    constants[3] = p.cloud_effective_radius_m;
    constants[4] = p.cloud_asymmetry;
    constants[5] = p.cloud_longwave_absorption_m2_kg;
}

// ---- sub-step-mean insolation (substep_forcing.cpp:75-127) ------------------
void refd_insolation(void* handle, std::int64_t substep, float* out) {
    const auto& mesh = *static_cast<PlanetMesh*>(handle);
    const auto parameters = PlanetParameters::earth_development();
    Field2D<float> field(mesh.cell_count(), 0.0F);
    compute_substep_mean_insolation(mesh, parameters, climate_substep(substep, parameters), field,
                                    1U);
    std::copy(field.values().begin(), field.values().end(), out);
}

// The 16 quadrature nodes: [time, weight, sin decl, cos decl, flux] each.
void refd_insolation_nodes(std::int64_t substep, double* nodes) {
    const auto parameters = PlanetParameters::earth_development();
    const auto table = substep_forcing_nodes(parameters, climate_substep(substep, parameters));
    for (std::size_t i = 0; i < table.size(); ++i) {
        nodes[5 * i] = table[i].time_s;
        nodes[5 * i + 1] = table[i].weight;
        nodes[5 * i + 2] = table[i].sin_declination;
        nodes[5 * i + 3] = table[i].cos_declination;
        nodes[5 * i + 4] = table[i].incident_flux_W_m2;
    }
}

}  // extern "C"

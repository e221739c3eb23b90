// C-ABI of the GB300 heat-transport path (include/planetsim_gb300.h).
//
// Maps the reference's exception conventions onto status codes:
// std::invalid_argument -> PSGB_ERR_INVALID_ARGUMENT, std::logic_error ->
// PSGB_ERR_LOGIC, allocation failures -> PSGB_ERR_OUT_OF_MEMORY, CUDA errors ->
// PSGB_ERR_CUDA; the message is kept per thread for psgb_last_error().
#include "../../include/planetsim_gb300.h"
#include "autotune.hpp"
#include "capi_internal.hpp"

#include "column.hpp"
#include "host/insolation.hpp"
#include "operators.hpp"
#include "profile.hpp"
#include "solver.hpp"

#include <atomic>
#include <cmath>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

namespace psgb::capi {

thread_local std::string g_last_error;

int fail(int code, const std::string& message) {
    g_last_error = message;
    return code;
}

}  // namespace psgb::capi

namespace {

using psgb::capi::fail;
using psgb::capi::g_last_error;

cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

void require(bool ok, const char* message) {
    if (!ok) throw std::invalid_argument(message);
}

void require_memory(int memory) {
    require(memory == PSGB_MEMORY_HOST || memory == PSGB_MEMORY_DEVICE, "memory must be PSGB_MEMORY_HOST or PSGB_MEMORY_DEVICE");
}

std::size_t dtype_size(int dtype) {
    if (dtype == PSGB_DTYPE_F64) return 8;
    if (dtype == PSGB_DTYPE_F32) return 4;
    throw std::invalid_argument("dtype must be PSGB_DTYPE_F64 or PSGB_DTYPE_F32");
}

// The planet's device state, uploaded on first use.
const psgb::DevMesh& device_mesh(psgb_planet* h) {
    psgb::upload_planet(*h->planet);
    return h->planet->dev;
}

// Device staging buffers of max(P, edges) doubles each.
double* stage(psgb_planet* h, int index) {
    const psgb::DevMesh& d = device_mesh(h);
    const std::size_t len = std::max<std::size_t>(std::max<std::size_t>(d.p, d.edges), d.fine_cells);
    while (static_cast<int>(h->stage.size()) <= index) h->stage.push_back(h->stage_store.alloc<double>(len));
    h->stage_len = len;
    return h->stage[index];
}

psgb::Batch& solo(psgb_planet* h) {
    if (!h->planet->solo) h->planet->solo = psgb::make_batch({h->planet.get()});
    return *h->planet->solo;
}

// Copy `count` elements in (host or device source) to a device destination.
void copy_in(void* dst, const void* src, std::size_t bytes, int memory, cudaStream_t st) {
    PSGB_CUDA(cudaMemcpyAsync(dst, src, bytes, memory == PSGB_MEMORY_HOST ? cudaMemcpyHostToDevice
                                                                        : cudaMemcpyDeviceToDevice, st));
}
void copy_out(void* dst, const void* src, std::size_t bytes, int memory, cudaStream_t st) {
    PSGB_CUDA(cudaMemcpyAsync(dst, src, bytes, memory == PSGB_MEMORY_HOST ? cudaMemcpyDeviceToHost
                                                                        : cudaMemcpyDeviceToDevice, st));
}

}  // namespace

namespace psgb::capi {

psgb::SolveOptions to_options(const psgb_solve_options* o) {
    psgb_solve_options d;
    psgb_solve_options_default(&d);
    if (o == nullptr) o = &d;
    psgb::SolveOptions s;
    require(o->precision == PSGB_PRECISION_FP64 || o->precision == PSGB_PRECISION_MIXED, "unknown precision");
    require(o->method == PSGB_METHOD_PCG || o->method == PSGB_METHOD_BICGSTAB, "unknown Krylov method");
    require(o->tolerance > 0.0 && std::isfinite(o->tolerance), "tolerance must be positive");
    require(o->inner_tolerance > 0.0 && o->inner_tolerance < 1.0, "inner tolerance must be in (0, 1)");
    require(o->max_iterations > 0 && o->max_refinements > 0 && o->poll > 0, "iteration limits must be positive");
    require(o->pre_sweeps >= 1 && o->post_sweeps >= 0 && o->pre_sweeps <= 8 && o->post_sweeps <= 8,
            "Jacobi sweeps must be 1..8 (pre) and 0..8 (post)");
    require(o->jacobi_omega > 0.0 && o->jacobi_omega < 2.0, "Jacobi damping must be in (0, 2)");
    require(o->schedule == PSGB_SCHEDULE_AUTO || o->schedule == PSGB_SCHEDULE_KERNELS ||
                o->schedule == PSGB_SCHEDULE_PERSISTENT, "unknown schedule");
    s.precision = o->precision;
    s.method = o->method;
    s.tolerance = o->tolerance;
    s.inner_tolerance = o->inner_tolerance;
    s.max_iterations = o->max_iterations;
    s.max_refinements = o->max_refinements;
    s.poll = o->poll;
    s.schedule = o->schedule;
    return s;
}

void apply_smoother(psgb::Batch& b, const psgb_solve_options* o) {
    psgb_solve_options d;
    psgb_solve_options_default(&d);
    if (o == nullptr) o = &d;
    if (b.tuned) return;   // per-level settings from an autotune take precedence
    b.smoother.pre = o->pre_sweeps;
    b.smoother.post = o->post_sweeps;
    b.smoother.omega = o->jacobi_omega;
}

int status_of(const psgb::InstanceScalars& s) {
    switch (s.outer_status) {
        case psgb::kConverged: return PSGB_OK;
        case psgb::kNonFinite: return PSGB_ERR_NON_FINITE;
        case psgb::kCap: return s.status == psgb::kBreakdown ? PSGB_ERR_BREAKDOWN : PSGB_ERR_NOT_CONVERGED;
        default: return PSGB_ERR_NOT_CONVERGED;
    }
}

const char* status_message(int code) {
    switch (code) {
        case PSGB_ERR_NON_FINITE: return "solve produced a non-finite residual (non-finite input?)";
        case PSGB_ERR_BREAKDOWN: return "Krylov breakdown before the tolerance was reached";
        case PSGB_ERR_NOT_CONVERGED: return "iteration or refinement cap reached before the tolerance";
        default: return "";
    }
}

void fill_report(const psgb::InstanceScalars& s, psgb_solve_report* r) {
    if (r == nullptr) return;
    r->status = status_of(s);
    r->refinements = s.refinements;
    r->iterations = s.inner_total;
    r->relative_residual = s.outer_b_norm > 0.0 ? s.outer_r_norm / s.outer_b_norm : 0.0;
}

// Per-entry conductance in the batch's fine ELL layout from per-undirected-edge values.
void scatter_edge_conductance(const psgb::Planet& p, const double* per_edge, std::int64_t base,
                              std::size_t P0, std::vector<double>& out) {
    const psgb::HostMesh& m = p.mesh;
    for (std::size_t c = 0; c < m.cells; ++c) {
        for (std::uint32_t k = 0; k < m.edge_count[c]; ++k) {
            const double g = per_edge[m.nb_edge[m.edge_offset[c] + k]];
            if (!(g >= 0.0) || !std::isfinite(g)) throw std::invalid_argument("edge conductance must be finite and non-negative");
            out[k * P0 + base + c] = g;
        }
    }
}

// Assemble (A/s + K L) on every planet of the batch unless the parameters equal the
// ones the current matrix was built from.
void assemble_step_matrix(psgb::Batch& b, const psgb_step_params* params, cudaStream_t st) {
    const std::uint32_t I = b.instances;
    if (b.assembled_edges.size() != I) b.assembled_edges.assign(I, {});
    if (b.stored_edges.size() != I) {
        b.stored_edges.assign(I, {});
        b.stored_generation.assign(I, 0);
    }
    // The matrix depends on C, dt, K and the per-edge conductances: scalars and the
    // conductance source go into a key; arrays passed in are compared with the ones the
    // current matrix was built from (no copy unless they changed); stored arrays by
    // their generation.
    std::vector<double> key;
    std::vector<const double*> edges(I, nullptr);
    bool per_edge = false;
    for (std::uint32_t i = 0; i < I; ++i) {
        const psgb_step_params& p = params[i];
        require(p.heat_capacity_J_m2_K > 0.0 && std::isfinite(p.heat_capacity_J_m2_K), "heat capacity must be finite and positive");
        require(p.dt_s > 0.0 && std::isfinite(p.dt_s), "time step must be finite and positive");
        if (p.edge_conductance_stored) {
            require(p.edge_conductance == nullptr, "edge_conductance must be NULL when the stored conductance is used");
            require(!b.stored_edges[i].empty(), "no per-edge conductance is stored for this planet");
            edges[i] = b.stored_edges[i].data();
        } else {
            edges[i] = p.edge_conductance;
        }
        if (edges[i] == nullptr) {
            require(p.conductance_W_K > 0.0 && std::isfinite(p.conductance_W_K), "transport conductance must be finite and positive");
        }
        per_edge = per_edge || edges[i] != nullptr;
        key.push_back(p.heat_capacity_J_m2_K);
        key.push_back(p.dt_s);
        key.push_back(edges[i] == nullptr ? p.conductance_W_K : -1.0);
        key.push_back(p.edge_conductance_stored ? static_cast<double>(b.stored_generation[i]) : -1.0);
    }
    bool same = b.matrix_ready && key == b.assembled_key;
    for (std::uint32_t i = 0; same && i < I; ++i) {
        if (edges[i] == nullptr || params[i].edge_conductance_stored) continue;
        const std::size_t e = b.planets[i]->mesh.edges;
        same = b.assembled_edges[i].size() == e &&
               std::memcmp(b.assembled_edges[i].data(), edges[i], e * sizeof(double)) == 0;
    }
    if (same && b.reassemble) {
        // the parameters are staged on the device already: the device part of the
        // assembly again (fine matrix, Galerkin values, coarsest inverses)
        psgb::assemble_transport(b, b.slope_field, b.conductance, b.step_edge_conductance, st);
        psgb::prepare_levels(b, st);
        return;
    }
    if (same) return;
    const std::size_t P0 = b.levels[0].rows;
    std::vector<double> slope_of(I), conductance(I);
    for (std::uint32_t i = 0; i < I; ++i) {
        slope_of[i] = params[i].dt_s / params[i].heat_capacity_J_m2_K;
        conductance[i] = edges[i] == nullptr ? params[i].conductance_W_K : 0.0;
    }
    PSGB_CUDA(cudaMemcpyAsync(b.slope_of, slope_of.data(), I * sizeof(double), cudaMemcpyHostToDevice, st));
    PSGB_CUDA(cudaMemcpyAsync(b.conductance, conductance.data(), I * sizeof(double), cudaMemcpyHostToDevice, st));
    const double* edge_g = nullptr;
    if (per_edge) {
        if (b.edge_g == nullptr) b.edge_g = b.store.alloc<double>(6 * P0);
        std::vector<double> g(6 * P0, 0.0);
        for (std::uint32_t i = 0; i < I; ++i) {
            if (edges[i] != nullptr) {
                scatter_edge_conductance(*b.planets[i], edges[i], b.fine_base[i], P0, g);
            } else {
                const psgb::HostMesh& m = b.planets[i]->mesh;
                for (std::size_t c = 0; c < m.cells; ++c)
                    for (std::uint32_t k = 0; k < m.edge_count[c]; ++k) g[k * P0 + b.fine_base[i] + c] = params[i].conductance_W_K;
            }
        }
        PSGB_CUDA(cudaMemcpyAsync(b.edge_g, g.data(), g.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        PSGB_CUDA(cudaStreamSynchronize(st));
        edge_g = b.edge_g;
    }
    // slope field (dt/C per cell of every planet), kept for reassembly
    std::vector<double> slope(P0, 1.0);
    for (std::uint32_t i = 0; i < I; ++i) {
        const std::size_t n = b.planets[i]->mesh.cells;
        for (std::size_t c = 0; c < n; ++c) slope[b.fine_base[i] + c] = slope_of[i];
    }
    if (b.slope_field == nullptr) b.slope_field = b.store.alloc<double>(P0);
    PSGB_CUDA(cudaMemcpyAsync(b.slope_field, slope.data(), P0 * sizeof(double), cudaMemcpyHostToDevice, st));
    psgb::assemble_transport(b, b.slope_field, b.conductance, edge_g, st);
    psgb::prepare_levels(b, st);
    PSGB_CUDA(cudaStreamSynchronize(st));
    b.assembled_key = key;
    for (std::uint32_t i = 0; i < I; ++i) {
        if (edges[i] != nullptr && !params[i].edge_conductance_stored) {
            b.assembled_edges[i].assign(edges[i], edges[i] + b.planets[i]->mesh.edges);
        } else {
            b.assembled_edges[i].clear();
        }
    }
    b.step_edge_conductance = edge_g;
}

// One transport step on every planet of a batch; inputs already in b.t0 / b.src.
void run_step(psgb::Batch& b, const psgb::SolveOptions& opt, cudaStream_t st) {
    psgb::StepView v = step_view(b);
    psgb::launch_step_rhs(v, b.t0, b.src, b.bb, b.tmp, b.xr, st);
    psgb::solve(b, opt, b.bb, b.xr, st);
    psgb::launch_step_finish(v, b.xr, b.t0, b.src, b.hout, b.tnew, b.partial, b.sums, st);
    PSGB_CUDA(cudaGetLastError());
}

void step_reports(psgb::Batch& b, psgb_step_report* reports, cudaStream_t st) {
    std::vector<double> sums(std::size_t(b.instances) * 8);
    PSGB_CUDA(cudaMemcpyAsync(sums.data(), b.sums, sums.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    PSGB_CUDA(cudaStreamSynchronize(st));
    if (reports == nullptr) return;
    for (std::uint32_t i = 0; i < b.instances; ++i) {
        psgb_step_report& r = reports[i];
        fill_report(b.host_scalars[i], &r.solve);
        const double* s = &sums[std::size_t(i) * 8];
        r.sum_W = s[0];
        r.absolute_sum_W = s[1];
        r.dissipation_W_K = s[2];
        r.closure = s[4] > 0.0 ? std::fabs(s[5] - s[3]) / s[4] : std::fabs(s[5] - s[3]);
    }
}

}  // namespace psgb::capi

using namespace psgb::capi;

namespace {

}  // namespace


extern "C" {

const char* psgb_last_error(void) { return g_last_error.c_str(); }
int psgb_abi_version(void) { return PSGB_ABI_VERSION; }

void psgb_solve_options_default(psgb_solve_options* out) {
    if (out == nullptr) return;
    out->precision = PSGB_PRECISION_FP64;
    out->method = PSGB_METHOD_BICGSTAB;
    out->tolerance = 1e-10;
    out->inner_tolerance = 1e-4;
    out->max_iterations = 1000;
    out->max_refinements = 20;
    out->poll = 4;
    out->pre_sweeps = 2;
    out->post_sweeps = 2;
    out->jacobi_omega = 0.8;
    out->schedule = PSGB_SCHEDULE_AUTO;
}

namespace {
std::uint64_t next_planet_serial() {
    static std::atomic<std::uint64_t> serials{0};
    return ++serials;
}
}  // namespace

int psgb_planet_create(uint32_t level, double radius_m, psgb_planet** out) {
    return guarded([&] {
        require(out != nullptr, "output handle pointer is null");
        *out = nullptr;
        auto h = std::make_unique<psgb_planet>();
        h->planet = psgb::make_planet(level, radius_m);
        h->serial = next_planet_serial();
        *out = h.release();
        return PSGB_OK;
    });
}

int psgb_planet_create_agglomerated(uint32_t level, double radius_m, psgb_planet** out) {
    return guarded([&] {
        require(out != nullptr, "output handle pointer is null");
        *out = nullptr;
        auto h = std::make_unique<psgb_planet>();
        h->planet = psgb::make_planet(level, radius_m, true);
        h->serial = next_planet_serial();
        *out = h.release();
        return PSGB_OK;
    });
}

int psgb_planet_graph_view(const psgb_planet* h, psgb_graph_view* out) {
    return guarded([&] {
        require(h != nullptr && out != nullptr, "null argument");
        const psgb::TransportGraph& g = h->planet->graph;
        *out = psgb_graph_view{g.area_m2.data(), g.offset.data(), g.neighbour.data(), g.weight.data(),
                               g.weight_sum.data()};
        return PSGB_OK;
    });
}

int psgb_planet_group_of_cell(const psgb_planet* h, uint32_t* out) {
    return guarded([&] {
        require(h != nullptr && out != nullptr, "null argument");
        const auto& g = h->planet->group_of_cell;
        require(!g.empty(), "not an agglomerated planet");
        std::copy(g.begin(), g.end(), out);
        return PSGB_OK;
    });
}

void psgb_planet_destroy(psgb_planet* planet) { delete planet; }

int psgb_planet_info_get(const psgb_planet* h, psgb_planet_info* out) {
    return guarded([&] {
        require(h != nullptr && out != nullptr, "null argument");
        const psgb::Planet& p = *h->planet;
        std::memset(out, 0, sizeof(*out));
        out->cells = p.mesh.cells;
        out->edges = p.mesh.edges;
        out->directed_edges = p.mesh.directed;
        out->corners = p.mesh.corners;
        out->levels = static_cast<uint32_t>(p.hierarchy.levels.size());
        for (std::size_t l = 0; l < p.hierarchy.levels.size() && l < 8; ++l) out->level_rows[l] = p.hierarchy.levels[l].size;
        out->device_bytes = p.store.bytes() + (p.solo ? p.solo->store.bytes() : 0) + h->stage_store.bytes();
        out->fine_cells = p.group_of_cell.size();
        return PSGB_OK;
    });
}

int psgb_planet_mesh_view(const psgb_planet* h, psgb_mesh_view* out) {
    return guarded([&] {
        require(h != nullptr && out != nullptr, "null argument");
        const psgb::HostMesh& m = h->planet->mesh;
        out->center = m.center.data();
        out->east = m.east.data();
        out->north = m.north.data();
        out->area_m2 = m.area_m2.data();
        out->source_vertex = m.source_vertex.data();
        out->edge_offset = m.edge_offset.data();
        out->edge_count = m.edge_count.data();
        out->neighbor = m.nb_cell.data();
        out->edge = m.nb_edge.data();
        out->corner = m.nb_corner.data();
        out->normal_east = m.normal_east.data();
        out->normal_north = m.normal_north.data();
        out->edge_first = m.edge_first.data();
        out->edge_second = m.edge_second.data();
        out->edge_length_m = m.edge_length_m.data();
        out->edge_distance_m = m.edge_distance_m.data();
        out->corner_unit = m.corner_unit.data();
        out->graph_weight = h->planet->graph.weight.data();
        out->graph_weight_sum = h->planet->graph.weight_sum.data();
        return PSGB_OK;
    });
}

int psgb_planet_hierarchy_level(const psgb_planet* h, uint32_t level, uint64_t sizes[4],
                                const uint32_t** offset, const uint32_t** column,
                                const uint32_t** aggregate, const int64_t** target) {
    return guarded([&] {
        require(h != nullptr && sizes != nullptr, "null argument");
        const auto& levels = h->planet->hierarchy.levels;
        require(level < levels.size(), "multigrid level out of range");
        const psgb::HostLevel& l = levels[level];
        sizes[0] = l.size;
        sizes[1] = l.column.size();
        sizes[2] = l.aggregate.size();
        sizes[3] = l.target.size();
        if (offset) *offset = l.offset.data();
        if (column) *column = l.column.data();
        if (aggregate) *aggregate = l.aggregate.data();
        if (target) *target = l.target.data();
        return PSGB_OK;
    });
}

int psgb_laplacian(psgb_planet* h, int dtype, const void* scalar, void* result, int memory, void* stream) {
    return guarded([&] {
        require(h != nullptr && scalar != nullptr && result != nullptr, "null argument");
        require_memory(memory);
        const std::size_t es = dtype_size(dtype);
        const psgb::DevMesh& d = device_mesh(h);
        cudaStream_t st = as_stream(stream);
        const void* in = scalar;
        void* out = result;
        if (memory == PSGB_MEMORY_HOST) {
            double* a = stage(h, 0);
            double* b = stage(h, 1);
            copy_in(a, scalar, d.n * es, memory, st);
            in = a;
            out = b;
        }
        if (dtype == PSGB_DTYPE_F64) psgb::launch_laplacian<double>(d, static_cast<const double*>(in), static_cast<double*>(out), st);
        else psgb::launch_laplacian<float>(d, static_cast<const float*>(in), static_cast<float*>(out), st);
        PSGB_CUDA(cudaGetLastError());
        if (memory == PSGB_MEMORY_HOST) {
            copy_out(result, out, d.n * es, memory, st);
            PSGB_CUDA(cudaStreamSynchronize(st));
        }
        return PSGB_OK;
    });
}

int psgb_gradient(psgb_planet* h, int dtype, const void* scalar, void* east, void* north, int memory, void* stream) {
    return guarded([&] {
        require(h != nullptr && scalar != nullptr && east != nullptr && north != nullptr, "null argument");
        require_memory(memory);
        const std::size_t es = dtype_size(dtype);
        const psgb::DevMesh& d = device_mesh(h);
        cudaStream_t st = as_stream(stream);
        const void* in = scalar;
        void *e = east, *n = north;
        if (memory == PSGB_MEMORY_HOST) {
            double* a = stage(h, 0);
            copy_in(a, scalar, d.n * es, memory, st);
            in = a;
            e = stage(h, 1);
            n = stage(h, 2);
        }
        if (dtype == PSGB_DTYPE_F64) psgb::launch_gradient<double>(d, static_cast<const double*>(in), static_cast<double*>(e), static_cast<double*>(n), st);
        else psgb::launch_gradient<float>(d, static_cast<const float*>(in), static_cast<float*>(e), static_cast<float*>(n), st);
        PSGB_CUDA(cudaGetLastError());
        if (memory == PSGB_MEMORY_HOST) {
            copy_out(east, e, d.n * es, memory, st);
            copy_out(north, n, d.n * es, memory, st);
            PSGB_CUDA(cudaStreamSynchronize(st));
        }
        return PSGB_OK;
    });
}

int psgb_divergence(psgb_planet* h, int dtype, const void* edge_flux, void* result, int memory, void* stream) {
    return guarded([&] {
        require(h != nullptr && edge_flux != nullptr && result != nullptr, "null argument");
        require_memory(memory);
        const std::size_t es = dtype_size(dtype);
        const psgb::DevMesh& d = device_mesh(h);
        cudaStream_t st = as_stream(stream);
        const void* in = edge_flux;
        void* out = result;
        if (memory == PSGB_MEMORY_HOST) {
            double* a = stage(h, 0);
            copy_in(a, edge_flux, d.edges * es, memory, st);
            in = a;
            out = stage(h, 1);
        }
        if (dtype == PSGB_DTYPE_F64) psgb::launch_divergence<double>(d, static_cast<const double*>(in), static_cast<double*>(out), st);
        else psgb::launch_divergence<float>(d, static_cast<const float*>(in), static_cast<float*>(out), st);
        PSGB_CUDA(cudaGetLastError());
        if (memory == PSGB_MEMORY_HOST) {
            copy_out(result, out, d.n * es, memory, st);
            PSGB_CUDA(cudaStreamSynchronize(st));
        }
        return PSGB_OK;
    });
}

int psgb_diffusion_source(psgb_planet* h, double conductance_W_K, const double* temperature_K,
                          double* source_W_m2, int memory, void* stream) {
    return guarded([&] {
        require(h != nullptr && temperature_K != nullptr && source_W_m2 != nullptr, "null argument");
        require_memory(memory);
        const psgb::DevMesh& d = device_mesh(h);
        cudaStream_t st = as_stream(stream);
        const double* in = temperature_K;
        double* out = source_W_m2;
        if (memory == PSGB_MEMORY_HOST) {
            double* a = stage(h, 0);
            copy_in(a, temperature_K, d.n * 8, memory, st);
            in = a;
            out = stage(h, 1);
        }
        psgb::launch_diffusion_source(d, conductance_W_K, in, out, st);
        PSGB_CUDA(cudaGetLastError());
        if (memory == PSGB_MEMORY_HOST) {
            copy_out(source_W_m2, out, d.n * 8, memory, st);
            PSGB_CUDA(cudaStreamSynchronize(st));
        }
        return PSGB_OK;
    });
}

int psgb_group_mean(psgb_planet* h, const double* fine_a, const double* fine_b, double* node_a, double* node_b,
                    int memory, void* stream) {
    return guarded([&] {
        require(h != nullptr && fine_a != nullptr && node_a != nullptr, "null argument");
        require((fine_b == nullptr) == (node_b == nullptr), "second field: both pointers or neither");
        require(!h->planet->group_of_cell.empty(), "not an agglomerated planet");
        require_memory(memory);
        const psgb::DevMesh& d = device_mesh(h);
        cudaStream_t st = as_stream(stream);
        const double *a = fine_a, *b = fine_b;
        double *ma = node_a, *mb = node_b;
        if (memory == PSGB_MEMORY_HOST) {
            double* sa = stage(h, 0);
            copy_in(sa, fine_a, std::size_t(d.fine_cells) * 8, memory, st);
            a = sa;
            ma = stage(h, 2);
            if (fine_b != nullptr) {
                double* sb = stage(h, 1);
                copy_in(sb, fine_b, std::size_t(d.fine_cells) * 8, memory, st);
                b = sb;
                mb = stage(h, 3);
            }
        }
        psgb::launch_group_mean(d, a, b, ma, mb, st);
        PSGB_CUDA(cudaGetLastError());
        if (memory == PSGB_MEMORY_HOST) {
            copy_out(node_a, ma, std::size_t(d.n) * 8, memory, st);
            if (node_b != nullptr) copy_out(node_b, mb, std::size_t(d.n) * 8, memory, st);
            PSGB_CUDA(cudaStreamSynchronize(st));
        }
        return PSGB_OK;
    });
}

int psgb_group_scatter(psgb_planet* h, const double* node_value, double* fine_value, int memory, void* stream) {
    return guarded([&] {
        require(h != nullptr && node_value != nullptr && fine_value != nullptr, "null argument");
        require(!h->planet->group_of_cell.empty(), "not an agglomerated planet");
        require_memory(memory);
        const psgb::DevMesh& d = device_mesh(h);
        cudaStream_t st = as_stream(stream);
        const double* in = node_value;
        double* out = fine_value;
        if (memory == PSGB_MEMORY_HOST) {
            double* s = stage(h, 0);
            copy_in(s, node_value, std::size_t(d.n) * 8, memory, st);
            in = s;
            out = stage(h, 1);
        }
        psgb::launch_group_scatter(d, in, out, st);
        PSGB_CUDA(cudaGetLastError());
        if (memory == PSGB_MEMORY_HOST) {
            copy_out(fine_value, out, std::size_t(d.fine_cells) * 8, memory, st);
            PSGB_CUDA(cudaStreamSynchronize(st));
        }
        return PSGB_OK;
    });
}

int psgb_multigrid_set_matrix(psgb_planet* h, const double* diagonal, const double* off_diagonal, int memory,
                              void* stream) {
    return guarded([&] {
        require(h != nullptr && diagonal != nullptr && off_diagonal != nullptr, "null argument");
        require_memory(memory);
        psgb::Batch& b = solo(h);
        const psgb::Planet& p = *h->planet;
        cudaStream_t st = as_stream(stream);
        if (b.csr_values == nullptr) b.csr_values = b.store.alloc<double>(p.mesh.directed);
        copy_in(b.tmp2, diagonal, p.mesh.cells * 8, memory, st);
        copy_in(b.csr_values, off_diagonal, p.mesh.directed * 8, memory, st);
        psgb::set_matrix_csr(b, b.tmp2, b.csr_values, st);
        psgb::prepare_levels(b, st);
        PSGB_CUDA(cudaStreamSynchronize(st));
        b.assembled_key.clear();
        return PSGB_OK;
    });
}

int psgb_multigrid_level_values(psgb_planet* h, uint32_t level, double* diagonal, double* off_diagonal) {
    return guarded([&] {
        require(h != nullptr && diagonal != nullptr && off_diagonal != nullptr, "null argument");
        psgb::Batch& b = solo(h);
        require(b.matrix_ready, "no matrix has been set");
        const auto& levels = h->planet->hierarchy.levels;
        require(level < levels.size(), "multigrid level out of range");
        const psgb::HostLevel& hl = levels[level];
        const psgb::BatchLevel& L = b.levels[level];
        const std::size_t P = L.rows, W = L.width;
        std::vector<double> vd((W + 1) * P);
        PSGB_CUDA(cudaMemcpy(vd.data(), L.vd64, vd.size() * sizeof(double), cudaMemcpyDeviceToHost));
        for (std::uint32_t r = 0; r < hl.size; ++r) {
            diagonal[r] = vd[W * P + r];
            for (std::uint32_t k = hl.offset[r]; k < hl.offset[r + 1]; ++k) off_diagonal[k] = vd[(k - hl.offset[r]) * P + r];
        }
        return PSGB_OK;
    });
}

int psgb_multigrid_precondition(psgb_planet* h, int dtype, const void* rhs, void* solution, int memory,
                                void* stream) {
    return guarded([&] {
        require(h != nullptr && rhs != nullptr && solution != nullptr, "null argument");
        require_memory(memory);
        const std::size_t es = dtype_size(dtype);
        psgb::Batch& b = solo(h);
        require(b.matrix_ready, "precondition before set_matrix");
        const std::size_t n = h->planet->mesh.cells;
        cudaStream_t st = as_stream(stream);
        if (dtype == PSGB_DTYPE_F64) {
            copy_in(b.bb, rhs, n * es, memory, st);
            psgb::vcycle<double>(b, b.bb, b.k64[9], psgb::kGateAlways, false, st);
            PSGB_CUDA(cudaGetLastError());
            copy_out(solution, b.k64[9], n * es, memory, st);
        } else {
            copy_in(b.k32[8], rhs, n * es, memory, st);
            psgb::vcycle<float>(b, b.k32[8], b.k32[9], psgb::kGateAlways, false, st);
            PSGB_CUDA(cudaGetLastError());
            copy_out(solution, b.k32[9], n * es, memory, st);
        }
        if (memory == PSGB_MEMORY_HOST) PSGB_CUDA(cudaStreamSynchronize(st));
        return PSGB_OK;
    });
}

int psgb_solve_newton_system(psgb_planet* h, const psgb_solve_options* options, double conductance_W_K,
                             const double* slope, const double* rhs, double* x, psgb_solve_report* report,
                             int memory, void* stream) {
    return guarded([&] {
        require(h != nullptr && slope != nullptr && rhs != nullptr && x != nullptr, "null argument");
        require_memory(memory);
        require(std::isfinite(conductance_W_K) && conductance_W_K > 0.0, "transport conductance must be finite and positive");
        const psgb::SolveOptions opt = to_options(options);
        psgb::Batch& b = solo(h);
        apply_smoother(b, options);
        const std::size_t n = h->planet->mesh.cells;
        cudaStream_t st = as_stream(stream);
        copy_in(b.tmp2, slope, n * 8, memory, st);
        PSGB_CUDA(cudaMemcpyAsync(b.conductance, &conductance_W_K, sizeof(double), cudaMemcpyHostToDevice, st));
        psgb::assemble_transport(b, b.tmp2, b.conductance, nullptr, st);
        psgb::prepare_levels(b, st);
        b.assembled_key.clear();
        copy_in(b.bb, rhs, n * 8, memory, st);
        psgb::launch_mask_rhs(n, b.tmp2, b.bb, st);
        copy_in(b.xr, x, n * 8, memory, st);
        psgb::solve(b, opt, b.bb, b.xr, st);
        // held rows are decoupled identity rows with a zero right-hand side: x = 0 exactly
        psgb::launch_mask_rhs(n, b.tmp2, b.xr, st);
        copy_out(x, b.xr, n * 8, memory, st);
        PSGB_CUDA(cudaStreamSynchronize(st));
        fill_report(b.host_scalars[0], report);
        const int code = status_of(b.host_scalars[0]);
        if (code != PSGB_OK) g_last_error = status_message(code);
        return code;
    });
}

int psgb_transport_step(psgb_planet* h, const psgb_step_params* params, const psgb_solve_options* options,
                        const double* t0_K, const double* source_W_m2, double* t_new_K, double* transport_W_m2,
                        psgb_step_report* report, int memory, void* stream) {
    return guarded([&] {
        require(h != nullptr && params != nullptr && t0_K != nullptr && source_W_m2 != nullptr && t_new_K != nullptr,
                "null argument");
        require_memory(memory);
        const psgb::SolveOptions opt = to_options(options);
        psgb::Batch& b = solo(h);
        apply_smoother(b, options);
        cudaStream_t st = as_stream(stream);
        assemble_step_matrix(b, params, st);
        const std::size_t n = h->planet->mesh.cells;
        copy_in(b.t0, t0_K, n * 8, memory, st);
        copy_in(b.src, source_W_m2, n * 8, memory, st);
        run_step(b, opt, st);
        copy_out(t_new_K, b.tnew, n * 8, memory, st);
        if (transport_W_m2 != nullptr) copy_out(transport_W_m2, b.hout, n * 8, memory, st);
        psgb_step_report local;
        step_reports(b, &local, st);
        if (report != nullptr) *report = local;
        if (local.solve.status != PSGB_OK) g_last_error = status_message(local.solve.status);
        return local.solve.status;
    });
}

int psgb_transport_step_multi(psgb_planet* h, const psgb_step_params* params, const psgb_solve_options* options,
                              uint32_t count, const double* const* t0_K, const double* const* source_W_m2,
                              double* const* t_new_K, double* const* transport_W_m2, psgb_step_report* reports,
                              int memory, void* stream) {
    return guarded([&] {
        require(h != nullptr && params != nullptr && t0_K != nullptr && source_W_m2 != nullptr && t_new_K != nullptr,
                "null argument");
        require(count >= 1 && count <= static_cast<uint32_t>(psgb::mr::kRhs),
                "a block holds 1 to 32 right-hand sides");
        require_memory(memory);
        require(!params->edge_conductance_stored, "the block step takes per-edge conductances as an array");
        for (uint32_t j = 0; j < count; ++j) {
            require(t0_K[j] != nullptr && source_W_m2[j] != nullptr && t_new_K[j] != nullptr, "null array in the block");
        }
        const psgb::SolveOptions opt = to_options(options);
        require(opt.method == psgb::kBiCGSTAB, "the multi-right-hand-side block solve runs BiCGSTAB");
        psgb::Batch& b = solo(h);
        apply_smoother(b, options);
        cudaStream_t st = as_stream(stream);
        assemble_step_matrix(b, params, st);
        if (!h->multi) h->multi = std::make_unique<psgb::mr::Space>();
        psgb::mr::Space& sp = *h->multi;
        psgb::mr::prepare(b, sp, opt);
        const std::uint32_t n = static_cast<std::uint32_t>(h->planet->mesh.cells);
        const std::uint32_t P0 = b.levels[0].rows;
        // the sub-steps' T0 and S on the device: the caller's arrays, or staged host copies
        std::vector<const double*> in(2 * psgb::mr::kRhs, nullptr);
        if (memory == PSGB_MEMORY_HOST) {
            while (h->multi_stage.size() < 2 * count) h->multi_stage.push_back(sp.store.alloc<double>(P0));
            for (uint32_t j = 0; j < count; ++j) {
                copy_in(h->multi_stage[2 * j], t0_K[j], n * 8, memory, st);
                copy_in(h->multi_stage[2 * j + 1], source_W_m2[j], n * 8, memory, st);
                in[j] = h->multi_stage[2 * j];
                in[psgb::mr::kRhs + j] = h->multi_stage[2 * j + 1];
            }
        } else {
            for (uint32_t j = 0; j < count; ++j) {
                in[j] = t0_K[j];
                in[psgb::mr::kRhs + j] = source_W_m2[j];
            }
        }
        PSGB_CUDA(cudaMemcpyAsync(sp.pointers, in.data(), in.size() * sizeof(const double*), cudaMemcpyHostToDevice, st));
        psgb::mr::load(n, P0, static_cast<int>(count), sp.pointers, sp.pointers + psgb::mr::kRhs, b.area,
                       params->dt_s / params->heat_capacity_J_m2_K, sp.bb, sp.xr, st);
        psgb::mr::solve(b, sp, opt, st);
        // the flux form of every solved temperature, with the single step's kernels
        const psgb::StepView v = psgb::step_view(b);
        int worst = PSGB_OK;
        for (uint32_t j = 0; j < count; ++j) {
            psgb::mr::take(P0, static_cast<int>(j), sp.xr, b.xr, st);
            psgb::launch_step_finish(v, b.xr, in[j], in[psgb::mr::kRhs + j], b.hout, b.tnew, b.partial, b.sums, st);
            copy_out(t_new_K[j], b.tnew, n * 8, memory, st);
            if (transport_W_m2 != nullptr && transport_W_m2[j] != nullptr) {
                copy_out(transport_W_m2[j], b.hout, n * 8, memory, st);
            }
            double sums[8];
            PSGB_CUDA(cudaMemcpyAsync(sums, b.sums, sizeof(sums), cudaMemcpyDeviceToHost, st));
            PSGB_CUDA(cudaStreamSynchronize(st));
            psgb_step_report local;
            fill_report(sp.host[j], &local.solve);
            local.sum_W = sums[0];
            local.absolute_sum_W = sums[1];
            local.dissipation_W_K = sums[2];
            local.closure = sums[4] > 0.0 ? std::fabs(sums[5] - sums[3]) / sums[4] : std::fabs(sums[5] - sums[3]);
            if (reports != nullptr) reports[j] = local;
            if (local.solve.status != PSGB_OK && worst == PSGB_OK) worst = local.solve.status;
        }
        if (worst != PSGB_OK) g_last_error = status_message(worst);
        return worst;
    });
}

int psgb_batch_create(psgb_planet* const* planets, uint32_t count, psgb_batch** out) {
    return guarded([&] {
        require(planets != nullptr && out != nullptr && count > 0, "a batch needs planets");
        *out = nullptr;
        std::vector<psgb::Planet*> list;
        for (uint32_t i = 0; i < count; ++i) {
            require(planets[i] != nullptr, "null planet in batch");
            list.push_back(planets[i]->planet.get());
        }
        auto h = std::make_unique<psgb_batch>();
        h->batch = psgb::make_batch(list);
        *out = h.release();
        return PSGB_OK;
    });
}

void psgb_batch_destroy(psgb_batch* batch) { delete batch; }

uint64_t psgb_batch_device_bytes(const psgb_batch* batch) {
    return batch == nullptr ? 0 : batch->batch->store.bytes();
}

}  // extern "C"

namespace {

int batch_step(psgb_batch* h, const std::uint8_t* active, const psgb_step_params* params,
               const psgb_solve_options* options, const double* const* t0_K, const double* const* source_W_m2,
               double* const* t_new_K, double* const* transport_W_m2, psgb_step_report* reports, int memory,
               void* stream) {
    require(h != nullptr && params != nullptr && t0_K != nullptr && source_W_m2 != nullptr && t_new_K != nullptr,
            "null argument");
    require_memory(memory);
    const psgb::SolveOptions opt = to_options(options);
    psgb::Batch& b = *h->batch;
    apply_smoother(b, options);
    cudaStream_t st = as_stream(stream);
    // planets taking part: all, or the caller's mask
    std::vector<std::uint8_t> mask(b.instances, 1);
    if (active != nullptr) {
        for (std::uint32_t i = 0; i < b.instances; ++i) mask[i] = active[i] ? 1 : 0;
    }
    if (mask != b.host_active) {
        PSGB_CUDA(cudaMemcpyAsync(b.active, mask.data(), b.instances, cudaMemcpyHostToDevice, st));
        b.host_active = mask;
    }
    b.active_mask = false;
    for (auto m : mask) b.active_mask = b.active_mask || m == 0;
    assemble_step_matrix(b, params, st);
    for (std::uint32_t i = 0; i < b.instances; ++i) {
        if (!mask[i]) continue;
        const std::size_t n = b.planets[i]->mesh.cells;
        require(t0_K[i] != nullptr && source_W_m2[i] != nullptr && t_new_K[i] != nullptr, "null planet array");
        copy_in(b.t0 + b.fine_base[i], t0_K[i], n * 8, memory, st);
        copy_in(b.src + b.fine_base[i], source_W_m2[i], n * 8, memory, st);
    }
    run_step(b, opt, st);
    for (std::uint32_t i = 0; i < b.instances; ++i) {
        if (!mask[i]) continue;
        const std::size_t n = b.planets[i]->mesh.cells;
        copy_out(t_new_K[i], b.tnew + b.fine_base[i], n * 8, memory, st);
        if (transport_W_m2 != nullptr && transport_W_m2[i] != nullptr) {
            copy_out(transport_W_m2[i], b.hout + b.fine_base[i], n * 8, memory, st);
        }
    }
    std::vector<psgb_step_report> local(b.instances);
    step_reports(b, local.data(), st);
    int worst = PSGB_OK;
    for (std::uint32_t i = 0; i < b.instances; ++i) {
        if (reports != nullptr) reports[i] = local[i];
        if (mask[i] && local[i].solve.status != PSGB_OK && worst == PSGB_OK) worst = local[i].solve.status;
    }
    if (worst != PSGB_OK) g_last_error = status_message(worst);
    return worst;
}

}  // namespace

extern "C" {

int psgb_batch_transport_step(psgb_batch* h, const psgb_step_params* params, const psgb_solve_options* options,
                              const double* const* t0_K, const double* const* source_W_m2,
                              double* const* t_new_K, double* const* transport_W_m2, psgb_step_report* reports,
                              int memory, void* stream) {
    return guarded([&] {
        return batch_step(h, nullptr, params, options, t0_K, source_W_m2, t_new_K, transport_W_m2, reports, memory,
                          stream);
    });
}

int psgb_batch_transport_step_masked(psgb_batch* h, const uint8_t* active, const psgb_step_params* params,
                                     const psgb_solve_options* options, const double* const* t0_K,
                                     const double* const* source_W_m2, double* const* t_new_K,
                                     double* const* transport_W_m2, psgb_step_report* reports, int memory,
                                     void* stream) {
    return guarded([&] {
        require(active != nullptr, "null mask");
        return batch_step(h, active, params, options, t0_K, source_W_m2, t_new_K, transport_W_m2, reports, memory,
                          stream);
    });
}

namespace {

void fill_tuning(const psgb::Tuning& t, psgb_tuning* out) {
    std::memset(out, 0, sizeof(*out));
    out->levels = static_cast<std::uint32_t>(t.pre.size());
    for (std::size_t l = 0; l < t.pre.size() && l < PSGB_MAX_LEVELS; ++l) {
        out->pre_sweeps[l] = t.pre[l];
        out->post_sweeps[l] = t.post[l];
        out->stencil_tiles[l] = t.sets_stencil[l];
        out->vector_tiles[l] = t.sets_vector[l];
        out->block_sweeps[l] = l < t.inner.size() ? t.inner[l] : 1;
    }
    out->jacobi_omega = t.omega;
    out->tuned_solve_ms = t.tuned_ms;
    out->default_solve_ms = t.default_ms;
    out->trial_solves = t.trials;
    out->coarse_tail_level = t.tail_level;
    out->coarse_tail_single = t.tail_cluster != 0 ? 3 : t.tail_shared ? 2 : (t.tail_spread ? 0 : 1);
    out->coarse_tail_blocks = t.tail_blocks;
    out->coarse_tail_cluster = t.tail_cluster;
    out->coarse_correction = t.correction;
}

}  // namespace

int psgb_batch_autotune(psgb_batch* h, const psgb_step_params* params, const psgb_solve_options* options,
                        const double* const* t0_K, const double* const* source_W_m2, int memory, void* stream,
                        psgb_tuning* out) {
    return guarded([&] {
        require(h != nullptr && params != nullptr && t0_K != nullptr && source_W_m2 != nullptr, "null argument");
        require_memory(memory);
        const psgb::SolveOptions opt = to_options(options);
        psgb::Batch& b = *h->batch;
        require(b.levels.size() <= PSGB_MAX_LEVELS, "batch deeper than PSGB_MAX_LEVELS levels");
        if (!b.tuned) apply_smoother(b, options);
        cudaStream_t st = as_stream(stream);
        std::vector<std::uint8_t> all(b.instances, 1);
        if (all != b.host_active) {
            PSGB_CUDA(cudaMemcpyAsync(b.active, all.data(), b.instances, cudaMemcpyHostToDevice, st));
            b.host_active = all;
        }
        b.active_mask = false;
        assemble_step_matrix(b, params, st);
        for (std::uint32_t i = 0; i < b.instances; ++i) {
            const std::size_t n = b.planets[i]->mesh.cells;
            require(t0_K[i] != nullptr && source_W_m2[i] != nullptr, "null planet array");
            copy_in(b.t0 + b.fine_base[i], t0_K[i], n * 8, memory, st);
            copy_in(b.src + b.fine_base[i], source_W_m2[i], n * 8, memory, st);
        }
        // the trials solve exactly what a step solves: its right-hand side, from its
        // initial guess (the temperature before the step)
        psgb::launch_step_rhs(step_view(b), b.t0, b.src, b.bb, b.tmp, b.xr, st);
        const psgb::Tuning t = psgb::autotune(b, opt, b.bb, b.xr, b.tmp2, st);
        if (out != nullptr) fill_tuning(t, out);
        return PSGB_OK;
    });
}

int psgb_batch_set_reassembly(psgb_batch* h, int every_step) {
    return guarded([&] {
        require(h != nullptr, "null argument");
        h->batch->reassemble = every_step != 0;
        return PSGB_OK;
    });
}

int psgb_batch_set_priority(psgb_batch* h, int high) {
    return guarded([&] {
        require(h != nullptr, "null argument");
        psgb::Batch& b = *h->batch;
        require(b.stream != nullptr, "this batch solves on its caller's stream (no stream of its own)");
        int least = 0, greatest = 0;
        PSGB_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        cudaStream_t fresh = nullptr;
        PSGB_CUDA(cudaStreamCreateWithPriority(&fresh, cudaStreamNonBlocking, high != 0 ? greatest : least));
        PSGB_CUDA(cudaStreamSynchronize(b.stream));
        PSGB_CUDA(cudaStreamDestroy(b.stream));
        b.stream = fresh;
        return PSGB_OK;
    });
}

int psgb_batch_set_edge_conductance(psgb_batch* h, const double* const* edge_conductance) {
    return guarded([&] {
        require(h != nullptr && edge_conductance != nullptr, "null argument");
        psgb::Batch& b = *h->batch;
        if (b.stored_edges.size() != b.instances) {
            b.stored_edges.assign(b.instances, {});
            b.stored_generation.assign(b.instances, 0);
        }
        for (std::uint32_t i = 0; i < b.instances; ++i) {
            const double* e = edge_conductance[i];
            if (e == nullptr) {
                b.stored_edges[i].clear();
            } else {
                const std::size_t n = b.planets[i]->mesh.edges;
                for (std::size_t k = 0; k < n; ++k)
                    require(std::isfinite(e[k]) && e[k] >= 0.0, "edge conductances must be finite and non-negative");
                b.stored_edges[i].assign(e, e + n);
            }
            ++b.stored_generation[i];
        }
        return PSGB_OK;
    });
}

int psgb_batch_get_tuning(const psgb_batch* h, psgb_tuning* out) {
    return guarded([&] {
        require(h != nullptr && out != nullptr, "null argument");
        require(h->batch->levels.size() <= PSGB_MAX_LEVELS, "batch deeper than PSGB_MAX_LEVELS levels");
        fill_tuning(psgb::current_tuning(*h->batch), out);
        return PSGB_OK;
    });
}

namespace {

// A psgb_tuning applied to a batch (NULL: back to the options' uniform sweeps).
void set_tuning_of(psgb::Batch& b, const psgb_tuning* tuning) {
    if (tuning == nullptr) {
    psgb::clear_tuning(b);
    return;
    }
    require(tuning->levels == b.levels.size(), "tuning levels do not match the batch");
    psgb::Tuning t;
    for (std::uint32_t l = 0; l < tuning->levels; ++l) {
        t.pre.push_back(tuning->pre_sweeps[l]);
        t.post.push_back(tuning->post_sweeps[l]);
        t.sets_stencil.push_back(static_cast<std::uint8_t>(tuning->stencil_tiles[l]));
        t.sets_vector.push_back(static_cast<std::uint8_t>(tuning->vector_tiles[l]));
        t.inner.push_back(tuning->block_sweeps[l] == 0 ? 1 : tuning->block_sweeps[l]);
    }
    t.omega = tuning->jacobi_omega;
    t.correction = tuning->coarse_correction == 0.0 ? 1.0 : tuning->coarse_correction;
    t.tail_level = tuning->coarse_tail_level;
    require(tuning->coarse_tail_single >= 0 && tuning->coarse_tail_single <= 3,
            "coarse_tail_single must be 0, 1, 2 or 3");
    t.tail_spread = tuning->coarse_tail_single == 0;
    t.tail_shared = tuning->coarse_tail_single == 2;
    if (tuning->coarse_tail_single == 3) {
        const std::uint32_t c = tuning->coarse_tail_cluster;
        require(c == 2 || c == 4 || c == 8, "coarse_tail_cluster must be 2, 4 or 8 blocks");
        t.tail_cluster = c;
    }
    psgb::apply_tuning(b, t);
}

}  // namespace

int psgb_batch_set_tuning(psgb_batch* h, const psgb_tuning* tuning) {
    return guarded([&] {
        require(h != nullptr, "null argument");
        set_tuning_of(*h->batch, tuning);
        return PSGB_OK;
    });
}

int psgb_planet_set_tuning(psgb_planet* h, const psgb_tuning* tuning) {
    return guarded([&] {
        require(h != nullptr, "null argument");
        set_tuning_of(solo(h), tuning);
        return PSGB_OK;
    });
}

int psgb_planet_get_tuning(psgb_planet* h, psgb_tuning* out) {
    return guarded([&] {
        require(h != nullptr && out != nullptr, "null argument");
        psgb::Batch& b = solo(h);
        require(b.levels.size() <= PSGB_MAX_LEVELS, "planet deeper than PSGB_MAX_LEVELS levels");
        fill_tuning(psgb::current_tuning(b), out);
        return PSGB_OK;
    });
}

int psgb_column_radiation(uint32_t cells, uint32_t layers, const psgb_column_constants* constants,
                          const double* temperature_K, const double* humidity, const double* cloud_water,
                          const double* surface_temperature_K, const double* surface_pressure_Pa,
                          double* emissivity, double* absorbed, double* fraction, double* reflectance,
                          double* scalars, int memory, void* stream) {
    return guarded([&] {
        require(constants != nullptr && temperature_K != nullptr && humidity != nullptr && cloud_water != nullptr &&
                    surface_temperature_K != nullptr && surface_pressure_Pa != nullptr && emissivity != nullptr &&
                    absorbed != nullptr && fraction != nullptr && reflectance != nullptr && scalars != nullptr,
                "null argument");
        require(layers >= 1 && layers <= 16, "column radiation supports 1 to 16 layers");
        require_memory(memory);
        const psgb::ColumnConstants k{constants->dry_optical_depth, constants->vapour_absorption_m2_kg,
                                      constants->in_cloud_water_path_kg_m2, constants->effective_radius_m,
                                      constants->cloud_asymmetry, constants->cloud_longwave_absorption_m2_kg,
                                      constants->reference_pressure_Pa, constants->gravity_m_s2,
                                      constants->stefan_boltzmann};
        require(k.gravity > 0.0 && k.reference_pressure > 0.0 && k.in_cloud_water_path > 0.0 && k.effective_radius > 0.0,
                "column constants must be positive");
        if (cells == 0) return PSGB_OK;
        cudaStream_t st = as_stream(stream);
        if (memory == PSGB_MEMORY_DEVICE) {
            psgb::launch_column_radiation(cells, layers, k, temperature_K, humidity, cloud_water, surface_temperature_K,
                                          surface_pressure_Pa, emissivity, absorbed, fraction, reflectance, scalars, st);
            PSGB_CUDA(cudaGetLastError());
            return PSGB_OK;
        }
        const std::size_t lc = std::size_t(layers) * cells;
        psgb::DeviceStore tmp;
        double* d_t = tmp.alloc<double>(lc);
        double* d_q = tmp.alloc<double>(lc);
        double* d_l = tmp.alloc<double>(lc);
        double* d_ts = tmp.alloc<double>(cells);
        double* d_ps = tmp.alloc<double>(cells);
        double* d_e = tmp.alloc<double>(lc);
        double* d_a = tmp.alloc<double>(lc);
        double* d_f = tmp.alloc<double>(lc);
        double* d_r = tmp.alloc<double>(lc);
        double* d_s = tmp.alloc<double>(std::size_t(5) * cells);
        copy_in(d_t, temperature_K, lc * 8, memory, st);
        copy_in(d_q, humidity, lc * 8, memory, st);
        copy_in(d_l, cloud_water, lc * 8, memory, st);
        copy_in(d_ts, surface_temperature_K, cells * 8, memory, st);
        copy_in(d_ps, surface_pressure_Pa, cells * 8, memory, st);
        psgb::launch_column_radiation(cells, layers, k, d_t, d_q, d_l, d_ts, d_ps, d_e, d_a, d_f, d_r, d_s, st);
        PSGB_CUDA(cudaGetLastError());
        copy_out(emissivity, d_e, lc * 8, memory, st);
        copy_out(absorbed, d_a, lc * 8, memory, st);
        copy_out(fraction, d_f, lc * 8, memory, st);
        copy_out(reflectance, d_r, lc * 8, memory, st);
        copy_out(scalars, d_s, std::size_t(5) * cells * 8, memory, st);
        PSGB_CUDA(cudaStreamSynchronize(st));
        return PSGB_OK;
    });
}

uint64_t psgb_launch_count(void) { return psgb::launches_total(); }

int psgb_profile_begin(const char* family) {
    return guarded([&] {
        const int f = psgb::family_of(family);
        require(f >= 0, "unknown kernel family");
        PSGB_CUDA(cudaDeviceSynchronize());
        if (!psgb::profile_begin(f)) throw std::runtime_error("could not start the profile");
        return PSGB_OK;
    });
}

int psgb_profile_end(double* total_ms, uint64_t* launches, uint64_t* swept_bytes) {
    return guarded([&] {
        require(total_ms != nullptr && launches != nullptr && swept_bytes != nullptr, "null argument");
        PSGB_CUDA(cudaDeviceSynchronize());
        std::uint64_t n = 0;
        if (!psgb::profile_end(total_ms, &n)) throw std::logic_error("no profile is active");
        *launches = n;
        *swept_bytes = psgb::profile_bytes_exchange();
        return PSGB_OK;
    });
}

int psgb_substep_mean_insolation_gpu(psgb_planet* h, int64_t substep, float* out, int memory, void* stream) {
    return guarded([&] {
        require(h != nullptr && out != nullptr, "null argument");
        require_memory(memory);
        const psgb::DevMesh& d = device_mesh(h);
        cudaStream_t st = as_stream(stream);
        const psgb::InsolationNodes nodes = psgb::substep_forcing_nodes(substep);
        float* o = memory == PSGB_MEMORY_DEVICE ? out : reinterpret_cast<float*>(stage(h, 0));
        psgb::launch_substep_insolation(d, nodes, o, st);
        PSGB_CUDA(cudaGetLastError());
        if (memory == PSGB_MEMORY_HOST) {
            PSGB_CUDA(cudaMemcpyAsync(out, o, std::size_t(d.n) * sizeof(float), cudaMemcpyDeviceToHost, st));
            PSGB_CUDA(cudaStreamSynchronize(st));
        }
        return PSGB_OK;
    });
}

int psgb_substep_mean_insolation(const psgb_planet* h, int64_t substep, float* out) {
    return guarded([&] {
        require(h != nullptr && out != nullptr, "null argument");
        psgb::substep_mean_insolation(h->planet->mesh, substep, out);
        return PSGB_OK;
    });
}

}  // extern "C"

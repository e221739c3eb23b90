/*
 * planetsim_gb300.h - C ABI of the GB300 (sm_103a) implicit heat-transport path of
 * PlanetSim (fgianni/planet_game).
 *
 * Every entry point is plain C: opaque handles, plain pointers and sizes, an int
 * status (PSGB_OK = 0) and a thread-local message from psgb_last_error(). Array
 * arguments are HOST pointers when `memory` is PSGB_MEMORY_HOST (the call copies,
 * runs and synchronises) or DEVICE pointers when it is PSGB_MEMORY_DEVICE (the call
 * is ordered on `stream`, a cudaStream_t or NULL for the legacy default stream).
 * Cell arrays are in the reference's cell order (the order make_icosphere
 * produces); edge arrays in its edge-id order; CSR arrays in its
 * TransportGraph order.
 *
 * Each entry point names the reference interface it replaces; the C++ shim that
 * re-exports those interfaces with their original signatures is described with the
 * library's integration notes.
 *
 * Threads: different planets and different batches may be used from different host
 * threads at once (each owns its device memory and private stream); calls on one planet,
 * or on one batch, must not overlap.
 *
 * ABI version 2: psgb_planet_info and psgb_tuning grew fields (fine_cells; the coarse
 * tail's spread and block count). Version 3: the serving loop (psgb_server_*) and
 * PSGB_ERR_TIMEOUT. Version 4: the block step of one planet (psgb_transport_step_multi),
 * per-step reassembly (psgb_batch_set_reassembly), coarse_tail_single = 2 (the
 * shared-memory coarse tail). Version 5: coarse_tail_single = 3 and psgb_tuning's
 * coarse_tail_cluster (the coarse tail on a thread-block cluster per planet). Version 6:
 * psgb_tuning's coarse_correction (the V-cycle's coarse-grid correction scale). Version 7:
 * psgb_planet_set_tuning / psgb_planet_get_tuning; block-local sweeps in the block step.
 * Version 8: psgb_batch_set_priority.
 *
 * A server's calls may come from any thread; its lanes step on threads of their own.
 */
#ifndef PLANETSIM_GB300_H
#define PLANETSIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PSGB_ABI_VERSION 8

/* status codes */
#define PSGB_OK 0
#define PSGB_ERR_INVALID_ARGUMENT 1 /* std::invalid_argument in the reference */
#define PSGB_ERR_OUT_OF_MEMORY 2
#define PSGB_ERR_NOT_CONVERGED 3    /* iteration or refinement cap reached */
#define PSGB_ERR_BREAKDOWN 4        /* Krylov breakdown (rho, omega or shadow.v = 0) */
#define PSGB_ERR_NON_FINITE 5
#define PSGB_ERR_CUDA 6
#define PSGB_ERR_LOGIC 7            /* std::logic_error in the reference */
#define PSGB_ERR_BUDGET 8           /* admission refused by the HBM budget */
#define PSGB_ERR_TIMEOUT 9          /* a wait ran out before the request finished */

#define PSGB_MEMORY_HOST 0
#define PSGB_MEMORY_DEVICE 1

#define PSGB_DTYPE_F64 0
#define PSGB_DTYPE_F32 1

#define PSGB_PRECISION_FP64 0       /* plain FP64 Krylov + multigrid */
#define PSGB_PRECISION_MIXED 1      /* FP32 inner Krylov + multigrid, FP64 refinement */

#define PSGB_METHOD_PCG 0
#define PSGB_METHOD_BICGSTAB 1

/* How a solve is scheduled on the GPU. */
#define PSGB_SCHEDULE_AUTO 0        /* the library's choice: currently the kernel schedule (faster on GB300) */
#define PSGB_SCHEDULE_KERNELS 1     /* one kernel per phase; Krylov chunks replayed as CUDA graphs */
#define PSGB_SCHEDULE_PERSISTENT 2  /* one cooperative kernel per solve (grid barriers between phases) */

typedef struct psgb_planet psgb_planet;
typedef struct psgb_batch psgb_batch;

/* Last error message of the calling thread ("" if none). */
const char* psgb_last_error(void);
int psgb_abi_version(void);

/* ---- mesh, transport graph and multigrid hierarchy ------------------------------
 * Replaces make_icosphere (sim/planet/mesh/icosphere.cpp:200) +
 * mesh_transport_graph (sim/planet/surface/heat_transport.cpp:433) + the
 * GraphMultigrid constructor (heat_transport.hpp:62, heat_transport.cpp:549-552).
 * The mesh is bit-identical to the reference's; the hierarchy's aggregates, coarse
 * patterns and Galerkin targets equal the reference's build_hierarchy. */
int psgb_planet_create(uint32_t level, double radius_m, psgb_planet** out);
void psgb_planet_destroy(psgb_planet* planet);

typedef struct psgb_planet_info {
    uint64_t cells, edges, directed_edges, corners;
    uint32_t levels;             /* multigrid levels (the last one is solved densely) */
    uint32_t level_rows[8];      /* rows per multigrid level */
    uint64_t device_bytes;       /* HBM held by the planet (mesh + its solo batch) */
    uint64_t fine_cells;         /* agglomerated planets: cells of the fine mesh; 0 otherwise */
} psgb_planet_info;
int psgb_planet_info_get(const psgb_planet* planet, psgb_planet_info* out);

/* Host views of the mesh arrays (valid while the planet lives); layout as the
 * reference PlanetMesh (sim/planet/mesh/planet_mesh.hpp:44-125). */
typedef struct psgb_mesh_view {
    const double* center;        /* [cells][3] */
    const double* east;          /* [cells][3] */
    const double* north;         /* [cells][3] */
    const double* area_m2;       /* [cells] */
    const uint32_t* source_vertex;
    const uint32_t* edge_offset; /* [cells] first directed edge */
    const uint8_t* edge_count;   /* [cells] 5 or 6 */
    const uint32_t* neighbor;    /* [directed] */
    const uint32_t* edge;        /* [directed] */
    const uint32_t* corner;      /* [directed] first corner of each directed edge */
    const float* normal_east;    /* [directed] */
    const float* normal_north;   /* [directed] */
    const uint32_t* edge_first;  /* [edges] */
    const uint32_t* edge_second; /* [edges] */
    const double* edge_length_m; /* [edges] */
    const double* edge_distance_m;
    const double* corner_unit;   /* [corners][3] */
    const double* graph_weight;  /* [directed] l/d, the TransportGraph weight */
    const double* graph_weight_sum; /* [cells] */
} psgb_mesh_view;
int psgb_planet_mesh_view(const psgb_planet* planet, psgb_mesh_view* out);

/* The transport one mesh level coarser, as the reference's production path runs it:
 * agglomerated_transport_graph / agglomerated_mesh (heat_transport.cpp:456-543). The
 * planet's nodes are the cells of the level-1 mesh (its mesh view), each taking the
 * summed areas of the fine cells nearest to it; every transport entry point
 * (diffusion source, set_matrix, solves, steps, batches) then works on that graph.
 * Level 0: the mesh itself. */
int psgb_planet_create_agglomerated(uint32_t level, double radius_m, psgb_planet** out);
/* Host views of the transport graph (valid while the planet lives): node areas, CSR
 * offsets [nodes + 1], neighbours, weights l/d and their sums per node. */
typedef struct psgb_graph_view {
    const double* area_m2;
    const uint32_t* offset;
    const uint32_t* neighbour;
    const double* weight;
    const double* weight_sum;
} psgb_graph_view;
int psgb_planet_graph_view(const psgb_planet* planet, psgb_graph_view* out);
/* Agglomerated planets: the node of every fine cell ([fine_cells], HOST). */
int psgb_planet_group_of_cell(const psgb_planet* planet, uint32_t* out);
/* Agglomerated planets, the production response's two sides (surface_energy.cpp:
 * 1285-1296 and 1583/1595): the nodes' area-weighted means of fine-cell fields
 * (sum over each node's fine cells in cell order of A_cell v_cell, over the node's
 * area; bit-identical to that loop), for one field or two (fine_b and node_b both
 * NULL or both set); and every fine cell taking its node's value. */
int psgb_group_mean(psgb_planet* planet, const double* fine_a, const double* fine_b, double* node_a,
                    double* node_b, int memory, void* stream);
int psgb_group_scatter(psgb_planet* planet, const double* node_value, double* fine_value, int memory,
                       void* stream);

/* Integer structure of one multigrid level (heat_transport.cpp:54-66): CSR
 * offsets [rows + 1] and columns, aggregate of each row ([rows], none on the
 * coarsest level) and the Galerkin target of each off-diagonal (-1: the aggregate's
 * diagonal). Host pointers, valid while the planet lives; sizes in `sizes`:
 * {rows, off-diagonals, aggregate length, target length}. */
int psgb_planet_hierarchy_level(const psgb_planet* planet, uint32_t level, uint64_t sizes[4],
                                const uint32_t** offset, const uint32_t** column,
                                const uint32_t** aggregate, const int64_t** target);

/* ---- finite-volume operators: sim/planet/operators/finite_volume.hpp:21-44 ----- */
/* laplacian<T>(mesh, scalar, result): cells -> cells */
int psgb_laplacian(psgb_planet* planet, int dtype, const void* scalar, void* result, int memory,
                   void* stream);
/* gradient<T>(mesh, scalar, east, north): cells -> 2 x cells */
int psgb_gradient(psgb_planet* planet, int dtype, const void* scalar, void* east, void* north,
                  int memory, void* stream);
/* divergence<T>(mesh, edge_normal_flux, result): edges -> cells */
int psgb_divergence(psgb_planet* planet, int dtype, const void* edge_flux, void* result, int memory,
                    void* stream);

/* ---- heat transport: sim/planet/surface/heat_transport.hpp -------------------- */
/* diffusion_source (heat_transport.hpp:122): K * laplacian, W/m^2 */
int psgb_diffusion_source(psgb_planet* planet, double conductance_W_K, const double* temperature_K,
                          double* source_W_m2, int memory, void* stream);

/* GraphMultigrid::set_matrix (heat_transport.hpp:69): diagonal [cells], off-diagonals
 * in the graph's CSR order [directed]. */
int psgb_multigrid_set_matrix(psgb_planet* planet, const double* diagonal, const double* off_diagonal,
                              int memory, void* stream);
/* GraphMultigrid::precondition (heat_transport.hpp:70): one V-cycle, x = M^-1 rhs.
 * The GB300 V-cycle smooths with damped Jacobi (the reference: block-hybrid
 * symmetric Gauss-Seidel), so x approximates the same inverse differently. */
int psgb_multigrid_precondition(psgb_planet* planet, int dtype, const void* rhs, void* solution,
                                int memory, void* stream);

/* The values the GPU holds on multigrid level `level` after set_matrix / a step's
 * assembly: diagonal [rows] and off-diagonals in the level's CSR order (FP64; the
 * Galerkin sums of heat_transport.cpp:157-171, in the reference's summation order). */
int psgb_multigrid_level_values(psgb_planet* planet, uint32_t level, double* diagonal, double* off_diagonal);

typedef struct psgb_solve_options {
    int precision;               /* PSGB_PRECISION_* */
    int method;                  /* PSGB_METHOD_* */
    double tolerance;            /* ||b - A x||_2 <= tolerance ||b||_2, FP64 residual */
    double inner_tolerance;      /* mixed precision: residual reduction per refinement */
    int max_iterations;          /* Krylov iterations per (inner) solve */
    int max_refinements;         /* FP64 refinement steps */
    int poll;                    /* Krylov iterations between host status reads */
    int pre_sweeps, post_sweeps; /* Jacobi sweeps per level */
    double jacobi_omega;         /* Jacobi damping */
    int schedule;                /* PSGB_SCHEDULE_*; results are identical for every schedule */
} psgb_solve_options;
void psgb_solve_options_default(psgb_solve_options* out);

typedef struct psgb_solve_report {
    int status;                  /* PSGB_OK or PSGB_ERR_* */
    int refinements;             /* FP64 refinement steps taken */
    int iterations;              /* Krylov iterations, summed over refinements */
    double relative_residual;    /* ||b - A x|| / ||b|| in FP64 */
} psgb_solve_report;

/* The linear solve of the implicit step on the planet's graph:
 *   (A_c / s_c) x_c + K sum_e w_e (x_c - x_n) = rhs_c      (s_c > 0; else x_c = 0 rows)
 * Replaces solve_newton_system (heat_transport.cpp:337-429). x holds the initial
 * guess on entry (zeros reproduce the reference's start). */
int psgb_solve_newton_system(psgb_planet* planet, const psgb_solve_options* options,
                             double conductance_W_K, const double* slope, const double* rhs,
                             double* x, psgb_solve_report* report, int memory, void* stream);

/* One implicit diffusive heat-transport sub-step with the linear column response
 * T = T0 + (dt/C)(S + H): the response solve_implicit_transport
 * (heat_transport.cpp:595-772) receives from a linear tile, solved directly:
 *   (C/dt M + K L) T = C/dt M T0 + M S,
 * then the conservative flux form H = K lap(T) and T_new = T0 + (dt/C)(S + H). */
typedef struct psgb_step_params {
    double heat_capacity_J_m2_K; /* C */
    double dt_s;                 /* dt */
    double conductance_W_K;      /* K (used when edge_conductance is NULL) */
    const double* edge_conductance; /* optional, per undirected edge [edges], W/K; HOST */
    int edge_conductance_stored;    /* nonzero: the per-edge conductance stored with
                                       psgb_batch_set_edge_conductance (edge_conductance NULL) */
} psgb_step_params;

typedef struct psgb_step_report {
    psgb_solve_report solve;
    double sum_W;                /* sum A H (zero to rounding) */
    double absolute_sum_W;       /* sum A |H| */
    double dissipation_W_K;      /* sum A H T (<= 0) */
    double closure;              /* |sum A C dT/dt - sum A S| / sum A |S| */
} psgb_step_report;

int psgb_transport_step(psgb_planet* planet, const psgb_step_params* params,
                        const psgb_solve_options* options, const double* t0_K, const double* source_W_m2,
                        double* t_new_K, double* transport_W_m2, psgb_step_report* report, int memory,
                        void* stream);

/* The same step, allocating nothing (no counterpart in the reference). For callers that
 * may not call cudaMalloc or any other allocating CUDA routine while they run: a loop
 * with a fixed memory budget reserved up front, a host that lends the library a GPU under
 * a hard memory cap, a plugin host whose allocator owns the device memory. All solver
 * workspace lives in one static 8 MiB device array of this library, which every GPU that
 * loads the library holds until the process exits. DEVICE pointers only, ordered on
 * `stream`; the call waits for `stream` before it returns. Planets of at most 10,242
 * cells (a level-5 mesh); larger ones fail with PSGB_ERR_INVALID_ARGUMENT, and so does
 * edge_conductance_stored (pass the per-edge array instead). The first call on a device
 * looks up that array's device address; make it before any stream capture. CUDA loads
 * kernels lazily by default, so make one warm-up call per precision (or set
 * CUDA_MODULE_LOADING=EAGER) before relying on the no-allocation property. Calls share
 * the array and it keeps the last call's contents: calls that overlap on the GPU race,
 * serialise them. */
int psgb_transport_step_noalloc(psgb_planet* planet, const psgb_step_params* params,
                                const psgb_solve_options* options, const double* t0_K,
                                const double* source_W_m2, double* t_new_K, double* transport_W_m2,
                                psgb_step_report* report, void* stream);

/* Up to 32 sub-steps of ONE planet with the same parameters (C, dt, conductances),
 * solved together as one block: replaces `count` calls of solve_implicit_transport
 * (heat_transport.cpp:595-772) that share the planet's matrix and differ in their
 * states and sources (ensembles, perturbed sources). The vectors of all sub-steps are
 * interleaved so that every sweep reads the matrix and its column indices once for all
 * of them. Sub-step j takes t0_K[j] and source_W_m2[j] and writes t_new_K[j] (and
 * transport_W_m2[j] when that array and its entry are not NULL) and reports[j]; each
 * equals psgb_transport_step of that sub-step alone bit for bit (untuned, or under the
 * same tuning without block-local sweeps, which the block solve does not apply).
 * BiCGSTAB only; per-edge conductance as an array (not stored). HOST or DEVICE arrays
 * per `memory`; returns the first failing sub-step's status. */
int psgb_transport_step_multi(psgb_planet* planet, const psgb_step_params* params,
                              const psgb_solve_options* options, uint32_t count, const double* const* t0_K,
                              const double* const* source_W_m2, double* const* t_new_K,
                              double* const* transport_W_m2, psgb_step_report* reports, int memory,
                              void* stream);

/* ---- batches: many planets of uneven levels solved together -------------------
 * Concatenated block layout (each planet padded to 256-row tiles), per-planet
 * convergence masks, one stream of launches for all planets. */
int psgb_batch_create(psgb_planet* const* planets, uint32_t count, psgb_batch** out);
void psgb_batch_destroy(psgb_batch* batch);
uint64_t psgb_batch_device_bytes(const psgb_batch* batch);
/* Per planet i: params[i], t0[i], source[i] in, t_new[i] (and optionally
 * transport[i]) out, reports[i]. */
int psgb_batch_transport_step(psgb_batch* batch, const psgb_step_params* params,
                              const psgb_solve_options* options, const double* const* t0_K,
                              const double* const* source_W_m2, double* const* t_new_K,
                              double* const* transport_W_m2, psgb_step_report* reports, int memory,
                              void* stream);

/* The same with only the planets whose `active[i]` (host, one byte per planet) is
 * non-zero taking part; the others' arrays may be NULL and their state is untouched
 * (continuous batching: a request loop steps whichever planets have requests). */
int psgb_batch_transport_step_masked(psgb_batch* batch, const uint8_t* active, const psgb_step_params* params,
                                     const psgb_solve_options* options, const double* const* t0_K,
                                     const double* const* source_W_m2, double* const* t_new_K,
                                     double* const* transport_W_m2, psgb_step_report* reports, int memory,
                                     void* stream);

/* The implicit transport solve with a general tile response: replaces
 * solve_implicit_transport (heat_transport.cpp:595-772) with its ImplicitTransportSettings
 * and ImplicitTransportResult (heat_transport.hpp:82-119). The response stays with the
 * caller, as TransportResponse (heat_transport.hpp:78-80): for sources h (W/m^2) it
 * writes the cell mean temperatures T(h) (K) and their slopes dT/dh (K m^2/W; 0 holds a
 * cell); HOST arrays of `cells` values; a nonzero return aborts the solve. The two-point
 * Laplacians and every linear Newton system run on the GPU (the system with `options`:
 * precision, method, smoother; its tolerance and iteration cap come from `settings`).
 * All arrays are HOST arrays in the planet's cell order; `latent_W_m2` may be NULL.
 * The Newton iterate lives in device memory; each evaluation copies h to the host and
 * T, dT/dh back (pinned buffers). */
typedef int (*psgb_transport_response)(void* user, uint64_t cells, const double* source_W_m2, double* mean_K,
                                       double* slope_K_m2_W);
typedef struct psgb_transport_settings {
    int max_newton_iterations;        /* 30 */
    int max_line_search_halvings;     /* 12 */
    double rounding_floor_W_m2;       /* 1e-3: a failed line search below this ends the solve */
    int max_non_monotone_steps;       /* 4: full steps across kinks above it */
    double max_non_monotone_growth;   /* 100: largest merit growth such a step may bring */
    double newton_tolerance_W_m2;     /* 1e-6: stop at max |h - K lap T(h)| below this */
    double cg_relative_tolerance;     /* 1e-6: inner (inexact) Newton solves */
    int max_cg_iterations;            /* 2000 */
} psgb_transport_settings;
void psgb_transport_settings_default(psgb_transport_settings* out);
typedef struct psgb_transport_result {
    double consistency_residual_W_m2; /* max |H - h| at the last iterate */
    int newton_iterations;
    int cg_iterations;                /* Krylov iterations summed over Newton iterations */
    double sum_W;                     /* sum A H: zero to rounding */
    double absolute_sum_W;            /* sum A |H| */
    double dissipation_W_K;           /* sum A H T <= 0 */
} psgb_transport_result;
int psgb_solve_implicit_transport(psgb_planet* planet, double conductance_W_K, const double* source_floor_W_m2,
                                  psgb_transport_response response, void* user,
                                  const psgb_transport_settings* settings, const psgb_solve_options* options,
                                  const double* latent_W_m2, double* source_out_W_m2, double* mean_out_K,
                                  psgb_transport_result* result);

/* The same solve with the response on the GPU: the whole Newton iteration (response,
 * Laplacians, merit sums, line search trials, linear systems) stays in device memory;
 * the host reads two scalars per evaluation (the merit sum A F^2 and max |F|) to take
 * the line search's decisions. The response is called on the host with DEVICE arrays of
 * `cells` values and the solve's stream, and enqueues its work on that stream. The
 * floor, latent heat and outputs are HOST or DEVICE arrays as `memory` says. */
typedef int (*psgb_device_response)(void* user, uint64_t cells, const double* source_W_m2, double* mean_K,
                                    double* slope_K_m2_W, void* stream);
int psgb_solve_implicit_transport_device(psgb_planet* planet, double conductance_W_K,
                                         const double* source_floor_W_m2, psgb_device_response response,
                                         void* user, const psgb_transport_settings* settings,
                                         const psgb_solve_options* options, const double* latent_W_m2,
                                         double* source_out_W_m2, double* mean_out_K,
                                         psgb_transport_result* result, int memory, void* stream);

/* The quartic column response of the reference's transport test (test_heat_transport.cpp:
 * 30-76) as a GPU kernel: per cell the root x of a x + r x^4 = b + h by
 * solve_column_surface's Newton without evaporation (column_step.cpp:254-270; bit-
 * identical), slope 1/(a + 4 r x^3); cells whose index is a multiple of hold_stride are
 * held at hold_K (slope 0) when they would pass it (hold_stride 0: none). `b` is a
 * DEVICE array of `cells` values. With `planet` set (an agglomerated planet), the cells
 * are its FINE cells: h is scattered from the nodes, the quartic runs per fine cell and
 * the nodes take the area-weighted means (surface_energy.cpp:1240-1296); `scratch` is
 * DEVICE memory of 2 fine-cell arrays. */
typedef struct psgb_quartic_response {
    double a;
    double radiative;          /* r; the test's 0.75 * 0.97 * sigma */
    const double* b;
    uint32_t hold_stride;      /* the test's 7 */
    double hold_K;             /* the test's 273.15 */
    psgb_planet* planet;       /* NULL: per node */
    double* scratch;
} psgb_quartic_response;
/* psgb_device_response with user = psgb_quartic_response*. */
int psgb_quartic_device_response(void* user, uint64_t cells, const double* source_W_m2, double* mean_K,
                                 double* slope_K_m2_W, void* stream);

/* ---- non-symmetric solves: heat_transport.hpp:140-238, incomplete_lu.hpp:14-43 ---- */

/* IncompleteLU (incomplete_lu.hpp:14-43): block ILU(0) of diagonal * scale + off on a
 * CSR pattern (row i's off-diagonal columns neighbour[offset[i] .. offset[i + 1])),
 * blocks of rows [block_start[b], block_start[b + 1]) factored on their own. HOST arrays;
 * factored on the GPU at creation, level-scheduled inside each block, bit-identical to
 * the reference's factor. PSGB_ERR_BREAKDOWN on a zero pivot (the reference's
 * std::runtime_error). */
typedef struct psgb_incomplete_lu psgb_incomplete_lu;
int psgb_incomplete_lu_create(uint32_t rows, const uint32_t* offset, const uint32_t* neighbour,
                              const double* diagonal, const double* off, const uint32_t* block_start,
                              uint32_t blocks, double diagonal_scale, psgb_incomplete_lu** out);
/* IncompleteLU::solve: x <- (LU)^-1 x. */
int psgb_incomplete_lu_solve(psgb_incomplete_lu* lu, double* x, int memory, void* stream);
void psgb_incomplete_lu_destroy(psgb_incomplete_lu* lu);

/* AdvectionDiffusion (heat_transport.hpp:140-166): per CSR entry of the planet's graph
 * the eddies' conductance G (W/K, symmetric) and per layer the mass leaving across the
 * face (kg/s, layer-major, antisymmetric); c_p; per node the eddies' latent heat E
 * (W/m^2) or NULL. Arrays HOST or DEVICE with the call's `memory`. */
typedef struct psgb_advection_diffusion {
    uint32_t layers;
    const double* conductance_W_K;
    const double* outflow_kg_s;
    double heat_capacity_J_kg_K;      /* 1004.64 */
    const double* eddy_latent_W_m2;
} psgb_advection_diffusion;

/* advection_diffusion_source (heat_transport.hpp:168-175): H_eddy and H_advective per
 * node for given theta_c and s_l (layer-major); bit-identical. */
int psgb_advection_diffusion_source(psgb_planet* planet, const psgb_advection_diffusion* transport,
                                    const double* mean_K, const double* energy_J_kg, double* eddy_W_m2,
                                    double* advective_W_m2, int memory, void* stream);

/* solve_implicit_tracer (heat_transport.hpp:198-238): the layers' mixing ratios
 * (layer-major, layers x nodes) carried implicitly by the advective fluxes (upwind), the
 * eddies and the vertical fluxes that close each layer's divergence; BiCGSTAB with the
 * stacked system's block ILU(0) on the GPU; the flux form of the solution. */
typedef struct psgb_tracer_result {
    int iterations;
    double relative_residual;
    double clipped_kg;
    double column_divergence_kg_s;
} psgb_tracer_result;
int psgb_solve_implicit_tracer(psgb_planet* planet, const psgb_advection_diffusion* transport,
                               const double* layer_mass_kg, const double* tracer, double dt_s,
                               double relative_tolerance, int max_iterations, double* tracer_out,
                               psgb_tracer_result* result, int memory, void* stream);

/* solve_implicit_advection_diffusion (heat_transport.hpp:240-248): Newton on h with
 * h = H(theta_c(h), s(h)), the line search of the implicit transport solve; the Newton
 * system J = I - dH/dh on the graph's pattern solved by BiCGSTAB preconditioned with the
 * V-cycle of the eddies' symmetric part, then the block ILU(0) of J on what is left.
 * The response (AdvectionResponse, heat_transport.hpp:170-173) gives theta_c, its slope,
 * and per layer s_l and ds_l/dh (layer-major): on the host (HOST arrays) or on the GPU
 * (DEVICE arrays, enqueued on `stream`); give exactly one. `initial_source_W_m2` (may be
 * NULL) starts the iteration (ImplicitTransportSettings::initial_source_W_m2). */
typedef int (*psgb_advection_response)(void* user, uint64_t nodes, uint32_t layers, const double* source_W_m2,
                                       double* mean_K, double* slope_K_m2_W, double* energy_J_kg,
                                       double* energy_slope_J_kg_m2_W);
typedef int (*psgb_device_advection_response)(void* user, uint64_t nodes, uint32_t layers,
                                              const double* source_W_m2, double* mean_K, double* slope_K_m2_W,
                                              double* energy_J_kg, double* energy_slope_J_kg_m2_W, void* stream);
typedef struct psgb_advection_result {
    double consistency_residual_W_m2;
    int newton_iterations;
    int linear_iterations;
    double sum_W;
    double absolute_sum_W;
    double eddy_absolute_sum_W;
    double advective_absolute_sum_W;
} psgb_advection_result;
int psgb_solve_implicit_advection_diffusion(psgb_planet* planet, const psgb_advection_diffusion* transport,
                                            const double* source_floor_W_m2, const double* initial_source_W_m2,
                                            psgb_advection_response host_response,
                                            psgb_device_advection_response device_response, void* user,
                                            const psgb_transport_settings* settings, double* source_out_W_m2,
                                            double* mean_out_K, double* energy_out_J_kg,
                                            psgb_advection_result* result, int memory, void* stream);

/* Stores per-edge conductances with a batch (HOST arrays, one per planet, [edges] W/K;
 * NULL entries clear a planet's): steps whose params set edge_conductance_stored use them
 * without passing (and without the library comparing) the arrays on every call. */
int psgb_batch_set_edge_conductance(psgb_batch* batch, const double* const* edge_conductance);

/* Nonzero: every step of the batch assembles its matrix again on the device (the fine
 * matrix from the staged C, dt and conductances, the Galerkin values of every coarse
 * level, the coarsest levels' inverses), as the reference does on every call of
 * solve_implicit_transport (heat_transport.cpp:613); zero (the default): the assembled
 * matrix is reused while C, dt and the conductances are unchanged. Results are the same
 * either way. */
int psgb_batch_set_reassembly(psgb_batch* batch, int every_step);

/* Nonzero: the batch's solves run on a stream of the device's highest priority (its
 * kernels are scheduled first where batches stepped side by side compete for the GPU, e.g.
 * the lanes whose planets need the most iterations); zero (the default): normal priority.
 * Not while a step of the batch runs. Results are the same either way. */
int psgb_batch_set_priority(psgb_batch* batch, int high);

/* Per-level settings of a batch's solve. The reference has no counterpart (its smoother
 * is fixed, heat_transport.cpp:258-286); the autotuner picks them for the batch's GPU:
 * launch shapes (tiles per thread; never change a result) and damped-Jacobi sweeps per
 * level (change the preconditioner; every tuned solve still meets the tolerance). */
#define PSGB_MAX_LEVELS 12
typedef struct psgb_tuning {
    uint32_t levels;                      /* multigrid levels of the batch */
    int pre_sweeps[PSGB_MAX_LEVELS];      /* per level, 1..8 */
    int post_sweeps[PSGB_MAX_LEVELS];     /* per level, 0..8 */
    int stencil_tiles[PSGB_MAX_LEVELS];   /* tiles per thread of the stencil launches: 1 or 2 */
    int vector_tiles[PSGB_MAX_LEVELS];    /* tiles per thread of the vector launches: 1 or 4 */
    double jacobi_omega;
    double tuned_solve_ms;                /* autotune: trial solve with the chosen settings */
    double default_solve_ms;              /* autotune: trial solve with the settings before */
    int trial_solves;                     /* autotune: solves timed */
    int coarse_tail_level;                /* levels from this one down run one block per planet; 0: none */
    int block_sweeps[PSGB_MAX_LEVELS];    /* per level: Jacobi sweeps per smoothing launch, each tile in shared
                                             memory with its neighbours in other tiles held (1..8; 1 = plain) */
    int coarse_tail_single;               /* 0: a large planet's tail runs on several co-resident blocks
                                             (cooperative launch, per-planet barriers); 1: one block each;
                                             2: one block each with the tail levels' vectors in shared memory;
                                             3: a thread-block cluster each (coarse_tail_cluster blocks) with
                                             the vectors in the cluster's distributed shared memory */
    uint32_t coarse_tail_blocks;          /* out: blocks of the tail launch last built under these settings
                                             (before one: the launch they ask for; 0: no tail) */
    uint32_t coarse_tail_cluster;         /* coarse_tail_single = 3: blocks per planet's cluster, 2, 4 or 8 */
    double coarse_correction;             /* scale of the coarse-grid correction, x += s P e (0 or 1: plain;
                                             over-correction, 1.5 to 2, cuts the Krylov iterations) */
} psgb_tuning;

/* Times trial solves of one sub-step (the inputs as for psgb_batch_transport_step, every
 * planet taking part, each solve from the step's own initial guess; nothing is written
 * back) and keeps the fastest settings that meet the options' tolerance on every planet. While a batch holds a tuning, its solves use
 * it instead of the options' uniform sweeps and damping. */
int psgb_batch_autotune(psgb_batch* batch, const psgb_step_params* params, const psgb_solve_options* options,
                        const double* const* t0_K, const double* const* source_W_m2, int memory, void* stream,
                        psgb_tuning* out);
/* The settings the batch's solves use now. */
int psgb_batch_get_tuning(const psgb_batch* batch, psgb_tuning* out);
/* Applies settings (e.g. a tuning kept from an earlier run); NULL returns to the options'
 * uniform sweeps and the default launch shapes. */
int psgb_batch_set_tuning(psgb_batch* batch, const psgb_tuning* tuning);
/* The same settings for a planet's own solves (psgb_transport_step,
 * psgb_transport_step_multi, psgb_multigrid_precondition, psgb_solve_newton_system): a
 * tuning of a one-planet batch of this planet carries over bit for bit; NULL returns to
 * the options' uniform sweeps. */
int psgb_planet_set_tuning(psgb_planet* planet, const psgb_tuning* tuning);
int psgb_planet_get_tuning(psgb_planet* planet, psgb_tuning* out);

/* ---- column radiation: sim/planet/atmosphere/atmosphere_column.hpp ----------------
 * column_radiation (humidity variant, :85-104) + cloud_optics (:599-623) +
 * add_cloud_longwave (:627-634) + longwave_fluxes (:125-143) for `cells` columns of
 * `layers` (1..16) equal-mass layers; layer-major arrays [layers][cells]. */
typedef struct psgb_column_constants {
    double dry_optical_depth, vapour_absorption_m2_kg, in_cloud_water_path_kg_m2,
        effective_radius_m, cloud_asymmetry, cloud_longwave_absorption_m2_kg,
        reference_pressure_Pa, gravity_m_s2, stefan_boltzmann;
} psgb_column_constants;
/* outputs: emissivity, absorbed [layers][cells]; fraction, reflectance [layers][cells];
 * scalars [5][cells] = downward surface LW, OLR, SW transmission, column cloud
 * fraction, column cloud optical depth. */
int psgb_column_radiation(uint32_t cells, uint32_t layers, const psgb_column_constants* constants,
                          const double* temperature_K, const double* humidity, const double* cloud_water,
                          const double* surface_temperature_K, const double* surface_pressure_Pa,
                          double* emissivity, double* absorbed, double* fraction, double* reflectance,
                          double* scalars, int memory, void* stream);

/* ---- launch accounting and kernel timing (no counterpart in the reference) -------
 * psgb_launch_count: kernels this library has launched since it was loaded.
 * psgb_profile_begin: from now on, time every launch of one kernel family ("smooth",
 * "residual", "restrict", "prolong", "dense", "krylov_spmv", "krylov_vector", "refine",
 * "setup", "step", "operator", "column") with CUDA events on its launching stream.
 * psgb_profile_end: synchronises, returns the summed device time (ms) and launch count of
 * that family, and the algorithmic bytes the Jacobi sweeps moved since the profile began. */
uint64_t psgb_launch_count(void);
int psgb_profile_begin(const char* family);
int psgb_profile_end(double* total_ms, uint64_t* launches, uint64_t* swept_bytes);

/* ---- inputs ---------------------------------------------------------------------
 * Sub-step-mean insolation of sub-step `substep` for the Earth-development planet
 * (compute_substep_mean_insolation, sim/planet/orbit/substep_forcing.cpp:102-127),
 * computed on the host; cells floats. */
int psgb_substep_mean_insolation(const psgb_planet* planet, int64_t substep, float* out);
/* The same on the GPU: the sub-step's 16 orbit nodes on the host, the per-cell
 * quadrature in a kernel; `out` [cells] FP32, HOST or DEVICE per `memory`. Within one
 * FP32 ulp of the reference (CUDA's acos/sin against the host library's). */
int psgb_substep_mean_insolation_gpu(psgb_planet* planet, int64_t substep, float* out, int memory, void* stream);

/* ---- the serving loop (no counterpart in the reference: it steps one planet per call)
 * A continuous-batching request loop for implicit heat-transport sub-steps of registered
 * planets of uneven mesh levels. Planets of one mesh level form a lane: while admitted,
 * the lane's batch (mesh, hierarchy, matrix) and its planets' temperatures stay in device
 * memory, and a worker thread steps, in rounds, the oldest queued request of every planet
 * of the lane together (psgb_batch_transport_step_masked); requests arriving during a
 * round join the next one, and the lanes' rounds overlap on the GPU. Lanes are admitted
 * against a device-memory budget: the least recently used idle lanes are evicted first
 * (their temperatures copied back to the host), or the lane waits until one goes idle; a
 * lane larger than the budget fails its requests with PSGB_ERR_BUDGET. Under memory
 * pressure lanes take turns (yield_after_s). A request's new temperature is the step from
 * the planet's state after its earlier requests. */
typedef struct psgb_server psgb_server;

typedef struct psgb_server_config {
    double budget_bytes;          /* device memory for resident lanes */
    double bytes_per_cell;        /* a resident lane's estimate per cell (<= 0: 700) */
    psgb_solve_options options;   /* every step's solve */
    int autotune;                 /* nonzero: tune each lane at its first admission (psgb_batch_autotune),
                                     reapplied at later admissions */
    int device;                   /* CUDA device of the lanes */
    double yield_after_s;         /* a lane waiting for memory this long makes the resident lanes
                                     that stepped since take turns with it (<= 0: 0.25 s) */
} psgb_server_config;

typedef struct psgb_server_stats {
    uint64_t submitted, completed, failed, rounds, evictions, admissions;
    uint64_t resident_bytes;
    uint32_t resident_lanes, planets;
    double p50_ms, p99_ms;        /* submit-to-done latency of the completed requests */
} psgb_server_stats;

int psgb_server_create(const psgb_server_config* config, psgb_server** out);
/* Stops the lanes after their running round; requests still queued fail. */
void psgb_server_destroy(psgb_server* server);
/* Registers a planet (before its level's first request): mesh level and radius, its step
 * parameters (params->edge_conductance: optional HOST array per undirected edge), its
 * initial temperature (HOST, cells). */
int psgb_server_add_planet(psgb_server* server, uint32_t level, double radius_m, const psgb_step_params* params,
                           const double* t0_K, uint32_t* planet_out);
/* Queues one sub-step of `planet` with this source (HOST, cells; copied). */
int psgb_server_submit(psgb_server* server, uint32_t planet, const double* source_W_m2, uint64_t* request_out);
/* Waits for a request (timeout_s < 0: no limit). Returns its status (PSGB_OK, a solve
 * status, PSGB_ERR_BUDGET, ...) and, once finished, forgets it after copying the new
 * temperature (t_new_K, HOST, cells; may be NULL) and the report (may be NULL);
 * PSGB_ERR_TIMEOUT while it is still queued or running. Every request is waited on once. */
int psgb_server_wait(psgb_server* server, uint64_t request, double timeout_s, double* t_new_K,
                     psgb_step_report* report);
/* The planet's temperature after its finished requests (HOST, cells). */
int psgb_server_state(psgb_server* server, uint32_t planet, double* t_K);
int psgb_server_stats_get(psgb_server* server, psgb_server_stats* out);
/* Forgets the counts and latencies so far (after a warm-up); resident lanes stay. Call
 * it while the server is idle (every submitted request waited on): a request still queued
 * or running when it resets completes into the new counts without being counted as
 * submitted there. */
int psgb_server_stats_reset(psgb_server* server);

#ifdef __cplusplus
}
#endif

#endif /* PLANETSIM_GB300_H */

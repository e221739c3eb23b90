"""ctypes declarations of the C-ABI in include/planetsim_gb300.h.

The library is the in-tree ``planet_game_gb300/lib/libplanetsim_gb300.so``. Loading
it never falls back to anything else: if the file is missing, ``load()`` raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIBRARY = Path(__file__).resolve().parent / "lib" / "libplanetsim_gb300.so"

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_OUT_OF_MEMORY = 2
ERR_NOT_CONVERGED = 3
ERR_BREAKDOWN = 4
ERR_NON_FINITE = 5
ERR_CUDA = 6
ERR_LOGIC = 7
ERR_BUDGET = 8
ERR_TIMEOUT = 9

MEMORY_HOST = 0
MEMORY_DEVICE = 1
DTYPE_F64 = 0
DTYPE_F32 = 1
PRECISION_FP64 = 0
PRECISION_MIXED = 1
METHOD_PCG = 0
METHOD_BICGSTAB = 1
SCHEDULE_AUTO = 0
SCHEDULE_KERNELS = 1
SCHEDULE_PERSISTENT = 2


class PlanetInfo(C.Structure):
    _fields_ = [("cells", C.c_uint64), ("edges", C.c_uint64), ("directed_edges", C.c_uint64),
                ("corners", C.c_uint64), ("levels", C.c_uint32), ("level_rows", C.c_uint32 * 8),
                ("device_bytes", C.c_uint64), ("fine_cells", C.c_uint64)]


class GraphView(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in ("area_m2", "offset", "neighbour", "weight", "weight_sum")]


class MeshView(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in (
        "center", "east", "north", "area_m2", "source_vertex", "edge_offset", "edge_count", "neighbor",
        "edge", "corner", "normal_east", "normal_north", "edge_first", "edge_second", "edge_length_m",
        "edge_distance_m", "corner_unit", "graph_weight", "graph_weight_sum")]


class SolveOptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("method", C.c_int), ("tolerance", C.c_double),
                ("inner_tolerance", C.c_double), ("max_iterations", C.c_int), ("max_refinements", C.c_int),
                ("poll", C.c_int), ("pre_sweeps", C.c_int), ("post_sweeps", C.c_int),
                ("jacobi_omega", C.c_double), ("schedule", C.c_int)]


MAX_LEVELS = 12


class TransportSettings(C.Structure):
    _fields_ = [("max_newton_iterations", C.c_int), ("max_line_search_halvings", C.c_int),
                ("rounding_floor_W_m2", C.c_double), ("max_non_monotone_steps", C.c_int),
                ("max_non_monotone_growth", C.c_double), ("newton_tolerance_W_m2", C.c_double),
                ("cg_relative_tolerance", C.c_double), ("max_cg_iterations", C.c_int)]


class TransportResult(C.Structure):
    _fields_ = [("consistency_residual_W_m2", C.c_double), ("newton_iterations", C.c_int),
                ("cg_iterations", C.c_int), ("sum_W", C.c_double), ("absolute_sum_W", C.c_double),
                ("dissipation_W_K", C.c_double)]


# int response(void* user, uint64_t cells, const double* source, double* mean, double* slope)
TransportResponse = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint64, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                C.POINTER(C.c_double))
# psgb_device_response: (user, cells, source, mean, slope, stream), device pointers
DeviceResponse = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p)


class AdvectionDiffusion(C.Structure):
    _fields_ = [("layers", C.c_uint32), ("conductance_W_K", C.c_void_p), ("outflow_kg_s", C.c_void_p),
                ("heat_capacity_J_kg_K", C.c_double), ("eddy_latent_W_m2", C.c_void_p)]


class TracerResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("relative_residual", C.c_double), ("clipped_kg", C.c_double),
                ("column_divergence_kg_s", C.c_double)]


class AdvectionResult(C.Structure):
    _fields_ = [("consistency_residual_W_m2", C.c_double), ("newton_iterations", C.c_int),
                ("linear_iterations", C.c_int), ("sum_W", C.c_double), ("absolute_sum_W", C.c_double),
                ("eddy_absolute_sum_W", C.c_double), ("advective_absolute_sum_W", C.c_double)]


# psgb_advection_response (host arrays) and psgb_device_advection_response (device pointers)
AdvectionResponse = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint64, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p)
DeviceAdvectionResponse = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint64, C.c_uint32, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p)


class QuarticResponse(C.Structure):
    _fields_ = [("a", C.c_double), ("radiative", C.c_double), ("b", C.c_void_p), ("hold_stride", C.c_uint32),
                ("hold_K", C.c_double), ("planet", C.c_void_p), ("scratch", C.c_void_p)]


class Tuning(C.Structure):
    _fields_ = [("levels", C.c_uint32), ("pre_sweeps", C.c_int * MAX_LEVELS), ("post_sweeps", C.c_int * MAX_LEVELS),
                ("stencil_tiles", C.c_int * MAX_LEVELS), ("vector_tiles", C.c_int * MAX_LEVELS),
                ("jacobi_omega", C.c_double), ("tuned_solve_ms", C.c_double), ("default_solve_ms", C.c_double),
                ("trial_solves", C.c_int), ("coarse_tail_level", C.c_int), ("block_sweeps", C.c_int * MAX_LEVELS),
                ("coarse_tail_single", C.c_int), ("coarse_tail_blocks", C.c_uint32),
                ("coarse_tail_cluster", C.c_uint32), ("coarse_correction", C.c_double)]


class SolveReport(C.Structure):
    _fields_ = [("status", C.c_int), ("refinements", C.c_int), ("iterations", C.c_int),
                ("relative_residual", C.c_double)]


class StepParams(C.Structure):
    _fields_ = [("heat_capacity_J_m2_K", C.c_double), ("dt_s", C.c_double), ("conductance_W_K", C.c_double),
                ("edge_conductance", C.c_void_p), ("edge_conductance_stored", C.c_int)]


class StepReport(C.Structure):
    _fields_ = [("solve", SolveReport), ("sum_W", C.c_double), ("absolute_sum_W", C.c_double),
                ("dissipation_W_K", C.c_double), ("closure", C.c_double)]


class ServerConfig(C.Structure):
    _fields_ = [("budget_bytes", C.c_double), ("bytes_per_cell", C.c_double), ("options", SolveOptions),
                ("autotune", C.c_int), ("device", C.c_int), ("yield_after_s", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [(name, C.c_uint64) for name in (
        "submitted", "completed", "failed", "rounds", "evictions", "admissions", "resident_bytes")] + [
        ("resident_lanes", C.c_uint32), ("planets", C.c_uint32), ("p50_ms", C.c_double), ("p99_ms", C.c_double)]


class ColumnConstants(C.Structure):
    _fields_ = [(name, C.c_double) for name in (
        "dry_optical_depth", "vapour_absorption_m2_kg", "in_cloud_water_path_kg_m2", "effective_radius_m",
        "cloud_asymmetry", "cloud_longwave_absorption_m2_kg", "reference_pressure_Pa", "gravity_m_s2",
        "stefan_boltzmann")]


P = C.c_void_p
_SIGNATURES = {
    "psgb_last_error": (C.c_char_p, []),
    "psgb_abi_version": (C.c_int, []),
    "psgb_planet_create": (C.c_int, [C.c_uint32, C.c_double, C.POINTER(P)]),
    "psgb_planet_create_agglomerated": (C.c_int, [C.c_uint32, C.c_double, C.POINTER(P)]),
    "psgb_planet_graph_view": (C.c_int, [P, C.POINTER(GraphView)]),
    "psgb_planet_group_of_cell": (C.c_int, [P, P]),
    "psgb_group_mean": (C.c_int, [P, P, P, P, P, C.c_int, P]),
    "psgb_group_scatter": (C.c_int, [P, P, P, C.c_int, P]),
    "psgb_planet_destroy": (None, [P]),
    "psgb_planet_info_get": (C.c_int, [P, C.POINTER(PlanetInfo)]),
    "psgb_planet_mesh_view": (C.c_int, [P, C.POINTER(MeshView)]),
    "psgb_planet_hierarchy_level": (C.c_int, [P, C.c_uint32, C.POINTER(C.c_uint64), C.POINTER(P), C.POINTER(P),
                                              C.POINTER(P), C.POINTER(P)]),
    "psgb_laplacian": (C.c_int, [P, C.c_int, P, P, C.c_int, P]),
    "psgb_gradient": (C.c_int, [P, C.c_int, P, P, P, C.c_int, P]),
    "psgb_divergence": (C.c_int, [P, C.c_int, P, P, C.c_int, P]),
    "psgb_diffusion_source": (C.c_int, [P, C.c_double, P, P, C.c_int, P]),
    "psgb_multigrid_set_matrix": (C.c_int, [P, P, P, C.c_int, P]),
    "psgb_multigrid_precondition": (C.c_int, [P, C.c_int, P, P, C.c_int, P]),
    "psgb_multigrid_level_values": (C.c_int, [P, C.c_uint32, P, P]),
    "psgb_solve_options_default": (None, [C.POINTER(SolveOptions)]),
    "psgb_solve_newton_system": (C.c_int, [P, C.POINTER(SolveOptions), C.c_double, P, P, P,
                                           C.POINTER(SolveReport), C.c_int, P]),
    "psgb_transport_step": (C.c_int, [P, C.POINTER(StepParams), C.POINTER(SolveOptions), P, P, P, P,
                                      C.POINTER(StepReport), C.c_int, P]),
    "psgb_transport_step_noalloc": (C.c_int, [P, C.POINTER(StepParams), C.POINTER(SolveOptions), P, P, P, P,
                                              C.POINTER(StepReport), P]),
    "psgb_transport_step_multi": (C.c_int, [P, C.POINTER(StepParams), C.POINTER(SolveOptions), C.c_uint32,
                                            C.POINTER(P), C.POINTER(P), C.POINTER(P), C.POINTER(P),
                                            C.POINTER(StepReport), C.c_int, P]),
    "psgb_batch_create": (C.c_int, [C.POINTER(P), C.c_uint32, C.POINTER(P)]),
    "psgb_batch_destroy": (None, [P]),
    "psgb_batch_set_reassembly": (C.c_int, [P, C.c_int]),
    "psgb_batch_set_priority": (C.c_int, [P, C.c_int]),
    "psgb_batch_device_bytes": (C.c_uint64, [P]),
    "psgb_batch_transport_step": (C.c_int, [P, C.POINTER(StepParams), C.POINTER(SolveOptions), C.POINTER(P),
                                            C.POINTER(P), C.POINTER(P), C.POINTER(P), C.POINTER(StepReport),
                                            C.c_int, P]),
    "psgb_batch_transport_step_masked": (C.c_int, [P, P, C.POINTER(StepParams), C.POINTER(SolveOptions),
                                                   C.POINTER(P), C.POINTER(P), C.POINTER(P), C.POINTER(P),
                                                   C.POINTER(StepReport), C.c_int, P]),
    "psgb_batch_autotune": (C.c_int, [P, C.POINTER(StepParams), C.POINTER(SolveOptions), C.POINTER(P), C.POINTER(P),
                                      C.c_int, P, C.POINTER(Tuning)]),
    "psgb_batch_get_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "psgb_batch_set_edge_conductance": (C.c_int, [P, C.POINTER(P)]),
    "psgb_batch_set_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "psgb_planet_set_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "psgb_planet_get_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "psgb_transport_settings_default": (None, [C.POINTER(TransportSettings)]),
    "psgb_solve_implicit_transport": (C.c_int, [P, C.c_double, P, TransportResponse, P, C.POINTER(TransportSettings),
                                                C.POINTER(SolveOptions), P, P, P, C.POINTER(TransportResult)]),
    "psgb_solve_implicit_transport_device": (C.c_int, [P, C.c_double, P, P, P, C.POINTER(TransportSettings),
                                                       C.POINTER(SolveOptions), P, P, P, C.POINTER(TransportResult),
                                                       C.c_int, P]),
    "psgb_quartic_device_response": (C.c_int, [P, C.c_uint64, P, P, P, P]),
    "psgb_incomplete_lu_create": (C.c_int, [C.c_uint32, P, P, P, P, P, C.c_uint32, C.c_double, C.POINTER(P)]),
    "psgb_incomplete_lu_solve": (C.c_int, [P, P, C.c_int, P]),
    "psgb_incomplete_lu_destroy": (None, [P]),
    "psgb_advection_diffusion_source": (C.c_int, [P, C.POINTER(AdvectionDiffusion), P, P, P, P, C.c_int, P]),
    "psgb_solve_implicit_tracer": (C.c_int, [P, C.POINTER(AdvectionDiffusion), P, P, C.c_double, C.c_double, C.c_int,
                                             P, C.POINTER(TracerResult), C.c_int, P]),
    "psgb_solve_implicit_advection_diffusion": (C.c_int, [P, C.POINTER(AdvectionDiffusion), P, P, P, P, P,
                                                          C.POINTER(TransportSettings), P, P, P,
                                                          C.POINTER(AdvectionResult), C.c_int, P]),
    "psgb_column_radiation": (C.c_int, [C.c_uint32, C.c_uint32, C.POINTER(ColumnConstants), P, P, P, P, P, P, P,
                                        P, P, P, C.c_int, P]),
    "psgb_substep_mean_insolation": (C.c_int, [P, C.c_int64, P]),
    "psgb_substep_mean_insolation_gpu": (C.c_int, [P, C.c_int64, P, C.c_int, P]),
    "psgb_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(P)]),
    "psgb_server_destroy": (None, [P]),
    "psgb_server_add_planet": (C.c_int, [P, C.c_uint32, C.c_double, C.POINTER(StepParams), P,
                                         C.POINTER(C.c_uint32)]),
    "psgb_server_submit": (C.c_int, [P, C.c_uint32, P, C.POINTER(C.c_uint64)]),
    "psgb_server_wait": (C.c_int, [P, C.c_uint64, C.c_double, P, C.POINTER(StepReport)]),
    "psgb_server_state": (C.c_int, [P, C.c_uint32, P]),
    "psgb_server_stats_get": (C.c_int, [P, C.POINTER(ServerStats)]),
    "psgb_server_stats_reset": (C.c_int, [P]),
    "psgb_launch_count": (C.c_uint64, []),
    "psgb_profile_begin": (C.c_int, [C.c_char_p]),
    "psgb_profile_end": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
}

# Every symbol the header declares (checked by the CPU test suite).
EXPORTED = tuple(_SIGNATURES)

_lib: C.CDLL | None = None


class GB300Error(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"planetsim_gb300 error {code}: {message}")
        self.code = code


def load() -> C.CDLL:
    """Load the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIBRARY.exists():
            raise FileNotFoundError(f"{LIBRARY} is missing: run planet_game_gb300.build.build_library()")
        lib = C.CDLL(str(LIBRARY))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(code: int) -> int:
    if code != OK:
        raise GB300Error(code, load().psgb_last_error().decode())
    return code


def default_options() -> SolveOptions:
    o = SolveOptions()
    load().psgb_solve_options_default(C.byref(o))
    return o

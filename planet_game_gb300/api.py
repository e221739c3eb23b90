"""Python mirror of the reference's operator and solver API over the GB300 C-ABI.

Names follow the reference headers: ``make_icosphere`` / ``PlanetMesh``
(sim/planet/mesh/icosphere.hpp, planet_mesh.hpp), ``mesh_transport_graph`` /
``TransportGraph``, ``GraphMultigrid`` and ``diffusion_source``
(sim/planet/surface/heat_transport.hpp), ``laplacian`` / ``gradient`` /
``divergence`` (sim/planet/operators/finite_volume.hpp). Errors raise the same
Python exception families the reference raises in C++ (ValueError for
std::invalid_argument, RuntimeError otherwise).

Arrays are numpy (host memory; each call copies in and out) or CUDA torch tensors
(device memory; the call is ordered on torch's current stream). Everything computes on
the GPU through the C-ABI; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import capi

_DT = {np.dtype(np.float64): capi.DTYPE_F64, np.dtype(np.float32): capi.DTYPE_F32}


def _raise(code: int) -> None:
    if code == capi.OK:
        return
    msg = capi.load().psgb_last_error().decode()
    if code == capi.ERR_INVALID_ARGUMENT:
        raise ValueError(msg)
    raise capi.GB300Error(code, msg)


def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


def _ptr(a):
    if _is_torch(a):
        if not a.is_cuda or not a.is_contiguous():
            raise ValueError("torch tensors must be contiguous CUDA tensors")
        return C.c_void_p(a.data_ptr())
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("numpy arrays must be C-contiguous")
    return C.c_void_p(a.ctypes.data)


def _memory_of(*arrays) -> tuple[int, C.c_void_p]:
    kinds = {_is_torch(a) for a in arrays if a is not None}
    if len(kinds) != 1:
        raise ValueError("pass either all numpy arrays or all CUDA tensors")
    if kinds.pop():
        import torch

        return capi.MEMORY_DEVICE, C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return capi.MEMORY_HOST, C.c_void_p(None)


def _dtype_code(a) -> int:
    if _is_torch(a):
        import torch

        return {torch.float64: capi.DTYPE_F64, torch.float32: capi.DTYPE_F32}[a.dtype]
    return _DT[a.dtype]


def _empty_like(a, shape, dtype=None):
    if _is_torch(a):
        import torch

        return torch.empty(shape, dtype=dtype or a.dtype, device=a.device)
    return np.empty(shape, dtype=dtype or a.dtype)


def _view(ptr: int, dtype, count: int) -> np.ndarray:
    if count == 0:
        return np.empty(0, dtype=dtype)
    buf = (C.c_char * (count * np.dtype(dtype).itemsize)).from_address(ptr)
    return np.frombuffer(buf, dtype=dtype, count=count).copy()


class PlanetMesh:
    """A planet's SCVT mesh, its transport graph and multigrid hierarchy (one handle).

    Built by the host builder that reproduces the reference's make_icosphere bit for bit;
    the device copy is uploaded on first GPU use.
    """

    def __init__(self, level: int, radius_m: float, agglomerated: bool = False):
        lib = capi.load()
        h = C.c_void_p()
        create = lib.psgb_planet_create_agglomerated if agglomerated else lib.psgb_planet_create
        _raise(create(C.c_uint32(level), C.c_double(radius_m), C.byref(h)))
        self._h = h
        self.agglomerated = bool(agglomerated)
        # the mesh the transport runs on: one level coarser when agglomerated
        self.subdivision = max(int(level) - 1, 0) if agglomerated else int(level)
        self.radius_m = float(radius_m)
        info = capi.PlanetInfo()
        _raise(lib.psgb_planet_info_get(h, C.byref(info)))
        self.fine_cell_count = int(info.fine_cells)
        self.cell_count = int(info.cells)
        self.edge_count = int(info.edges)
        self.directed_edge_count = int(info.directed_edges)
        self.corner_count = int(info.corners)
        self.level_rows = [int(info.level_rows[i]) for i in range(info.levels)]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            capi.load().psgb_planet_destroy(h)
            self._h = None

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def device_bytes(self) -> int:
        info = capi.PlanetInfo()
        _raise(capi.load().psgb_planet_info_get(self._h, C.byref(info)))
        return int(info.device_bytes)

    def arrays(self) -> dict[str, np.ndarray]:
        """Copies of the mesh arrays (the reference PlanetMesh's fields, flattened)."""
        v = capi.MeshView()
        _raise(capi.load().psgb_planet_mesh_view(self._h, C.byref(v)))
        n, e, d, k = self.cell_count, self.edge_count, self.directed_edge_count, self.corner_count
        return {
            "center": _view(v.center, np.float64, 3 * n).reshape(n, 3),
            "east": _view(v.east, np.float64, 3 * n).reshape(n, 3),
            "north": _view(v.north, np.float64, 3 * n).reshape(n, 3),
            "area_m2": _view(v.area_m2, np.float64, n),
            "source_vertex": _view(v.source_vertex, np.uint32, n),
            "edge_offset": _view(v.edge_offset, np.uint32, n),
            "edge_count": _view(v.edge_count, np.uint8, n),
            "neighbor": _view(v.neighbor, np.uint32, d),
            "edge": _view(v.edge, np.uint32, d),
            "corner": _view(v.corner, np.uint32, d),
            "normal_east": _view(v.normal_east, np.float32, d),
            "normal_north": _view(v.normal_north, np.float32, d),
            "edge_first": _view(v.edge_first, np.uint32, e),
            "edge_second": _view(v.edge_second, np.uint32, e),
            "edge_length_m": _view(v.edge_length_m, np.float64, e),
            "edge_distance_m": _view(v.edge_distance_m, np.float64, e),
            "corner_unit": _view(v.corner_unit, np.float64, 3 * k).reshape(k, 3),
            "graph_weight": _view(v.graph_weight, np.float64, d),
            "graph_weight_sum": _view(v.graph_weight_sum, np.float64, n),
            "graph_area_m2": self._graph_area(),
        }

    def _graph_area(self) -> np.ndarray:
        g = capi.GraphView()
        _raise(capi.load().psgb_planet_graph_view(self._h, C.byref(g)))
        return _view(g.area_m2, np.float64, self.cell_count)

    def group_of_cell(self) -> np.ndarray:
        """Agglomerated planets: the transport node of every fine cell."""
        if not self.agglomerated:
            raise ValueError("not an agglomerated planet")
        out = np.empty(self.fine_cell_count, dtype=np.uint32)
        _raise(capi.load().psgb_planet_group_of_cell(self._h, _ptr(out)))
        return out

    @property
    def tuning(self) -> dict:
        """The per-level settings of this planet's own solves (transport_step,
        transport_step_multi, GraphMultigrid.precondition, solve_newton_system)."""
        t = capi.Tuning()
        _raise(capi.load().psgb_planet_get_tuning(self._h, C.byref(t)))
        return _tuning_dict(t)

    def set_tuning(self, tuning: dict | None) -> None:
        """Per-level settings for this planet's own solves: a one-planet Batch's tuning of
        this planet carries over bit for bit; None returns to the options' sweeps."""
        _raise(capi.load().psgb_planet_set_tuning(self._h, None if tuning is None else C.byref(_tuning_struct(tuning))))

    def hierarchy_level(self, level: int) -> dict[str, np.ndarray]:
        sizes = (C.c_uint64 * 4)()
        ptrs = [C.c_void_p() for _ in range(4)]
        _raise(capi.load().psgb_planet_hierarchy_level(self._h, level, sizes, *[C.byref(p) for p in ptrs]))
        rows, nnz, na, nt = (int(s) for s in sizes)
        return {
            "offset": _view(ptrs[0].value or 0, np.uint32, rows + 1),
            "column": _view(ptrs[1].value or 0, np.uint32, nnz),
            "aggregate": _view(ptrs[2].value or 0, np.uint32, na) if na else np.empty(0, np.uint32),
            "target": _view(ptrs[3].value or 0, np.int64, nt) if nt else np.empty(0, np.int64),
        }

    def substep_mean_insolation_gpu(self, substep: int = 0, out=None):
        """The sub-step-mean insolation computed on the GPU (numpy out, or a float32
        CUDA tensor `out` filled in place on the current stream)."""
        if out is None:
            out = np.empty(self.cell_count, dtype=np.float32)
        mem, st = _memory_of(out)
        _raise(capi.load().psgb_substep_mean_insolation_gpu(self._h, C.c_int64(substep), _ptr(out), mem, st))
        return out

    def substep_mean_insolation(self, substep: int = 0) -> np.ndarray:
        out = np.empty(self.cell_count, dtype=np.float32)
        _raise(capi.load().psgb_substep_mean_insolation(self._h, C.c_int64(substep), _ptr(out)))
        return out


def make_icosphere(subdivision: int, radius_m: float) -> PlanetMesh:
    return PlanetMesh(subdivision, radius_m)


def agglomerated_transport_graph(subdivision: int, radius_m: float) -> PlanetMesh:
    """The transport of a level-`subdivision` planet one mesh level coarser, as the
    reference's production path runs it (agglomerated_transport_graph, heat_transport.cpp:
    456-539): every fine cell joins the nearest cell of the coarser mesh, nodes take their
    fine cells' summed areas. The returned planet's cells are those nodes; its
    group_of_cell() maps fine cells onto them."""
    return PlanetMesh(subdivision, radius_m, agglomerated=True)


@dataclass
class TransportGraph:
    """CSR transport graph of a mesh (heat_transport.hpp:27-36)."""

    mesh: PlanetMesh
    area_m2: np.ndarray
    offset: np.ndarray
    neighbour: np.ndarray
    weight: np.ndarray
    weight_sum: np.ndarray

    def size(self) -> int:
        return len(self.area_m2)


def mesh_transport_graph(mesh: PlanetMesh) -> TransportGraph:
    a = mesh.arrays()
    offset = np.append(a["edge_offset"].astype(np.uint64), np.uint64(mesh.directed_edge_count))
    return TransportGraph(mesh, a["graph_area_m2"], offset, a["neighbor"].astype(np.uint64), a["graph_weight"],
                          a["graph_weight_sum"])


# ---- finite-volume operators --------------------------------------------------------

def laplacian(mesh: PlanetMesh, scalar):
    out = _empty_like(scalar, (mesh.cell_count,))
    mem, st = _memory_of(scalar, out)
    _raise(capi.load().psgb_laplacian(mesh.handle, _dtype_code(scalar), _ptr(scalar), _ptr(out), mem, st))
    return out


def gradient(mesh: PlanetMesh, scalar):
    east = _empty_like(scalar, (mesh.cell_count,))
    north = _empty_like(scalar, (mesh.cell_count,))
    mem, st = _memory_of(scalar, east)
    _raise(capi.load().psgb_gradient(mesh.handle, _dtype_code(scalar), _ptr(scalar), _ptr(east), _ptr(north),
                                     mem, st))
    return east, north


def divergence(mesh: PlanetMesh, edge_flux):
    out = _empty_like(edge_flux, (mesh.cell_count,))
    mem, st = _memory_of(edge_flux, out)
    _raise(capi.load().psgb_divergence(mesh.handle, _dtype_code(edge_flux), _ptr(edge_flux), _ptr(out), mem, st))
    return out


def diffusion_source(mesh: PlanetMesh, conductance_W_K: float, temperature_K):
    out = _empty_like(temperature_K, (mesh.cell_count,))
    mem, st = _memory_of(temperature_K, out)
    _raise(capi.load().psgb_diffusion_source(mesh.handle, C.c_double(conductance_W_K), _ptr(temperature_K),
                                             _ptr(out), mem, st))
    return out


def group_mean(planet: PlanetMesh, fine_a, fine_b=None):
    """Agglomerated planets: the nodes' area-weighted means of fine-cell fields, as the
    production response forms a group's air temperature and slope (surface_energy.cpp:
    1285-1296). Returns one array, or two when `fine_b` is given."""
    if len(fine_a) != planet.fine_cell_count or (fine_b is not None and len(fine_b) != planet.fine_cell_count):
        raise ValueError("fine-cell field does not match the planet's fine mesh")
    out_a = _empty_like(fine_a, (planet.cell_count,))
    out_b = None if fine_b is None else _empty_like(fine_b, (planet.cell_count,))
    mem, st = _memory_of(fine_a, fine_b, out_a)
    nil = C.c_void_p(None)
    _raise(capi.load().psgb_group_mean(planet.handle, _ptr(fine_a), nil if fine_b is None else _ptr(fine_b),
                                       _ptr(out_a), nil if out_b is None else _ptr(out_b), mem, st))
    return out_a if fine_b is None else (out_a, out_b)


def group_scatter(planet: PlanetMesh, node_value):
    """Agglomerated planets: every fine cell takes its node's value (the transport
    applied per fine cell, surface_energy.cpp:1583, 1595)."""
    if len(node_value) != planet.cell_count:
        raise ValueError("node field does not match the planet's transport graph")
    out = _empty_like(node_value, (planet.fine_cell_count,))
    mem, st = _memory_of(node_value, out)
    _raise(capi.load().psgb_group_scatter(planet.handle, _ptr(node_value), _ptr(out), mem, st))
    return out


# ---- multigrid and solves -------------------------------------------------------------

class GraphMultigrid:
    """The transport's aggregation-multigrid V-cycle (heat_transport.hpp:60-76) on the GPU."""

    def __init__(self, mesh: PlanetMesh):
        self.mesh = mesh

    def set_matrix(self, diagonal, off_diagonal) -> None:
        if len(diagonal) != self.mesh.cell_count or len(off_diagonal) != self.mesh.directed_edge_count:
            raise ValueError("multigrid matrix does not match the graph")
        mem, st = _memory_of(diagonal, off_diagonal)
        _raise(capi.load().psgb_multigrid_set_matrix(self.mesh.handle, _ptr(diagonal), _ptr(off_diagonal), mem, st))

    def level_values(self, level: int):
        """(diagonal, off-diagonals in CSR order) of a level as held on the GPU."""
        lv = self.mesh.hierarchy_level(level)
        rows = len(lv["offset"]) - 1
        d, o = np.empty(rows), np.empty(len(lv["column"]))
        _raise(capi.load().psgb_multigrid_level_values(self.mesh.handle, level, _ptr(d), _ptr(o)))
        return d, o

    def precondition(self, rhs):
        out = _empty_like(rhs, (self.mesh.cell_count,))
        mem, st = _memory_of(rhs, out)
        _raise(capi.load().psgb_multigrid_precondition(self.mesh.handle, _dtype_code(rhs), _ptr(rhs), _ptr(out),
                                                       mem, st))
        return out


def solve_options(**kw) -> capi.SolveOptions:
    o = capi.default_options()
    names = {
        "precision": {"fp64": capi.PRECISION_FP64, "mixed": capi.PRECISION_MIXED},
        "method": {"pcg": capi.METHOD_PCG, "bicgstab": capi.METHOD_BICGSTAB},
        "schedule": {"auto": capi.SCHEDULE_AUTO, "kernels": capi.SCHEDULE_KERNELS,
                     "persistent": capi.SCHEDULE_PERSISTENT},
    }
    for k, v in kw.items():
        if k in names and isinstance(v, str):
            v = names[k][v]
        setattr(o, k, v)
    return o


@dataclass
class SolveResult:
    status: int
    refinements: int
    iterations: int
    relative_residual: float


def solve_newton_system(mesh: PlanetMesh, conductance_W_K: float, slope, rhs, x0=None, **options):
    """(A/s) x + K L x = rhs on the mesh graph (the reference's solve_newton_system)."""
    x = np.zeros(mesh.cell_count) if x0 is None else (x0.clone() if _is_torch(x0) else np.array(x0, dtype=np.float64))
    rep = capi.SolveReport()
    o = solve_options(**options)
    mem, st = _memory_of(slope, rhs, x)
    code = capi.load().psgb_solve_newton_system(mesh.handle, C.byref(o), C.c_double(conductance_W_K), _ptr(slope),
                                                _ptr(rhs), _ptr(x), C.byref(rep), mem, st)
    if code not in (capi.OK, capi.ERR_NOT_CONVERGED, capi.ERR_BREAKDOWN):
        _raise(code)
    return x, SolveResult(rep.status, rep.refinements, rep.iterations, rep.relative_residual)


@dataclass
class ImplicitTransportResult:
    """ImplicitTransportResult (heat_transport.hpp:110-119)."""
    source_W_m2: np.ndarray
    mean_K: np.ndarray
    consistency_residual_W_m2: float
    newton_iterations: int
    cg_iterations: int
    sum_W: float
    absolute_sum_W: float
    dissipation_W_K: float


def transport_settings(**kw) -> capi.TransportSettings:
    s = capi.TransportSettings()
    capi.load().psgb_transport_settings_default(C.byref(s))
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def solve_implicit_transport(mesh: PlanetMesh, conductance_W_K: float, source_floor_W_m2, response,
                             settings: dict | None = None, latent_W_m2=None, **options) -> ImplicitTransportResult:
    """solve_implicit_transport (heat_transport.cpp:595-772) with a general response.

    `response` is either
    - a host callable `response(source) -> (mean_K, slope_K_m2_W)` on numpy arrays of
      the cells (copied across once per evaluation), or
    - a device response: a `QuarticResponse`, or `device=True` with a callable
      `response(cells, source, mean, slope, stream)` on device pointers;
    the Newton iterate, the Laplacians and the linear Newton systems (with `options`:
    precision, method, sweeps, schedule) stay on the GPU either way. The floor, latent
    heat and results are numpy arrays, or CUDA tensors on a device response."""
    n = mesh.cell_count
    if isinstance(response, QuarticResponse) or options.pop("device", False):
        floor = source_floor_W_m2 if _is_torch(source_floor_W_m2) else np.ascontiguousarray(source_floor_W_m2,
                                                                                          dtype=np.float64)
        latent = latent_W_m2
        if latent is not None and not _is_torch(latent):
            latent = np.ascontiguousarray(latent, dtype=np.float64)
        if latent is not None and _is_torch(latent) != _is_torch(floor):
            raise ValueError("pass the floor and the latent heat both as numpy arrays or both as CUDA tensors")
        return _solve_device(mesh, conductance_W_K, floor, response, transport_settings(**(settings or {})),
                             solve_options(**options), latent)
    floor = np.ascontiguousarray(source_floor_W_m2, dtype=np.float64)
    latent = None if latent_W_m2 is None else np.ascontiguousarray(latent_W_m2, dtype=np.float64)
    error: list[BaseException] = []

    def trampoline(_user, cells, source, mean, slope):
        try:
            h = np.ctypeslib.as_array(source, shape=(cells,))
            m, s = response(h.copy())
            np.ctypeslib.as_array(mean, shape=(cells,))[:] = m
            np.ctypeslib.as_array(slope, shape=(cells,))[:] = s
            return 0
        except BaseException as exc:   # reported after the call returns
            error.append(exc)
            return 1

    callback = capi.TransportResponse(trampoline)
    source_out = np.empty(n)
    mean_out = np.empty(n)
    res = capi.TransportResult()
    st = transport_settings(**(settings or {}))
    o = solve_options(**options)
    code = capi.load().psgb_solve_implicit_transport(
        mesh.handle, C.c_double(conductance_W_K), _ptr(floor), callback, None, C.byref(st), C.byref(o),
        _ptr(latent) if latent is not None else None, _ptr(source_out), _ptr(mean_out), C.byref(res))
    if error:
        raise error[0]
    _raise(code)
    return ImplicitTransportResult(source_out, mean_out, res.consistency_residual_W_m2, res.newton_iterations,
                                   res.cg_iterations, res.sum_W, res.absolute_sum_W, res.dissipation_W_K)


STEFAN_BOLTZMANN_W_M2_K4 = 5.670374419e-8


@dataclass
class QuarticResponse:
    """The quartic column response of the reference's transport test (test_heat_transport.
    cpp:30-76) evaluated on the GPU: per cell the root of a x + r x^4 = b + h, cells whose
    index is a multiple of `hold_stride` held at `hold_K` when they would pass it. With
    `fine=True` (an agglomerated planet) `b` is per FINE cell: each fine cell answers at
    its node's source and the nodes take the area-weighted means, as the production step
    forms a group's response (surface_energy.cpp:1240-1296)."""

    a: float
    b: object
    radiative: float = 0.75 * 0.97 * STEFAN_BOLTZMANN_W_M2_K4
    hold_stride: int = 7
    hold_K: float = 273.15
    fine: bool = False


def quartic_response(q: QuarticResponse, source):
    """The per-cell quartic response on the GPU: (T, dT/dh) for sources h (CUDA tensors)."""
    import torch

    if q.fine:
        raise ValueError("the fine-cell response runs inside a solve on an agglomerated planet")
    h = torch.as_tensor(source, dtype=torch.float64, device="cuda").contiguous()
    b = torch.as_tensor(q.b, dtype=torch.float64, device="cuda").contiguous()
    if b.numel() != h.numel():
        raise ValueError("the quartic's b does not match the sources")
    mean, slope = torch.empty_like(h), torch.empty_like(h)
    cq = capi.QuarticResponse(q.a, q.radiative, b.data_ptr(), q.hold_stride, q.hold_K, None, None)
    _raise(capi.load().psgb_quartic_device_response(C.byref(cq), C.c_uint64(h.numel()), C.c_void_p(h.data_ptr()),
                                                    C.c_void_p(mean.data_ptr()), C.c_void_p(slope.data_ptr()),
                                                    C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return mean, slope


def _solve_device(mesh: PlanetMesh, conductance_W_K: float, floor, response, st, o, latent):
    """The device-resident Newton solve; `response` a QuarticResponse or a callable
    (cells, source, mean, slope, stream) on device pointers."""
    import torch

    n = mesh.cell_count
    keep = []
    if isinstance(response, QuarticResponse):
        cells = mesh.fine_cell_count if response.fine else n
        if response.fine and not mesh.agglomerated:
            raise ValueError("a fine-cell response needs an agglomerated planet")
        b = torch.as_tensor(response.b, dtype=torch.float64, device="cuda").contiguous()
        if b.numel() != cells:
            raise ValueError("the quartic's b does not match the cells")
        scratch = torch.empty(2 * cells if response.fine else 1, dtype=torch.float64, device="cuda")
        q = capi.QuarticResponse(response.a, response.radiative, b.data_ptr(), response.hold_stride, response.hold_K,
                                 mesh.handle.value if response.fine else None, scratch.data_ptr())
        keep += [b, scratch, q]
        fn = C.cast(capi.load().psgb_quartic_device_response, C.c_void_p)
        user = C.cast(C.pointer(q), C.c_void_p)
    else:
        error: list[BaseException] = []

        def trampoline(_user, cells, source, mean, slope, stream):
            try:
                response(int(cells), source, mean, slope, stream)
                return 0
            except BaseException as exc:   # reported after the call returns
                error.append(exc)
                return 1

        cb = capi.DeviceResponse(trampoline)
        keep += [cb, error]
        fn = C.cast(cb, C.c_void_p)
        user = None
    on_device = _is_torch(floor)
    if on_device:
        source_out = torch.empty(n, dtype=torch.float64, device=floor.device)
        mean_out = torch.empty(n, dtype=torch.float64, device=floor.device)
        mem, stream = capi.MEMORY_DEVICE, C.c_void_p(torch.cuda.current_stream().cuda_stream)
    else:
        source_out, mean_out = np.empty(n), np.empty(n)
        mem, stream = capi.MEMORY_HOST, C.c_void_p(torch.cuda.current_stream().cuda_stream)
    res = capi.TransportResult()
    code = capi.load().psgb_solve_implicit_transport_device(
        mesh.handle, C.c_double(conductance_W_K), _ptr(floor), fn, user, C.byref(st), C.byref(o),
        _ptr(latent) if latent is not None else None, _ptr(source_out), _ptr(mean_out), C.byref(res), mem, stream)
    if not isinstance(response, QuarticResponse) and keep[1]:
        raise keep[1][0]
    _raise(code)
    return ImplicitTransportResult(source_out, mean_out, res.consistency_residual_W_m2, res.newton_iterations,
                                   res.cg_iterations, res.sum_W, res.absolute_sum_W, res.dissipation_W_K)


@dataclass
class StepResult:
    status: int
    refinements: int
    iterations: int
    relative_residual: float
    sum_W: float
    absolute_sum_W: float
    dissipation_W_K: float
    closure: float


def _step_result(r: capi.StepReport) -> StepResult:
    return StepResult(r.solve.status, r.solve.refinements, r.solve.iterations, r.solve.relative_residual, r.sum_W,
                      r.absolute_sum_W, r.dissipation_W_K, r.closure)


def step_params(heat_capacity_J_m2_K: float, dt_s: float, conductance_W_K: float = 0.0,
                edge_conductance=None) -> capi.StepParams:
    """`edge_conductance`: None (uniform K), an array per undirected edge, or "stored"
    (the batch's stored array, Batch.set_edge_conductance)."""
    p = capi.StepParams(heat_capacity_J_m2_K, dt_s, conductance_W_K, None, 0)
    if isinstance(edge_conductance, str):
        if edge_conductance != "stored":
            raise ValueError("edge_conductance must be an array, None or 'stored'")
        p.edge_conductance_stored = 1
    elif edge_conductance is not None:
        arr = np.ascontiguousarray(edge_conductance, dtype=np.float64)
        p.edge_conductance = arr.ctypes.data
        p._keep = arr  # keep the host array alive with the struct
    return p


def transport_step(mesh: PlanetMesh, t0_K, source_W_m2, heat_capacity_J_m2_K: float, dt_s: float,
                   conductance_W_K: float = 0.0, edge_conductance=None, **options):
    """One implicit heat-transport sub-step with the linear column response."""
    t_new = _empty_like(t0_K, (mesh.cell_count,))
    h = _empty_like(t0_K, (mesh.cell_count,))
    params = step_params(heat_capacity_J_m2_K, dt_s, conductance_W_K, edge_conductance)
    o = solve_options(**options)
    rep = capi.StepReport()
    mem, st = _memory_of(t0_K, source_W_m2, t_new, h)
    code = capi.load().psgb_transport_step(mesh.handle, C.byref(params), C.byref(o), _ptr(t0_K), _ptr(source_W_m2),
                                           _ptr(t_new), _ptr(h), C.byref(rep), mem, st)
    if code not in (capi.OK, capi.ERR_NOT_CONVERGED, capi.ERR_BREAKDOWN):
        _raise(code)
    return t_new, h, _step_result(rep)


def transport_step_multi(mesh: PlanetMesh, t0_K, sources_W_m2, heat_capacity_J_m2_K: float, dt_s: float,
                         conductance_W_K: float = 0.0, edge_conductance=None, transport=False, **options):
    """Up to 32 sub-steps of one planet with the same parameters, solved as one block
    (psgb_transport_step_multi): `t0_K` one state for every sub-step or a list of them,
    `sources_W_m2` a list of sources (numpy or CUDA tensors). Returns the new states (a
    list), the transports (a list, or None unless `transport`) and the reports; each
    sub-step's result equals transport_step of that sub-step alone bit for bit."""
    count = len(sources_W_m2)
    if not 1 <= count <= 32:
        raise ValueError("a block holds 1 to 32 sub-steps")
    t0s = list(t0_K) if isinstance(t0_K, (list, tuple)) else [t0_K] * count
    if len(t0s) != count:
        raise ValueError("one initial state, or one per sub-step")
    outs = [_empty_like(t0s[j], (mesh.cell_count,)) for j in range(count)]
    hs = [_empty_like(t0s[j], (mesh.cell_count,)) for j in range(count)] if transport else None
    params = step_params(heat_capacity_J_m2_K, dt_s, conductance_W_K, edge_conductance)
    o = solve_options(**options)
    mem, st = _memory_of(*t0s, *sources_W_m2, *outs)
    arrs = lambda xs: (C.c_void_p * count)(*[_ptr(x).value for x in xs])
    reps = (capi.StepReport * count)()
    code = capi.load().psgb_transport_step_multi(mesh.handle, C.byref(params), C.byref(o), count, arrs(t0s),
                                                 arrs(sources_W_m2), arrs(outs), arrs(hs) if hs else None, reps,
                                                 mem, st)
    if code not in (capi.OK, capi.ERR_NOT_CONVERGED, capi.ERR_BREAKDOWN):
        _raise(code)
    return outs, hs, [_step_result(r) for r in reps]


def transport_step_noalloc(mesh: PlanetMesh, t0_K, source_W_m2, heat_capacity_J_m2_K: float, dt_s: float,
                           conductance_W_K: float = 0.0, edge_conductance=None, **options):
    """The transport step through the entry point that allocates nothing (CUDA tensors
    only; the solver workspace is the library's static device scratch)."""
    if not (_is_torch(t0_K) and _is_torch(source_W_m2)):
        raise ValueError("the no-allocation step takes CUDA tensors")
    import torch

    n = mesh.cell_count
    current = torch.device("cuda", torch.cuda.current_device())
    for name, t in (("t0_K", t0_K), ("source_W_m2", source_W_m2)):
        if t.dtype != torch.float64 or t.numel() != n or not t.is_contiguous():
            raise ValueError(f"{name} must be a contiguous float64 tensor of {n} cells "
                             f"(got {t.dtype}, {t.numel()} elements)")
        if t.device != current:
            raise ValueError(f"{name} is on {t.device}; the no-allocation step runs on the current device {current}")
    if isinstance(edge_conductance, str):
        raise ValueError("the no-allocation step has no stored per-edge conductance: pass the array")
    t_new = torch.empty(n, dtype=torch.float64, device=current)
    h = torch.empty(n, dtype=torch.float64, device=current)
    params = step_params(heat_capacity_J_m2_K, dt_s, conductance_W_K, edge_conductance)
    o = solve_options(**options)
    rep = capi.StepReport()
    code = capi.load().psgb_transport_step_noalloc(mesh.handle, C.byref(params), C.byref(o), _ptr(t0_K),
                                                   _ptr(source_W_m2), _ptr(t_new), _ptr(h), C.byref(rep),
                                                   C.c_void_p(torch.cuda.current_stream().cuda_stream))
    if code not in (capi.OK, capi.ERR_NOT_CONVERGED, capi.ERR_BREAKDOWN):
        _raise(code)
    return t_new, h, _step_result(rep)


def _tuning_dict(t) -> dict:
    n = int(t.levels)
    return {"levels": n, "pre_sweeps": list(t.pre_sweeps[:n]), "post_sweeps": list(t.post_sweeps[:n]),
            "stencil_tiles": list(t.stencil_tiles[:n]), "vector_tiles": list(t.vector_tiles[:n]),
            "jacobi_omega": float(t.jacobi_omega), "tuned_solve_ms": float(t.tuned_solve_ms),
            "default_solve_ms": float(t.default_solve_ms), "trial_solves": int(t.trial_solves),
            "coarse_tail_level": int(t.coarse_tail_level), "block_sweeps": list(t.block_sweeps[:n]),
            "coarse_tail_single": int(t.coarse_tail_single), "coarse_tail_blocks": int(t.coarse_tail_blocks),
            "coarse_tail_cluster": int(t.coarse_tail_cluster), "coarse_correction": float(t.coarse_correction)}


def _tuning_struct(tuning: dict) -> capi.Tuning:
    t = capi.Tuning()
    t.levels = len(tuning["pre_sweeps"])
    for k in ("pre_sweeps", "post_sweeps", "stencil_tiles", "vector_tiles", "block_sweeps"):
        arr = getattr(t, k)
        for l, v in enumerate(tuning.get(k, [1] * t.levels)):
            arr[l] = int(v)
    t.jacobi_omega = float(tuning["jacobi_omega"])
    t.coarse_tail_level = int(tuning.get("coarse_tail_level", 0))
    t.coarse_tail_single = int(tuning.get("coarse_tail_single", 0))
    t.coarse_tail_cluster = int(tuning.get("coarse_tail_cluster", 0))
    t.coarse_correction = float(tuning.get("coarse_correction", 1.0))
    return t


class Batch:
    """Many planets of uneven levels in one concatenated layout, solved together."""

    def __init__(self, meshes: list[PlanetMesh]):
        self.meshes = list(meshes)
        arr = (C.c_void_p * len(meshes))(*[m.handle.value for m in meshes])
        h = C.c_void_p()
        _raise(capi.load().psgb_batch_create(arr, len(meshes), C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            capi.load().psgb_batch_destroy(h)
            self._h = None

    def device_bytes(self) -> int:
        return int(capi.load().psgb_batch_device_bytes(self._h))

    def _params(self, heat_capacity, dt, conductance, edge_conductance):
        n = len(self.meshes)
        params = (capi.StepParams * n)()
        params._keep = []   # the structs own the host arrays they point at
        for i in range(n):
            p = step_params(heat_capacity[i] if np.ndim(heat_capacity) else heat_capacity,
                            dt[i] if np.ndim(dt) else dt,
                            (conductance[i] if np.ndim(conductance) else conductance) if conductance is not None else 0.0,
                            edge_conductance if isinstance(edge_conductance, str)
                            else (edge_conductance[i] if edge_conductance is not None else None))
            params._keep.append(p)
            params[i] = p
        return params

    def set_edge_conductance(self, edge_conductance) -> None:
        """Store per-edge conductances with the batch (one array per planet, None clears);
        steps then pass edge_conductance="stored"."""
        n = len(self.meshes)
        keep = [None if e is None else np.ascontiguousarray(e, dtype=np.float64) for e in edge_conductance]
        arr = (C.c_void_p * n)(*[None if e is None else e.ctypes.data for e in keep])
        _raise(capi.load().psgb_batch_set_edge_conductance(self._h, arr))

    def set_reassembly(self, every_step: bool) -> None:
        """True: every step assembles the matrix, its Galerkin coarse values and the coarsest
        inverses again on the device (as the reference does per call); False (default):
        the assembled matrix is reused while C, dt and the conductances are unchanged."""
        _raise(capi.load().psgb_batch_set_reassembly(self._h, 1 if every_step else 0))

    def set_priority(self, high: bool) -> None:
        """True: this batch's solves run on a highest-priority stream (scheduled first where
        batches stepped side by side compete); False (default): normal priority."""
        _raise(capi.load().psgb_batch_set_priority(self._h, 1 if high else 0))

    def autotune(self, t0, sources, heat_capacity, dt, conductance=None, edge_conductance=None, **options) -> dict:
        """Pick per-level launch shapes and sweeps by timing trial solves of this sub-step;
        the batch keeps them (see `tuning`). Nothing is written back."""
        n = len(self.meshes)
        params = self._params(heat_capacity, dt, conductance, edge_conductance)
        mem, st = _memory_of(*t0, *sources)
        arrs = lambda xs: (C.c_void_p * n)(*[_ptr(x).value for x in xs])
        o = solve_options(**options)
        t = capi.Tuning()
        _raise(capi.load().psgb_batch_autotune(self._h, params, C.byref(o), arrs(t0), arrs(sources), mem, st,
                                               C.byref(t)))
        return _tuning_dict(t)

    @property
    def tuning(self) -> dict:
        t = capi.Tuning()
        _raise(capi.load().psgb_batch_get_tuning(self._h, C.byref(t)))
        return _tuning_dict(t)

    def set_tuning(self, tuning: dict | None) -> None:
        """Apply per-level settings (a dict from `autotune`/`tuning`); None clears them."""
        _raise(capi.load().psgb_batch_set_tuning(self._h, None if tuning is None else C.byref(_tuning_struct(tuning))))

    def transport_step(self, t0, sources, heat_capacity, dt, conductance=None, edge_conductance=None,
                       out=None, transport_out=None, active=None, **options):
        """One sub-step of every planet (or of the planets with active[i] true)."""
        n = len(self.meshes)
        params = self._params(heat_capacity, dt, conductance, edge_conductance)
        on = [True] * n if active is None else [bool(a) for a in active]
        if out is None:
            out = [_empty_like(t0[i], (m.cell_count,)) if on[i] else None for i, m in enumerate(self.meshes)]
        mem, st = _memory_of(*[x for x in (*t0, *sources, *out) if x is not None])
        arrs = lambda xs: (C.c_void_p * n)(*[_ptr(x).value if x is not None else None for x in xs])
        h_arr = arrs(transport_out) if transport_out is not None else None
        o = solve_options(**options)
        reps = (capi.StepReport * n)()
        if active is None:
            code = capi.load().psgb_batch_transport_step(self._h, params, C.byref(o), arrs(t0), arrs(sources),
                                                         arrs(out), h_arr, reps, mem, st)
        else:
            mask = (C.c_uint8 * n)(*[1 if a else 0 for a in on])
            code = capi.load().psgb_batch_transport_step_masked(self._h, mask, params, C.byref(o), arrs(t0),
                                                                arrs(sources), arrs(out), h_arr, reps, mem, st)
        if code not in (capi.OK, capi.ERR_NOT_CONVERGED, capi.ERR_BREAKDOWN):
            _raise(code)
        return out, [_step_result(r) for r in reps]


class TunedSolo:
    """Planets stepped one per call, each in a one-planet batch of its own - the drop-in
    solve of a single planet - with the launch shapes and damped-Jacobi sweeps autotuned
    once per mesh level (on the first planet of the level stepped) and reused for every
    other planet of that level. The plain one-planet-at-a-time FP64 comparator of the
    benchmark and of the serving comparator, tuned as the batched solves are.

    A planet's per-edge conductance is stored with its batch on its first step; later
    steps of the planet use that array."""

    def __init__(self, precision: str = "fp64", autotune: bool = True, **solver):
        self.options = dict(solver, precision=precision)
        self.autotune = autotune
        self._batches: dict[int, tuple] = {}
        self.tunings: dict[tuple, dict] = {}

    def batch_of(self, mesh: PlanetMesh, t0, source, heat_capacity, dt, conductance, edge_conductance=None):
        key = id(mesh)
        entry = self._batches.get(key)
        if entry is None:
            b = Batch([mesh])
            stored = None
            if edge_conductance is not None:
                b.set_edge_conductance([edge_conductance])
                stored = "stored"
            entry = (mesh, b, stored)
            self._batches[key] = entry
            if self.autotune:
                level = (mesh.subdivision, mesh.agglomerated)
                if level not in self.tunings:
                    self.tunings[level] = b.autotune([t0], [source], [heat_capacity], [dt], conductance=[conductance],
                                                     edge_conductance=stored, **self.options)
                else:
                    b.set_tuning(self.tunings[level])
        return entry[1], entry[2]

    def step(self, mesh: PlanetMesh, t0, source, heat_capacity, dt, conductance, edge_conductance=None,
             out=None, transport_out=None):
        """One sub-step of one planet: (t_new, report)."""
        b, stored = self.batch_of(mesh, t0, source, heat_capacity, dt, conductance, edge_conductance)
        outs, reps = b.transport_step([t0], [source], [heat_capacity], [dt], conductance=[conductance],
                                      edge_conductance=stored, out=None if out is None else [out],
                                      transport_out=None if transport_out is None else [transport_out],
                                      **self.options)
        return outs[0], reps[0]


def default_lanes(meshes: list[PlanetMesh], top_lane_planets: int = 4) -> list[list[int]]:
    """The highest level's planets apart from the others when a mix spans three or more
    levels (they need the most Krylov iterations), in lanes of at most `top_lane_planets`
    (each lane's chain of latency-bound launches then runs beside the others: on the
    64-planet mix two lanes of four L7 planets step in 11.5 ms where one lane of eight
    takes 12.6); otherwise one lane."""
    levels = [m.subdivision for m in meshes]
    if len(set(levels)) < 3:
        return [list(range(len(meshes)))]
    top = max(levels)
    tops = [i for i, l in enumerate(levels) if l == top]
    k = -(-len(tops) // max(1, top_lane_planets))
    return [[i for i, l in enumerate(levels) if l != top]] + [tops[j::k] for j in range(k)]


class LaneBatch:
    """Planets in several batches ("lanes") solved side by side on one GPU, one host thread
    per lane.

    A batch solves its planets in lockstep: every Krylov iteration runs every level's
    launches until its slowest planet converges, and the coarse levels' launches cost their
    latency however few planets are still running. Planets that converge much more slowly
    than the rest therefore run better in a lane of their own, concurrently with the
    others. `lanes`: lists of planet indices covering every planet once (default:
    `default_lanes`). The same calls as `Batch`, with per-lane tunings."""

    def __init__(self, meshes: list[PlanetMesh], lanes: list[list[int]] | None = None):
        from concurrent.futures import ThreadPoolExecutor

        self.meshes = list(meshes)
        self.lanes = [list(l) for l in (lanes if lanes is not None else default_lanes(self.meshes))]
        if sorted(i for l in self.lanes for i in l) != list(range(len(self.meshes))) or any(not l for l in self.lanes):
            raise ValueError("lanes must cover every planet exactly once")
        self.batches = [Batch([self.meshes[i] for i in lane]) for lane in self.lanes]
        self._pool = ThreadPoolExecutor(max_workers=len(self.lanes) - 1) if len(self.lanes) > 1 else None
        self.concurrent = True    # False: the lanes one after another (e.g. while a profile records)
        # the lanes of the mix's highest level set the step's pace: their kernels go first
        # where the lanes compete for the GPU (64-planet mix: 11.1 -> 10.7 ms a step)
        levels = [max(self.meshes[i].subdivision for i in lane) for lane in self.lanes]
        if len(set(levels)) > 1:
            for b, level in zip(self.batches, levels):
                if level == max(levels):
                    b.set_priority(True)

    def close(self) -> None:
        if getattr(self, "_pool", None) is not None:
            self._pool.shutdown()
            self._pool = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()

    def _pick(self, value, lane):
        """A per-planet list restricted to a lane; scalars, None and "stored" pass through."""
        if value is None or isinstance(value, str):
            return value
        if isinstance(value, (list, tuple)) or np.ndim(value) > 0:
            return [value[i] for i in lane]
        return value

    def _run(self, fn):
        """fn(k) for every lane k, lanes 1.. on worker threads, lane 0 here."""
        if self._pool is None or not self.concurrent:
            return [fn(k) for k in range(len(self.lanes))]
        futures = [self._pool.submit(fn, k) for k in range(1, len(self.lanes))]
        first = fn(0)
        return [first] + [f.result() for f in futures]

    def set_edge_conductance(self, edge_conductance) -> None:
        for lane, b in zip(self.lanes, self.batches):
            b.set_edge_conductance(self._pick(edge_conductance, lane))

    def autotune(self, t0, sources, heat_capacity, dt, conductance=None, edge_conductance=None, **options) -> list:
        """Each lane tuned on its own (one after another, so the trial timings are clean)."""
        return [b.autotune(self._pick(t0, lane), self._pick(sources, lane), self._pick(heat_capacity, lane),
                           self._pick(dt, lane), conductance=self._pick(conductance, lane),
                           edge_conductance=self._pick(edge_conductance, lane), **options)
                for lane, b in zip(self.lanes, self.batches)]

    @property
    def tuning(self) -> list:
        return [b.tuning for b in self.batches]

    def set_reassembly(self, every_step: bool) -> None:
        for b in self.batches:
            b.set_reassembly(every_step)

    def set_tuning(self, tunings) -> None:
        for b, t in zip(self.batches, tunings if tunings is not None else [None] * len(self.batches)):
            b.set_tuning(t)

    def transport_step(self, t0, sources, heat_capacity, dt, conductance=None, edge_conductance=None,
                       out=None, transport_out=None, active=None, **options):
        """One sub-step of every planet, the lanes concurrently; results in planet order."""
        n = len(self.meshes)

        def lane_step(k):
            lane = self.lanes[k]
            return self.batches[k].transport_step(
                self._pick(t0, lane), self._pick(sources, lane), self._pick(heat_capacity, lane),
                self._pick(dt, lane), conductance=self._pick(conductance, lane),
                edge_conductance=self._pick(edge_conductance, lane), out=self._pick(out, lane),
                transport_out=self._pick(transport_out, lane), active=self._pick(active, lane), **options)

        results = self._run(lane_step)
        outs, reps = [None] * n, [None] * n
        for lane, (o, r) in zip(self.lanes, results):
            for j, i in enumerate(lane):
                outs[i], reps[i] = o[j], r[j]
        return outs, reps


# ---- column radiation ----------------------------------------------------------------

def column_constants(**kw) -> capi.ColumnConstants:
    k = capi.ColumnConstants()
    for name, value in kw.items():
        setattr(k, name, value)
    return k


def column_radiation(constants: capi.ColumnConstants, temperature_K, humidity, cloud_water, surface_temperature_K,
                     surface_pressure_Pa):
    """Layer-major [layers, cells] inputs; returns emissivity, absorbed, fraction,
    reflectance ([layers, cells]) and scalars [5, cells]."""
    layers, cells = temperature_K.shape
    outs = [_empty_like(temperature_K, (layers, cells)) for _ in range(4)]
    scal = _empty_like(temperature_K, (5, cells))
    mem, st = _memory_of(temperature_K, humidity, cloud_water, surface_temperature_K, surface_pressure_Pa, scal)
    _raise(capi.load().psgb_column_radiation(cells, layers, C.byref(constants), _ptr(temperature_K), _ptr(humidity),
                                             _ptr(cloud_water), _ptr(surface_temperature_K),
                                             _ptr(surface_pressure_Pa), *[_ptr(o) for o in outs], _ptr(scal), mem, st))
    return (*outs, scal)

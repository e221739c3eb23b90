"""The non-symmetric transport solves over the C-ABI: the reference's IncompleteLU
(incomplete_lu.hpp:14-43), AdvectionDiffusion and its source, solve_implicit_tracer and
solve_implicit_advection_diffusion (heat_transport.hpp:140-248), all computing on the GPU.

Arrays are numpy (host) unless noted; CUDA tensors are accepted by the functions that
say so, with every array of one call on the same side."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import capi
from .api import PlanetMesh, _is_torch, _ptr, _raise, transport_settings


def _f64(a):
    return a if _is_torch(a) else np.ascontiguousarray(a, dtype=np.float64)


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def _count(a) -> int:
    return int(a.numel()) if _is_torch(a) else int(np.size(a))


class IncompleteLU:
    """Block ILU(0) of diagonal * scale + off (incomplete_lu.hpp:14-43), factored on the
    GPU at construction; `solve(x)` returns (LU)^-1 x. `offset`/`neighbour`: the
    off-diagonal CSR pattern; `block_start`: {0, ..., rows} (default: one block)."""

    def __init__(self, offset, neighbour, diagonal, off, block_start=None, diagonal_scale: float = 1.0):
        self._offset, self._neighbour = _u32(offset), _u32(neighbour)
        self._diagonal, self._off = _f64(diagonal), _f64(off)
        rows = len(self._diagonal)
        bs = _u32([0, rows] if block_start is None else block_start)
        self.rows = rows
        h = C.c_void_p()
        _raise(capi.load().psgb_incomplete_lu_create(C.c_uint32(rows), _ptr(self._offset), _ptr(self._neighbour),
                                                     _ptr(self._diagonal), _ptr(self._off), _ptr(bs),
                                                     C.c_uint32(len(bs) - 1), C.c_double(diagonal_scale),
                                                     C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            capi.load().psgb_incomplete_lu_destroy(h)
            self._h = None

    def solve(self, x):
        if _is_torch(x):
            import torch

            y = x.clone()
            _raise(capi.load().psgb_incomplete_lu_solve(self._h, _ptr(y), capi.MEMORY_DEVICE,
                                                        C.c_void_p(torch.cuda.current_stream().cuda_stream)))
            return y
        y = np.array(x, dtype=np.float64, copy=True)
        _raise(capi.load().psgb_incomplete_lu_solve(self._h, _ptr(y), capi.MEMORY_HOST, None))
        return y


@dataclass
class AdvectionDiffusion:
    """AdvectionDiffusion (heat_transport.hpp:140-166): per CSR entry the eddies'
    conductance (W/K), per layer and entry the outflowing mass (kg/s, layer-major), c_p,
    and per node the eddies' latent heat (W/m^2) or None."""

    layers: int
    conductance_W_K: np.ndarray
    outflow_kg_s: np.ndarray
    heat_capacity_J_kg_K: float = 1004.64
    eddy_latent_W_m2: np.ndarray | None = None
    _keep: list = field(default_factory=list, repr=False)

    def check(self, planet: PlanetMesh) -> None:
        """The arrays' sizes against the planet's graph (the C ABI takes bare pointers)."""
        entries, nodes = planet.directed_edge_count, planet.cell_count
        if self.layers < 0 or _count(self.conductance_W_K) != entries or \
                _count(self.outflow_kg_s) != self.layers * entries or \
                (self.eddy_latent_W_m2 is not None and _count(self.eddy_latent_W_m2) != nodes):
            raise ValueError("advection-diffusion inputs do not match the graph")

    def c_struct(self) -> capi.AdvectionDiffusion:
        g, o = _f64(self.conductance_W_K), _f64(self.outflow_kg_s)
        e = None if self.eddy_latent_W_m2 is None else _f64(self.eddy_latent_W_m2)
        self._keep = [g, o, e]
        return capi.AdvectionDiffusion(self.layers, _ptr(g).value, _ptr(o).value, self.heat_capacity_J_kg_K,
                                       None if e is None else _ptr(e).value)

    def on_device(self) -> bool:
        return _is_torch(self.conductance_W_K)


def _memory(transport: AdvectionDiffusion):
    if transport.on_device():
        import torch

        return capi.MEMORY_DEVICE, C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return capi.MEMORY_HOST, C.c_void_p(None)


def _empty(transport: AdvectionDiffusion, n: int):
    if transport.on_device():
        import torch

        return torch.empty(n, dtype=torch.float64, device="cuda")
    return np.empty(n)


def advection_diffusion_source(planet: PlanetMesh, transport: AdvectionDiffusion, mean_K, energy_J_kg):
    """advection_diffusion_source (heat_transport.hpp:168-175): (H_eddy, H_advective)."""
    n = planet.cell_count
    transport.check(planet)
    ts = transport.c_struct()
    m, e = _f64(mean_K), _f64(energy_J_kg)
    if _count(m) != n or _count(e) != transport.layers * n:
        raise ValueError("advection-diffusion inputs do not match the graph")
    eddy, adv = _empty(transport, n), _empty(transport, n)
    mem, st = _memory(transport)
    _raise(capi.load().psgb_advection_diffusion_source(planet.handle, C.byref(ts), _ptr(m), _ptr(e), _ptr(eddy),
                                                       _ptr(adv), mem, st))
    return eddy, adv


@dataclass
class TracerTransportResult:
    """TracerTransportResult (heat_transport.hpp:214-220)."""

    tracer: np.ndarray
    iterations: int
    relative_residual: float
    clipped_kg: float
    column_divergence_kg_s: float


def solve_implicit_tracer(planet: PlanetMesh, transport: AdvectionDiffusion, layer_mass_kg, tracer, dt_s: float,
                          relative_tolerance: float = 1e-12, max_iterations: int = 2000) -> TracerTransportResult:
    """solve_implicit_tracer (heat_transport.hpp:222-226): tracer layer-major."""
    n = planet.cell_count
    transport.check(planet)
    ts = transport.c_struct()
    mass, c0 = _f64(layer_mass_kg), _f64(tracer)
    if _count(mass) != n or _count(c0) != transport.layers * n:
        raise ValueError("tracer transport inputs do not match the graph")
    out = _empty(transport, transport.layers * n)
    res = capi.TracerResult()
    mem, st = _memory(transport)
    _raise(capi.load().psgb_solve_implicit_tracer(planet.handle, C.byref(ts), _ptr(mass), _ptr(c0), C.c_double(dt_s),
                                                  C.c_double(relative_tolerance), C.c_int(max_iterations), _ptr(out),
                                                  C.byref(res), mem, st))
    return TracerTransportResult(out, res.iterations, res.relative_residual, res.clipped_kg,
                                 res.column_divergence_kg_s)


@dataclass
class AdvectionDiffusionResult:
    """AdvectionDiffusionResult (heat_transport.hpp:175-186)."""

    source_W_m2: np.ndarray
    mean_K: np.ndarray
    energy_J_kg: np.ndarray
    consistency_residual_W_m2: float
    newton_iterations: int
    linear_iterations: int
    sum_W: float
    absolute_sum_W: float
    eddy_absolute_sum_W: float
    advective_absolute_sum_W: float


def solve_implicit_advection_diffusion(planet: PlanetMesh, transport: AdvectionDiffusion, source_floor_W_m2,
                                       response, settings: dict | None = None, initial_source_W_m2=None,
                                       device: bool = False) -> AdvectionDiffusionResult:
    """solve_implicit_advection_diffusion (heat_transport.hpp:240-248).

    Host response: `response(source) -> (mean, slope, energy, energy_slope)` on numpy
    arrays (energy layer-major, layers x nodes). With `device=True`:
    `response(nodes, layers, source, mean, slope, energy, energy_slope, stream)` on
    device pointers, enqueuing its work on `stream`."""
    n, L = planet.cell_count, transport.layers
    transport.check(planet)
    ts = transport.c_struct()
    floor = _f64(source_floor_W_m2)
    initial = None if initial_source_W_m2 is None else _f64(initial_source_W_m2)
    if _count(floor) != n or (initial is not None and _count(initial) != n):
        raise ValueError("advection-diffusion inputs do not match the graph")
    if _is_torch(floor) != transport.on_device() or (initial is not None and _is_torch(initial) != _is_torch(floor)):
        raise ValueError("pass every array as numpy or every array as CUDA tensors")
    error: list[BaseException] = []

    if device:
        def device_trampoline(_user, nodes, layers, source, mean, slope, energy, energy_slope, stream):
            try:
                response(int(nodes), int(layers), source, mean, slope, energy, energy_slope, stream)
                return 0
            except BaseException as exc:   # reported after the call returns
                error.append(exc)
                return 1

        dcb, hcb = capi.DeviceAdvectionResponse(device_trampoline), None
    else:
        def host_trampoline(_user, nodes, layers, source, mean, slope, energy, energy_slope):
            try:
                nn, nl = int(nodes), int(nodes) * int(layers)
                h = np.ctypeslib.as_array(C.cast(source, C.POINTER(C.c_double)), shape=(nn,)).copy()
                m, s, e, es = response(h)
                np.ctypeslib.as_array(C.cast(mean, C.POINTER(C.c_double)), shape=(nn,))[:] = m
                np.ctypeslib.as_array(C.cast(slope, C.POINTER(C.c_double)), shape=(nn,))[:] = s
                if nl:
                    np.ctypeslib.as_array(C.cast(energy, C.POINTER(C.c_double)), shape=(nl,))[:] = np.ravel(e)
                    np.ctypeslib.as_array(C.cast(energy_slope, C.POINTER(C.c_double)), shape=(nl,))[:] = \
                        np.ravel(es)
                return 0
            except BaseException as exc:
                error.append(exc)
                return 1

        hcb, dcb = capi.AdvectionResponse(host_trampoline), None
    source_out, mean_out, energy_out = _empty(transport, n), _empty(transport, n), _empty(transport, max(1, L * n))
    st_ = transport_settings(**(settings or {}))
    res = capi.AdvectionResult()
    mem, stream = _memory(transport)
    nil = C.c_void_p(None)
    code = capi.load().psgb_solve_implicit_advection_diffusion(
        planet.handle, C.byref(ts), _ptr(floor), nil if initial is None else _ptr(initial),
        nil if hcb is None else C.cast(hcb, C.c_void_p), nil if dcb is None else C.cast(dcb, C.c_void_p), None,
        C.byref(st_), _ptr(source_out), _ptr(mean_out), _ptr(energy_out), C.byref(res), mem, stream)
    if error:
        raise error[0]
    _raise(code)
    return AdvectionDiffusionResult(source_out, mean_out, energy_out[:L * n], res.consistency_residual_W_m2,
                                    res.newton_iterations, res.linear_iterations, res.sum_W, res.absolute_sum_W,
                                    res.eddy_absolute_sum_W, res.advective_absolute_sum_W)

"""ctypes bindings of the CPU oracle (oracle/planetsim_oracle.cpp) - TEST INFRASTRUCTURE.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as the
checker and the timed CPU baseline. The product never imports this module.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB = Path(__file__).resolve().parent / "lib" / "libplanetsim_oracle.so"


class Graph(C.Structure):
    _fields_ = [("n", C.c_uint64), ("offset", C.c_void_p), ("neighbour", C.c_void_p), ("weight", C.c_void_p),
                ("weight_sum", C.c_void_p), ("area", C.c_void_p)]


class Mesh(C.Structure):
    _fields_ = [("cells", C.c_uint64), ("edges", C.c_uint64), ("edge_offset", C.c_void_p),
                ("edge_count", C.c_void_p), ("neighbor", C.c_void_p), ("edge", C.c_void_p),
                ("normal_east", C.c_void_p), ("normal_north", C.c_void_p), ("edge_first", C.c_void_p),
                ("edge_length", C.c_void_p), ("edge_distance", C.c_void_p), ("area", C.c_void_p)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise FileNotFoundError(f"{LIB} is missing: __graft_entry__.build() compiles the oracle")
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        L.orc_hierarchy_new.restype = P
        L.orc_hierarchy_new.argtypes = [P]
        L.orc_hierarchy_free.argtypes = [P]
        L.orc_hierarchy_levels.restype = C.c_uint64
        L.orc_hierarchy_levels.argtypes = [P]
        L.orc_hierarchy_level.argtypes = [P, C.c_uint64, P, P, P, P, P]
        L.orc_hierarchy_set_matrix.argtypes = [P, P, P]
        L.orc_hierarchy_values.argtypes = [P, C.c_uint64, P, P]
        L.orc_vcycle_sgs.argtypes = [P, P, P]
        L.orc_vcycle_jacobi.argtypes = [P, C.c_int, C.c_int, C.c_double, C.c_double, P, P]
        L.orc_pcg.restype = C.c_int
        L.orc_pcg.argtypes = [P, P, C.c_double, P, P, P, C.c_double, C.c_int, P]
        L.orc_bicgstab.restype = C.c_int
        L.orc_bicgstab.argtypes = [P, P, C.c_double, P, P, C.c_double, C.c_int, P]
        L.orc_solve_implicit_transport_linear.argtypes = [P, C.c_double, P, P, C.c_double, C.c_double, P, P, P]
        L.orc_quartic_response.argtypes = [C.c_uint64, C.c_double, P, P, P, P]
        L.orc_solve_implicit_transport_quartic.argtypes = [P, C.c_double, C.c_double, P, C.c_double, C.c_double, P,
                                                           P, P, P]
        L.orc_transport_step.restype = C.c_int
        L.orc_transport_step.argtypes = [P, P, C.c_double, P, C.c_double, C.c_double, P, P, C.c_double, C.c_int,
                                         P, P, P, P]
        L.orc_column_radiation.argtypes = [C.c_uint64, C.c_uint32, P, P, P, P, P, P, P, P, P, P, P]
        L.orc_saturation_specific_humidity.restype = C.c_double
        L.orc_saturation_specific_humidity.argtypes = [C.c_double, C.c_double]
        for name in ("orc_laplacian_f64", "orc_laplacian_f32", "orc_divergence_f64", "orc_divergence_f32"):
            getattr(L, name).argtypes = [P, P, P]
        for name in ("orc_gradient_f64", "orc_gradient_f32"):
            getattr(L, name).argtypes = [P, P, P, P]
        L.orc_diffusion_source.argtypes = [P, C.c_double, P, P]
        L.orc_solve_implicit_transport_group_quartic.argtypes = [P, C.c_uint64, P, P, C.c_double, C.c_double, P, P,
                                                                 C.c_double, C.c_double, P, P, P]
        L.orc_ilu_new.restype = P
        L.orc_ilu_new.argtypes = [C.c_uint64, P, P, P, P, P, C.c_uint64, C.c_double]
        L.orc_ilu_zero_pivot.restype = C.c_int
        L.orc_ilu_zero_pivot.argtypes = [P]
        L.orc_ilu_solve.argtypes = [P, C.c_uint64, P]
        L.orc_ilu_free.argtypes = [P]
        L.orc_advection_source.argtypes = [C.c_uint64, P, P, P, C.c_uint64, P, P, P, P, P, P, P]
        L.orc_solve_implicit_tracer.argtypes = [C.c_uint64, P, P, C.c_uint64, P, P, C.c_double, P, P, C.c_double,
                                                C.c_double, C.c_int, P, P]
        L.orc_solve_implicit_advection_diffusion.argtypes = [P, C.c_uint64, P, P, P, C.c_double, C.c_double, P, P,
                                                             P, P, C.c_double, C.c_double, P, P, P, P]
        L.orc_icosphere_counts.restype = C.c_int
        L.orc_icosphere_counts.argtypes = [C.c_uint32, P, P, P]
        L.orc_icosphere.restype = C.c_int
        L.orc_icosphere.argtypes = [C.c_uint32, C.c_double] + [P] * 19
        L.orc_substep_mean_insolation.argtypes = [C.c_uint64, P, P, P, P, P, C.c_uint32, P]
        _lib = L
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(None)


def icosphere(level: int, radius_m: float) -> dict:
    """The reference's make_icosphere(level, radius_m) and its transport graph, built by the
    oracle's own restatement (mesh_oracle.cpp): the same keys as the product mesh's arrays()."""
    n, e, k = C.c_uint64(), C.c_uint64(), C.c_uint64()
    if lib().orc_icosphere_counts(level, C.byref(n), C.byref(e), C.byref(k)) != 0:
        raise ValueError(f"oracle mesh: level {level}")
    n, e, k = n.value, e.value, k.value
    d = 2 * e
    out = {
        "center": np.empty((n, 3)), "east": np.empty((n, 3)), "north": np.empty((n, 3)), "area_m2": np.empty(n),
        "source_vertex": np.empty(n, np.uint32), "edge_offset": np.empty(n, np.uint32),
        "edge_count": np.empty(n, np.uint8), "neighbor": np.empty(d, np.uint32), "edge": np.empty(d, np.uint32),
        "corner": np.empty(d, np.uint32), "normal_east": np.empty(d, np.float32),
        "normal_north": np.empty(d, np.float32), "edge_first": np.empty(e, np.uint32),
        "edge_second": np.empty(e, np.uint32), "edge_length_m": np.empty(e), "edge_distance_m": np.empty(e),
        "corner_unit": np.empty((k, 3)), "graph_weight": np.empty(d), "graph_weight_sum": np.empty(n),
    }
    order = ["center", "east", "north", "area_m2", "source_vertex", "edge_offset", "edge_count", "neighbor", "edge",
             "corner", "normal_east", "normal_north", "edge_first", "edge_second", "edge_length_m",
             "edge_distance_m", "corner_unit", "graph_weight", "graph_weight_sum"]
    if lib().orc_icosphere(level, float(radius_m), *[_p(out[name]) for name in order]) != 0:
        raise ValueError(f"oracle mesh: level {level}, radius {radius_m}")
    out["graph_area_m2"] = out["area_m2"]
    return out


def substep_mean_insolation(center, nodes) -> np.ndarray:
    """The reference's sub-step-mean insolation per cell (FP32), from unit cell centres
    [n, 3] and the sub-step's orbit nodes [16, 5] (time, weight, sin and cos of the
    declination, incident flux: the reference's substep_forcing_nodes)."""
    c = np.ascontiguousarray(center, dtype=np.float64)
    nd = np.ascontiguousarray(nodes, dtype=np.float64)
    cols = [np.ascontiguousarray(nd[:, j]) for j in (1, 2, 3, 4)]
    out = np.empty(len(c), dtype=np.float32)
    lib().orc_substep_mean_insolation(len(c), _p(c), *[_p(x) for x in cols], len(nd), _p(out))
    return out


class OracleMesh:
    """The flat mesh/graph arrays as the oracle's C structs (kept alive here)."""

    def __init__(self, arrays: dict):
        a = {k: np.ascontiguousarray(v) for k, v in arrays.items()}
        self.a = a
        n = len(a["area_m2"])
        self.n = n
        self.offset = np.append(a["edge_offset"], np.uint32(len(a["neighbor"]))).astype(np.uint32)
        self.neighbour = a["neighbor"].astype(np.uint32)
        # the transport graph's node areas: the cells' own, or an agglomeration's sums
        a.setdefault("graph_area_m2", a["area_m2"])
        self.graph = Graph(n, _p(self.offset), _p(self.neighbour), _p(a["graph_weight"]), _p(a["graph_weight_sum"]),
                           _p(a["graph_area_m2"]))
        self.mesh = Mesh(n, len(a["edge_length_m"]), _p(a["edge_offset"]), _p(a["edge_count"]), _p(a["neighbor"]),
                         _p(a["edge"]), _p(a["normal_east"]), _p(a["normal_north"]), _p(a["edge_first"]),
                         _p(a["edge_length_m"]), _p(a["edge_distance_m"]), _p(a["area_m2"]))

    def laplacian(self, x):
        out = np.empty_like(x)
        getattr(lib(), "orc_laplacian_f64" if x.dtype == np.float64 else "orc_laplacian_f32")(
            C.byref(self.mesh), _p(x), _p(out))
        return out

    def gradient(self, x):
        e, n = np.empty_like(x), np.empty_like(x)
        getattr(lib(), "orc_gradient_f64" if x.dtype == np.float64 else "orc_gradient_f32")(
            C.byref(self.mesh), _p(x), _p(e), _p(n))
        return e, n

    def divergence(self, f):
        out = np.empty(self.n, dtype=f.dtype)
        getattr(lib(), "orc_divergence_f64" if f.dtype == np.float64 else "orc_divergence_f32")(
            C.byref(self.mesh), _p(f), _p(out))
        return out

    def diffusion_source(self, K, t):
        out = np.empty(self.n)
        lib().orc_diffusion_source(C.byref(self.graph), K, _p(t), _p(out))
        return out

    def directed_conductance(self, per_edge):
        """Per-CSR-entry values from per-undirected-edge values."""
        return np.ascontiguousarray(np.asarray(per_edge)[self.a["edge"]], dtype=np.float64)

    def solve_implicit_transport_linear(self, K, base, slope, cg_tol=1e-12, newton_tol=1e-9):
        mean, src, stats = np.empty(self.n), np.empty(self.n), np.empty(6)
        lib().orc_solve_implicit_transport_linear(C.byref(self.graph), K, _p(base), _p(slope), cg_tol, newton_tol,
                                                  _p(mean), _p(src), _p(stats))
        return mean, src, stats

    def solve_implicit_transport_group_quartic(self, group_of_cell, fine_area, K, a, b_fine, floor, cg_tol=1e-6,
                                               newton_tol=1e-6):
        """The production group response on an agglomerated graph (this mesh's arrays carry
        the groups' areas as `graph_area_m2`): (mean, source, stats) per group."""
        keep = [np.ascontiguousarray(group_of_cell, np.uint32), np.ascontiguousarray(fine_area, np.float64),
                np.ascontiguousarray(b_fine, np.float64), np.ascontiguousarray(floor, np.float64)]
        mean, src, stats = np.empty(self.n), np.empty(self.n), np.empty(6)
        lib().orc_solve_implicit_transport_group_quartic(C.byref(self.graph), len(keep[0]), _p(keep[0]), _p(keep[1]),
                                                         K, a, _p(keep[2]), _p(keep[3]), cg_tol, newton_tol,
                                                         _p(mean), _p(src), _p(stats))
        return mean, src, stats

    def solve_implicit_transport_quartic(self, K, a, b, cg_tol=1e-6, newton_tol=1e-6):
        b = np.ascontiguousarray(b, np.float64)
        floor, mean, src, stats = np.empty(self.n), np.empty(self.n), np.empty(self.n), np.empty(6)
        lib().orc_solve_implicit_transport_quartic(C.byref(self.graph), K, a, _p(b), cg_tol, newton_tol, _p(floor),
                                                   _p(mean), _p(src), _p(stats))
        return floor, mean, src, stats


def quartic_response(a, b, source):
    """The quartic tile response of the reference's heat-transport test
    (tests/unit/test_heat_transport.cpp:30-76): T and dT/dh per cell."""
    b = np.ascontiguousarray(b, np.float64)
    source = np.ascontiguousarray(source, np.float64)
    mean, slope = np.empty(len(b)), np.empty(len(b))
    lib().orc_quartic_response(len(b), a, _p(b), _p(source), _p(mean), _p(slope))
    return mean, slope


class OracleHierarchy:
    def __init__(self, om: OracleMesh):
        self.om = om
        self.h = C.c_void_p(lib().orc_hierarchy_new(C.byref(om.graph)))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_hierarchy_free(self.h)

    def levels(self) -> int:
        return int(lib().orc_hierarchy_levels(self.h))

    def level(self, l: int) -> dict:
        sizes = np.zeros(4, np.uint64)
        ptrs = [C.c_void_p() for _ in range(4)]
        lib().orc_hierarchy_level(self.h, l, _p(sizes), *[C.byref(p) for p in ptrs])
        rows, nnz, na, nt = (int(s) for s in sizes)

        def view(ptr, dtype, count):
            if count == 0:
                return np.empty(0, dtype)
            raw = (C.c_char * (count * np.dtype(dtype).itemsize)).from_address(ptr.value)
            return np.frombuffer(raw, dtype=dtype, count=count).copy()

        return {"rows": rows, "offset": view(ptrs[0], np.uint32, rows + 1), "column": view(ptrs[1], np.uint32, nnz),
                "aggregate": view(ptrs[2], np.uint32, na), "target": view(ptrs[3], np.int64, nt)}

    def set_matrix(self, diag, off):
        diag, off = np.ascontiguousarray(diag, np.float64), np.ascontiguousarray(off, np.float64)
        lib().orc_hierarchy_set_matrix(self.h, _p(diag), _p(off))

    def values(self, l: int):
        lv = self.level(l)
        d, o = np.empty(lv["rows"]), np.empty(len(lv["column"]))
        lib().orc_hierarchy_values(self.h, l, _p(d), _p(o))
        return d, o

    def vcycle_sgs(self, rhs):
        out = np.empty(self.om.n)
        lib().orc_vcycle_sgs(self.h, _p(np.ascontiguousarray(rhs, np.float64)), _p(out))
        return out

    def vcycle_jacobi(self, rhs, pre=2, post=2, omega=0.8, correction=1.0):
        out = np.empty(self.om.n)
        lib().orc_vcycle_jacobi(self.h, pre, post, omega, correction, _p(np.ascontiguousarray(rhs, np.float64)),
                                _p(out))
        return out

    def pcg(self, K, slope, rhs, tol=1e-12, max_it=2000, edge_g=None):
        x = np.empty(self.om.n)
        it = lib().orc_pcg(self.h, C.byref(self.om.graph), K, _p(edge_g), _p(slope), _p(rhs), tol, max_it, _p(x))
        return x, it

    def bicgstab(self, K, slope, rhs, tol=1e-12, max_it=2000):
        x = np.empty(self.om.n)
        it = lib().orc_bicgstab(self.h, C.byref(self.om.graph), K, _p(slope), _p(rhs), tol, max_it, _p(x))
        return x, it

    def transport_step(self, K, C_heat, dt, t0, src, tol=1e-12, max_it=2000, edge_g=None):
        n = self.om.n
        ts, h, tn, sums = np.empty(n), np.empty(n), np.empty(n), np.empty(6)
        it = lib().orc_transport_step(self.h, C.byref(self.om.graph), K, _p(edge_g), C_heat, dt, _p(t0), _p(src), tol,
                                      max_it, _p(ts), _p(h), _p(tn), _p(sums))
        return {"t_solved": ts, "transport": h, "t_new": tn, "sums": sums, "iterations": it}


def column_radiation(constants, temperature, humidity, cloud, ts, ps):
    layers, cells = temperature.shape
    k = np.ascontiguousarray(constants, dtype=np.float64)
    ins = [np.ascontiguousarray(a, dtype=np.float64) for a in (temperature, humidity, cloud, ts, ps)]
    outs = [np.empty((layers, cells)) for _ in range(4)]
    scal = np.empty((5, cells))
    lib().orc_column_radiation(cells, layers, _p(k), *[_p(a) for a in ins], *[_p(o) for o in outs], _p(scal))
    return (*outs, scal)


def saturation_specific_humidity(t, p):
    return lib().orc_saturation_specific_humidity(float(t), float(p))


# ---- non-symmetric transport (nonsym_oracle.cpp) ------------------------------------

def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class OracleIlu:
    """IncompleteLU (incomplete_lu.cpp:33-152): block ILU(0), factored at construction."""

    def __init__(self, offset, neighbour, diagonal, off, block_start, scale: float = 1.0):
        self._keep = [_u32(offset), _u32(neighbour), _f64(diagonal), _f64(off), _u32(block_start)]
        o, nb, d, f, bs = self._keep
        self.rows = len(d)
        self._h = C.c_void_p(lib().orc_ilu_new(self.rows, _p(o), _p(nb), _p(d), _p(f), _p(bs), len(bs) - 1, scale))
        self.zero_pivot = bool(lib().orc_ilu_zero_pivot(self._h))

    def __del__(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().orc_ilu_free(self._h)
            self._h = None

    def solve(self, x):
        y = np.array(x, dtype=np.float64, copy=True)
        lib().orc_ilu_solve(self._h, self.rows, _p(y))
        return y


def advection_source(offset, neighbour, area, layers, conductance, outflow, latent, mean, energy):
    """advection_diffusion_source (heat_transport.cpp:774-815): (H_eddy, H_advective)."""
    o, nb = _u32(offset), _u32(neighbour)
    n = len(o) - 1
    eddy, adv = np.empty(n), np.empty(n)
    lib().orc_advection_source(n, _p(o), _p(nb), _p(_f64(area)), layers, _p(_f64(conductance)),
                               _p(_f64(outflow)), _p(_f64(latent)), _p(_f64(mean)), _p(_f64(energy)), _p(eddy),
                               _p(adv))
    return eddy, adv


def solve_implicit_tracer(offset, neighbour, layers, conductance, outflow, heat_capacity, layer_mass, tracer, dt,
                          tolerance=1e-12, max_iterations=2000):
    """solve_implicit_tracer (heat_transport.cpp:901-1081): the new tracer (layer-major) and
    (iterations, relative residual, clipped kg, column divergence)."""
    o, nb = _u32(offset), _u32(neighbour)
    n = len(o) - 1
    keep = [_f64(conductance), _f64(outflow), _f64(layer_mass), _f64(tracer)]
    out, stats = np.empty(layers * n), np.empty(4)
    lib().orc_solve_implicit_tracer(n, _p(o), _p(nb), layers, _p(keep[0]), _p(keep[1]), heat_capacity, _p(keep[2]),
                                    _p(keep[3]), dt, tolerance, max_iterations, _p(out), _p(stats))
    return out, stats


def solve_implicit_advection_diffusion(om: "OracleMesh", layers, conductance, outflow, latent, heat_capacity, a, b,
                                       epsilon, geopotential, floor, cg_tolerance=1e-6, newton_tolerance=1e-6):
    """solve_implicit_advection_diffusion (heat_transport.cpp:1083-1318) with the reference
    test's column (test_advection_diffusion.cpp:73-104): (H, theta, s, stats), stats =
    (newton, linear, consistency, sum, absolute, eddy absolute, advective absolute)."""
    n = om.n
    keep = [_f64(conductance), _f64(outflow), _f64(latent), _f64(b), _f64(epsilon), _f64(geopotential), _f64(floor)]
    src, mean, energy, stats = np.empty(n), np.empty(n), np.empty(layers * n), np.empty(7)
    lib().orc_solve_implicit_advection_diffusion(C.byref(om.graph), layers, _p(keep[0]), _p(keep[1]), _p(keep[2]),
                                                 heat_capacity, a, _p(keep[3]), _p(keep[4]), _p(keep[5]),
                                                 _p(keep[6]), cg_tolerance, newton_tolerance, _p(src), _p(mean),
                                                 _p(energy), _p(stats))
    return src, mean, energy, stats


# ---- many sub-steps of one planet, spread over the host cores -----------------------------

_WORKER: dict = {}
_GRAPH_KEYS = ("area_m2", "edge_offset", "edge_count", "neighbor", "edge", "normal_east", "normal_north",
               "edge_first", "edge_length_m", "edge_distance_m", "graph_weight", "graph_weight_sum", "graph_area_m2")


def _worker_init(path, K, C_heat, dt, edge_g):
    z = np.load(path)
    om = OracleMesh({k: z[k] for k in z.files})
    _WORKER.update(om=om, h=OracleHierarchy(om), K=K, C=C_heat, dt=dt,
                   g=None if edge_g is None else om.directed_conductance(edge_g))


def _worker_step(job):
    t0, src, tol = job
    w = _WORKER
    r = w["h"].transport_step(w["K"], w["C"], w["dt"], t0, src, tol=tol, edge_g=w["g"])
    return r["t_new"], r["transport"], r["iterations"]


def transport_steps(arrays: dict, K, C_heat, dt, t0s, sources, tol=1e-13, edge_g=None, processes=None):
    """Sub-steps (t0s[j], sources[j]) of one planet by the oracle, each process of a spawned
    pool holding the planet's hierarchy: [(t_new, transport, iterations)] in order."""
    import multiprocessing as mp
    import os
    import tempfile

    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "graph.npz")
        a = dict(arrays)
        a.setdefault("graph_area_m2", a["area_m2"])
        np.savez(path, **{k: a[k] for k in _GRAPH_KEYS})
        n = processes or max(1, min(len(sources), os.cpu_count() or 1))
        with mp.get_context("spawn").Pool(n, initializer=_worker_init, initargs=(path, K, C_heat, dt, edge_g)) as pool:
            return pool.map(_worker_step, [(t0s[j], sources[j], tol) for j in range(len(sources))], chunksize=1)

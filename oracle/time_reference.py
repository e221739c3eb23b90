"""Times the REFERENCE's own CPU implementation of the rows that widen the hot path, for
the measurement beside the GPU timings of `bench.py --workload next`.

The reference's sources are compiled where they lie (oracle/Makefile.ref -> oracle/_ref)
and driven through oracle/ref_driver.cpp, so this runs only where the reference checkout
is (the x86 container; the GPU host has neither the sources nor an x86 core):

    python oracle/time_reference.py /path/to/planet_game [--workers N]

Cases (the same shapes as `bench.py --workload next`, inputs from
planet_game_gb300.workloads with the same seeds):
  tracer       solve_implicit_tracer, the L7 mesh's agglomerated graph (40,962 nodes), 10 layers
  advection    solve_implicit_advection_diffusion, the L6 mesh graph (40,962 nodes), 3 layers,
               the reference test's quartic column
  insolation   compute_substep_mean_insolation, L8 (655,362 cells)
  agglomerated solve_implicit_transport, linear response, the L8 mesh's agglomerated graph
               (163,842 nodes), to a 1e-10 relative residual
Prints one JSON line: per case the median of 3 timed calls (after one warm-up), in ms.

    python oracle/time_reference.py /path/to/planet_game --headline

instead times the headline solve one core at a time: every planet of the 64-planet mix
(16 x L4, 24 x L5, 16 x L6, 8 x L7) solved to a 1e-10 relative residual by the reference's
solve_newton_system (PCG + SGS V-cycle, worker_count 1) and by the oracle's restatement
that bench.py's reference arm runs, on the same matrix (the planet's median conductance:
the reference's API takes one conductance per graph), the clock around the solve alone.
Oracle infrastructure: never imported by the product."""
from __future__ import annotations

import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
P = C.c_void_p
RADIUS = 6.371e6
CP = 1004.64


def p(a):
    return a.ctypes.data_as(P)


def load(reference: Path) -> C.CDLL:
    subprocess.run(["make", "-s", "-f", str(ROOT / "oracle" / "Makefile.ref"), f"REF={reference}",
                    f"OUT={ROOT / 'oracle' / '_ref'}", "-j8", "-C", str(ROOT)], check=True)
    R = C.CDLL(str(ROOT / "oracle" / "_ref" / "libref_driver.so"))
    R.refd_mesh_new.restype = P
    R.refd_mesh_new.argtypes = [C.c_uint32, C.c_double]
    R.refd_mesh_free.argtypes = [P]
    R.refd_mesh_counts.argtypes = [P, P]
    R.refd_graph.argtypes = [P, P, P, P, P, P]
    R.refd_agglomeration_counts.argtypes = [P, P]
    R.refd_agglomeration.argtypes = [P, P, P, P, P, P, P]
    R.refd_tracer.argtypes = [P, C.c_int, C.c_uint64, P, P, C.c_double, P, P, C.c_double, C.c_double, C.c_uint64,
                              P, P]
    R.refd_advection_solve.argtypes = [P, C.c_int, C.c_uint64, P, P, P, C.c_double, C.c_double, P, P, P, P,
                                       C.c_double, C.c_double, C.c_uint64, P, P, P, P]
    R.refd_insolation.argtypes = [P, C.c_int64, P]
    R.refd_solve_linear_agglomerated.argtypes = [P, C.c_double, P, P, C.c_double, C.c_double, C.c_uint64, P, P, P]
    R.refd_pcg_seconds.restype = C.c_double
    R.refd_pcg_seconds.argtypes = [P, C.c_double, P, P, C.c_double, C.c_int, C.c_uint64, P, P]
    return R


def graph(R, m, agglomerated: bool) -> dict:
    if agglomerated:
        c = np.zeros(3, dtype=np.uint64)
        R.refd_agglomeration_counts(m, p(c))
        n, d, f = (int(x) for x in c)
    else:
        c = np.zeros(4, dtype=np.uint64)
        R.refd_mesh_counts(m, p(c))
        n, d = int(c[0]), int(c[2])
    area, wsum, w = np.empty(n), np.empty(n), np.empty(d)
    off, nb = np.empty(n + 1, dtype=np.uint64), np.empty(d, dtype=np.uint64)
    if agglomerated:
        R.refd_agglomeration(m, p(area), p(off), p(nb), p(w), p(wsum), p(np.empty(f, dtype=np.uint64)))
    else:
        R.refd_graph(m, p(area), p(off), p(nb), p(w), p(wsum))
    return {"area": area, "offset": off, "neighbour": nb, "weight": w}


def median_ms(fn, repeats: int = 3) -> float:
    fn()
    times = []
    for _ in range(repeats):
        t = time.perf_counter()
        fn()
        times.append((time.perf_counter() - t) * 1e3)
    return statistics.median(times)


def main(reference: Path, workers: int) -> None:
    from planet_game_gb300 import workloads as W

    R = load(reference)
    out = {"workers": workers, "host": os.uname().machine}
    t = time.perf_counter()
    R.refd_mesh_free(P(R.refd_mesh_new(8, RADIUS)))   # make_icosphere (single-threaded in the reference)
    out["mesh_l8_ms"] = (time.perf_counter() - t) * 1e3
    # tracer: agglomerated L7 graph, 10 layers
    m7 = P(R.refd_mesh_new(7, RADIUS))
    g = graph(R, m7, True)
    layers = 10
    flux = W.antisymmetric_layer_fluxes(g["offset"], g["neighbour"], layers, 2e9, seed=71, column_balanced=False)
    cond = np.full(len(g["neighbour"]), 2e8)
    mass = g["area"] * 100000.0 / (9.81 * layers)
    tracer = W.tracer_field(layers * len(g["area"]), seed=72)
    res, stats = np.empty(layers * len(g["area"])), np.empty(4)
    out["tracer_ms"] = median_ms(lambda: R.refd_tracer(m7, 1, layers, p(cond), p(flux), CP, p(mass), p(tracer),
                                                       2.63e6, 1e-12, workers, p(res), p(stats)))
    out["tracer_iterations"] = int(stats[0])
    # agglomerated heat transport: L8 -> 163,842 nodes, linear response
    m8 = P(R.refd_mesh_new(8, RADIUS))
    g8 = graph(R, m8, True)
    n8 = len(g8["area"])
    t0, source = W.agglomerated_step_inputs(n8, seed=81)
    s = W.SUBSTEP_S / W.HEAT_CAPACITY
    base = t0 + s * source          # T = T0 + s (S + h): the step's linear response
    slope = np.full(n8, s)
    mean, src, st = np.empty(n8), np.empty(n8), np.empty(3)
    out["agglomerated_ms"] = median_ms(lambda: R.refd_solve_linear_agglomerated(
        m8, W.HEAT_CAPACITY * W.DIFFUSIVITY, p(base), p(slope), 1e-10, 1e-6, workers, p(mean), p(src), p(st)))
    out["agglomerated_newton"], out["agglomerated_cg_iterations"] = int(st[0]), int(st[1])
    # insolation at L8
    ins = np.empty(655362, dtype=np.float32)
    out["insolation_ms"] = median_ms(lambda: R.refd_insolation(m8, 0, p(ins)))
    # coupled advection-diffusion: L6 mesh graph, 3 layers, the test's column
    m6 = P(R.refd_mesh_new(6, RADIUS))
    g6 = graph(R, m6, False)
    n6 = len(g6["area"])
    flux6 = W.antisymmetric_layer_fluxes(g6["offset"], g6["neighbour"], 3, 5e9, seed=61, column_balanced=True)
    cond6 = 0.5 * RADIUS * RADIUS * g6["weight"]
    a = 3.0e5 / (30.0 * 86400.0)
    radiative = 0.75 * 0.97 * 5.670374419e-8
    b, floor = W.quartic_column(a, radiative, n6, seed=62)
    eps, phi = np.array([0.0, -0.08, -0.16]), np.array([3.0e4, 4.5e4, 7.0e4])
    src6, mn6, en6, st6 = np.empty(n6), np.empty(n6), np.empty(3 * n6), np.empty(7)
    out["advection_ms"] = median_ms(lambda: R.refd_advection_solve(
        m6, 0, 3, p(cond6), p(flux6), None, CP, a, p(b), p(eps), p(phi), p(floor), 1e-6, 1e-6, workers, p(src6),
        p(mn6), p(en6), p(st6)))
    out["advection_newton"], out["advection_linear"] = int(st6[0]), int(st6[1])
    for m in (m6, m7, m8):
        R.refd_mesh_free(m)
    print(json.dumps(out))


def headline(reference: Path) -> None:
    """The reference's PCG against the oracle's restatement of it, one core, per planet."""
    import planet_game_gb300 as pg
    from oracle import oracle as O
    from planet_game_gb300 import workloads as W

    R = load(reference)
    ref_s, port_s, ref_it, port_it, worst = 0.0, 0.0, 0, 0, 0.0
    per_level: dict[str, list[float]] = {}
    specs = W.planet_mix(2026)
    for spec in specs:
        mesh = pg.make_icosphere(spec.level, spec.radius)
        inp = W.step_inputs(mesh, spec.seed)
        arrays = mesh.arrays()
        n = mesh.cell_count
        s = inp.dt / inp.heat_capacity
        area = arrays["area_m2"]
        slope, rhs = np.full(n, s), area / s * inp.t0 + area * inp.source
        m = P(R.refd_mesh_new(spec.level, spec.radius))
        x_ref, it = np.empty(n), C.c_int(0)
        best = min(R.refd_pcg_seconds(m, inp.conductance, p(slope), p(rhs), 1e-10, 2000, 1, p(x_ref), C.byref(it))
                   for _ in range(3))
        R.refd_mesh_free(m)
        h = O.OracleHierarchy(O.OracleMesh(arrays))
        times = []
        for _ in range(3):
            t = time.perf_counter()
            x_port, port = h.pcg(inp.conductance, slope, rhs, 1e-10, 2000)
            times.append(time.perf_counter() - t)
        ref_s, port_s = ref_s + best, port_s + min(times)
        lv = per_level.setdefault(f"L{spec.level}", [0.0, 0.0])
        lv[0] += best
        lv[1] += min(times)
        ref_it, port_it = ref_it + it.value, port_it + port
        worst = max(worst, float(np.max(np.abs(x_port - x_ref)) / np.max(np.abs(x_ref))))
    print(json.dumps({"host": os.uname().machine, "planets": len(specs), "reference_s": ref_s, "port_s": port_s,
                      "port_over_reference": port_s / ref_s, "reference_pcg_iterations": ref_it,
                      "port_pcg_iterations": port_it, "max_relative_difference": worst,
                      "reference_substeps_per_s_one_core": len(specs) / ref_s,
                      "port_substeps_per_s_one_core": len(specs) / port_s,
                      "per_level_reference_port_s": per_level}))


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    workers = os.cpu_count() or 1
    if "--workers" in sys.argv:
        workers = int(sys.argv[sys.argv.index("--workers") + 1])
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    from oracle.build import reference_root

    reference = reference_root(args[0] if args else None)
    if reference is None:
        raise SystemExit("name the reference checkout: time_reference.py <path> (or set PLANETSIM_REFERENCE)")
    if "--headline" in sys.argv:
        headline(reference)
    else:
        main(reference, workers)

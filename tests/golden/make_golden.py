"""Writes the golden fixtures of tests/golden/ from the REFERENCE's own code.

The reference PlanetSim sources are compiled where they lie (oracle/Makefile.ref, into
oracle/_ref/) and driven through oracle/ref_driver.cpp. Every number saved here is
computed by the reference's functions; the inputs are seeded numpy draws saved with
them. Run in a container that has the reference checkout:

    python tests/golden/make_golden.py /path/to/planet_game

The fixtures are small (.npz / .json); the GPU machine never needs the reference.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
DRIVER = ROOT / "oracle" / "_ref" / "libref_driver.so"
RADIUS = 6.371e6
P = C.c_void_p


def p(a):
    return a.ctypes.data_as(P)


def P_(handle):
    return handle if isinstance(handle, P) else P(handle)


def load(reference: Path) -> C.CDLL:
    subprocess.run(["make", "-s", "-f", str(ROOT / "oracle" / "Makefile.ref"), f"REF={reference}",
                    f"OUT={ROOT / 'oracle' / '_ref'}", "-j8", "-C", str(ROOT)], check=True)
    R = C.CDLL(str(DRIVER))
    R.refd_mesh_new.restype = P
    R.refd_mesh_new.argtypes = [C.c_uint32, C.c_double]
    R.refd_mesh_free.argtypes = [P]
    R.refd_hierarchy_new.restype = P
    R.refd_hierarchy_new.argtypes = [P]
    R.refd_hierarchy_free.argtypes = [P]
    R.refd_hierarchy_level_count.restype = C.c_uint64
    R.refd_hierarchy_level_count.argtypes = [P]
    R.refd_pcg.restype = C.c_int
    R.refd_pcg.argtypes = [P, C.c_double, P, P, C.c_double, C.c_int, C.c_uint64, P]
    R.refd_solve_linear.argtypes = [P, C.c_double, P, P, C.c_double, C.c_double, C.c_uint64, P, P, P]
    R.refd_diffusion_source.argtypes = [P, C.c_double, P, P]
    R.refd_saturation_specific_humidity.restype = C.c_double
    R.refd_saturation_specific_humidity.argtypes = [C.c_double, C.c_double]
    R.refd_surface_gravity_earth.restype = C.c_double
    R.refd_column_radiation.restype = C.c_int
    R.refd_column_radiation.argtypes = [C.c_uint32, P, P, P, C.c_double, C.c_double, C.c_double, P, P, P, P, P, P]
    R.refd_insolation.argtypes = [P, C.c_int64, P]
    R.refd_insolation_nodes.argtypes = [C.c_int64, P]
    R.refd_quartic_response.argtypes = [C.c_uint64, C.c_double, P, P, P, P]
    R.refd_solve_quartic.argtypes = [P, C.c_double, C.c_double, P, C.c_double, C.c_double, C.c_uint64, P, P, P, P]
    R.refd_agglomeration_counts.argtypes = [P, P]
    R.refd_agglomeration.argtypes = [P, P, P, P, P, P, P]
    R.refd_graph.argtypes = [P, P, P, P, P, P]
    R.refd_incomplete_lu.argtypes = [C.c_uint64, P, P, P, P, P, C.c_uint64, C.c_double, P]
    R.refd_advection_source.argtypes = [P, C.c_int, C.c_uint64, P, P, P, C.c_double, P, P, P, P]
    R.refd_tracer.argtypes = [P, C.c_int, C.c_uint64, P, P, C.c_double, P, P, C.c_double, C.c_double, C.c_uint64,
                              P, P]
    R.refd_advection_solve.argtypes = [P, C.c_int, C.c_uint64, P, P, P, C.c_double, C.c_double, P, P, P, P,
                                       C.c_double, C.c_double, C.c_uint64, P, P, P, P]
    R.refd_solve_quartic_agglomerated.argtypes = [P, C.c_double, C.c_double, P, C.c_double, C.c_double, C.c_uint64,
                                                  P, P, P, P]
    return R


AGGLOMERATION_LEVELS = (0, 1, 3, 5)


def agglomeration_cases(R) -> None:
    """The agglomerated transport graph (heat_transport.cpp:456-539): for each fine level,
    the reference's group of every fine cell and the coarse graph (areas, CSR, weights).
    Integer maps in full; the L5 graph's doubles in full as well (2,562 nodes)."""
    out = {}
    for level in AGGLOMERATION_LEVELS:
        m = P(R.refd_mesh_new(level, RADIUS))
        counts = np.zeros(3, dtype=np.uint64)
        R.refd_agglomeration_counts(m, p(counts))
        n, d, f = (int(c) for c in counts)
        area, wsum = np.empty(n), np.empty(n)
        off, nb = np.empty(n + 1, dtype=np.uint64), np.empty(d, dtype=np.uint64)
        w, groups = np.empty(d), np.empty(f, dtype=np.uint64)
        R.refd_agglomeration(m, p(area), p(off), p(nb), p(w), p(wsum), p(groups))
        R.refd_mesh_free(m)
        out.update({f"area{level}": area, f"offset{level}": off.astype(np.uint32),
                    f"neighbour{level}": nb.astype(np.uint32), f"weight{level}": w,
                    f"weight_sum{level}": wsum, f"group{level}": groups.astype(np.uint32)})
    # The production pattern at L5: the quartic response per fine cell at its group's
    # source, group means over the cells, the reference's solve on the agglomerated graph.
    m = P(R.refd_mesh_new(5, RADIUS))
    cnt = np.zeros(4, np.uint64)
    R.refd_mesh_counts(m, p(cnt))
    cells, groups = int(cnt[0]), len(out["area5"])
    rng = np.random.default_rng(20261203)
    radiative = 0.75 * 0.97 * 5.670374419e-8
    a = 0.04 + 0.37
    target = 200.0 + 120.0 * rng.random(cells)
    out["qa"], out["qb"] = a, a * target + radiative * target ** 4
    for factor in (1, 10):
        K = factor * 0.5 * RADIUS * RADIUS
        floor, mean, src, stats = np.empty(groups), np.empty(groups), np.empty(groups), np.empty(6)
        R.refd_solve_quartic_agglomerated(m, a, K, p(out["qb"]), 1e-6, 1e-6, 4, p(floor), p(mean), p(src), p(stats))
        out.update({f"qK{factor}": K, f"qfloor{factor}": floor, f"qmean{factor}": mean, f"qsource{factor}": src,
                    f"qstats{factor}": stats})
    R.refd_mesh_free(m)
    np.savez_compressed(HERE / "agglomeration.npz", levels=np.array(AGGLOMERATION_LEVELS), **out)
    # L6-L8 as SHA-256 digests of the same arrays (groups as uint32, CSR as uint32, doubles)
    digests = {}
    for level in (6, 7, 8):
        m = P(R.refd_mesh_new(level, RADIUS))
        counts = np.zeros(3, dtype=np.uint64)
        R.refd_agglomeration_counts(m, p(counts))
        n, d, f = (int(c) for c in counts)
        area, wsum = np.empty(n), np.empty(n)
        off, nb = np.empty(n + 1, dtype=np.uint64), np.empty(d, dtype=np.uint64)
        w, groups = np.empty(d), np.empty(f, dtype=np.uint64)
        R.refd_agglomeration(m, p(area), p(off), p(nb), p(w), p(wsum), p(groups))
        R.refd_mesh_free(m)
        digests[str(level)] = {"group": sha(groups.astype(np.uint32)), "area": sha(area),
                               "offset": sha(off.astype(np.uint32)), "neighbour": sha(nb.astype(np.uint32)),
                               "weight": sha(w), "weight_sum": sha(wsum), "nodes": n}
    (HERE / "agglomeration_sha256.json").write_text(json.dumps(digests, indent=1, sort_keys=True))


def ref_graph(R, m, agglomerated: bool) -> dict:
    """The reference's transport graph of mesh handle `m` (its own, or its agglomeration)."""
    if agglomerated:
        counts = np.zeros(3, dtype=np.uint64)
        R.refd_agglomeration_counts(m, p(counts))
        n, d, f = (int(c) for c in counts)
    else:
        cnt = np.zeros(4, np.uint64)
        R.refd_mesh_counts(m, p(cnt))
        n, d = int(cnt[0]), int(cnt[2])
    area, wsum = np.empty(n), np.empty(n)
    off, nb, w = np.empty(n + 1, dtype=np.uint64), np.empty(d, dtype=np.uint64), np.empty(d)
    if agglomerated:
        groups = np.empty(f, dtype=np.uint64)
        R.refd_agglomeration(m, p(area), p(off), p(nb), p(w), p(wsum), p(groups))
    else:
        R.refd_graph(m, p(area), p(off), p(nb), p(w), p(wsum))
    return {"area": area, "offset": off, "neighbour": nb, "weight": w}


def reverse_entries(g: dict) -> np.ndarray:
    off, nb = g["offset"], g["neighbour"]
    rev = np.empty(len(nb), dtype=np.int64)
    for a in range(len(off) - 1):
        for k in range(off[a], off[a + 1]):
            b = nb[k]
            row = nb[off[b]:off[b + 1]]
            rev[k] = off[b] + int(np.nonzero(row == a)[0][0])
    return rev


def column_free_fluxes(g: dict, layers: int, scale: float, rng) -> np.ndarray:
    """Antisymmetric layer fluxes summing to zero over each face's column (the bottom
    layer's flux returns in the others), as test_advection_diffusion.cpp:47-70 builds."""
    assert layers == 3
    off, nb = g["offset"], g["neighbour"]
    E = len(nb)
    rev = reverse_entries(g)
    out = np.zeros(layers * E)
    for a in range(len(off) - 1):
        for k in range(off[a], off[a + 1]):
            if a < nb[k]:
                f = scale * (2.0 * rng.random() - 1.0)
                split = rng.random()
                flux = [f, -split * f, -(1.0 - split) * f]
                for l in range(layers):
                    out[l * E + k] = flux[l]
                    out[l * E + rev[k]] = -flux[l]
    return out


def noisy_fluxes(g: dict, layers: int, scale: float, divergent: bool, rng) -> np.ndarray:
    """Antisymmetric per-face layer fluxes of about `scale`, with or without column
    divergence (test_tracer_transport.cpp:33-60's construction, seeded numpy draws)."""
    off, nb = g["offset"], g["neighbour"]
    E = len(nb)
    rev = reverse_entries(g)
    out = np.zeros(layers * E)
    for a in range(len(off) - 1):
        for k in range(off[a], off[a + 1]):
            if a < nb[k]:
                flow = scale * (2.0 * rng.random(layers) - 1.0)
                if not divergent:
                    flow = flow - flow.mean()
                for l in range(layers):
                    out[l * E + k] = flow[l]
                    out[l * E + rev[k]] = -flow[l]
    return out


NONSYM_CP = 1004.64


def upper_entries(g: dict) -> np.ndarray:
    """The CSR entries a -> b with a < b, in CSR order: one per face."""
    off, nb = g["offset"], g["neighbour"]
    rows = np.repeat(np.arange(len(off) - 1), np.diff(off.astype(np.int64)))
    return np.nonzero(rows < nb.astype(np.int64))[0]


def half_fluxes(g: dict, flows: np.ndarray, layers: int) -> np.ndarray:
    """The antisymmetric flows on the faces' a < b entries only ([layers][faces])."""
    E = len(g["neighbour"])
    return flows.reshape(layers, E)[:, upper_entries(g)].copy()


def nonsym_cases(R, write: bool = True) -> dict:
    """The non-symmetric solves of the reference (heat_transport.cpp:774-1318) and its
    block ILU(0) (incomplete_lu.cpp), on the L3 mesh graph, the L3 mesh's agglomerated
    graph and the L4 mesh graph; inputs are seeded numpy draws shaped like the
    reference's tests (test_tracer_transport.cpp, test_advection_diffusion.cpp)."""
    rng = np.random.default_rng(20261204)
    out = {}
    m3 = P(R.refd_mesh_new(3, RADIUS))
    g3, g3a = ref_graph(R, m3, False), ref_graph(R, m3, True)
    # block ILU(0) on the L3 graph with a non-symmetric diagonally dominant matrix
    n4 = len(g3["area"])
    diag = 6.0 + 4.0 * rng.random(n4)
    offv = -rng.random(len(g3["neighbour"]))
    blocks = np.array(list(range(0, n4, 256)) + [n4], dtype=np.uint64)
    x = rng.standard_normal(n4)
    y = x.copy()
    R.refd_incomplete_lu(n4, p(g3["offset"]), p(g3["neighbour"]), p(diag), p(offv), p(blocks), len(blocks) - 1, 1.0,
                         p(y))
    out.update(ilu_diag=diag, ilu_off=offv, ilu_blocks=blocks.astype(np.uint32), ilu_x=x, ilu_y=y)
    # advection-diffusion source on the L3 graph
    n3, L = len(g3["area"]), 3
    K = 0.5 * RADIUS * RADIUS
    cond = K * g3["weight"]
    flux = column_free_fluxes(g3, L, 5.0e9, rng)   # also the coupled solves' fluxes, below
    mean = 250.0 + 50.0 * rng.random(n3)
    energy = 2.5e5 + 1.0e5 * rng.random(L * n3)
    latent = rng.normal(0.0, 3.0, n3)
    for tag, lat in (("dry", None), ("latent", latent)):
        eddy, adv = np.empty(n3), np.empty(n3)
        R.refd_advection_source(m3, 0, L, p(cond), p(flux), None if lat is None else p(lat), NONSYM_CP, p(mean),
                                p(energy), p(eddy), p(adv))
        out[f"src_eddy_{tag}"], out[f"src_adv_{tag}"] = eddy, adv
    out.update(flux=half_fluxes(g3, flux, L), src_mean=mean, src_energy=energy, src_latent=latent)
    # the tracer on the agglomerated L3 graph (3 layers) and the L4 graph (2 layers)
    month = 2.63e6
    for tag, (m, g, agg, layers, scale, eddy_g, divergent) in {
            "bal": (m3, g3a, 1, 3, 2e9, 2e8, False), "div": (m3, g3a, 1, 3, 2e9, 2e8, True),
            "eddy": (m3, g3a, 1, 2, 0.0, 1e13, False), "l3": (m3, g3, 0, 2, 5e9, 5e8, True)}.items():
        n = len(g["area"])
        E = len(g["neighbour"])
        flows = noisy_fluxes(g, layers, scale, divergent, rng) if scale > 0 else np.zeros(layers * E)
        conductance = np.full(E, eddy_g)
        mass = g["area"] * 100000.0 / (9.81 * layers)
        tracer = 0.01 * (1.0 + (2.0 * rng.random(layers * n) - 1.0)) + np.where(np.arange(layers * n) % 17 == 0, 0.0,
                                                                               1e-6)
        res, stats = np.empty(layers * n), np.empty(4)
        R.refd_tracer(m, agg, layers, p(conductance), p(flows), NONSYM_CP, p(mass), p(tracer), month, 1e-12, 1,
                      p(res), p(stats))
        out.update({f"tr_{tag}_layers": layers, f"tr_{tag}_agg": agg, f"tr_{tag}_eddy": eddy_g,
                    f"tr_{tag}_flux": half_fluxes(g, flows, layers), f"tr_{tag}_in": tracer, f"tr_{tag}_out": res,
                    f"tr_{tag}_stats": stats})
    # the coupled solve on the L3 graph: pure diffusion, advection, advection with latent heat
    a = 3.0e5 / (30.0 * 86400.0)
    radiative = 0.75 * 0.97 * 5.670374419e-8
    target = 200.0 + 120.0 * rng.random(n3)
    b = a * target + radiative * target ** 4
    floor = a * 100.0 + radiative * 100.0 ** 4 - b
    eps, phi = np.array([0.0, -0.08, -0.16]), np.array([3.0e4, 4.5e4, 7.0e4])
    out.update(ad_a=a, ad_b=b, ad_floor=floor, ad_eps=eps, ad_phi=phi)
    for tag, scale, with_latent in (("diff", 0.0, False), ("adv", 5.0e9, False), ("lat", 5.0e9, True)):
        flows = flux if scale > 0 else np.zeros(L * len(g3["neighbour"]))
        lat = None
        if with_latent:
            rnd = rng.random(n3)
            lat = np.zeros(n3)
            for i in range(n3):
                water = 0.0
                for k in range(g3["offset"][i], g3["offset"][i + 1]):
                    j = g3["neighbour"][k]
                    water += cond[k] / (NONSYM_CP * L) * 1e-3 * (rnd[j] - rnd[i])
                lat[i] = 2.501e6 * water / g3["area"][i]
        src, mn, en, stats = np.empty(n3), np.empty(n3), np.empty(L * n3), np.empty(7)
        R.refd_advection_solve(m3, 0, L, p(cond), p(flows), None if lat is None else p(lat), NONSYM_CP, a, p(b),
                               p(eps), p(phi), p(floor), 1e-6, 1e-6, 1, p(src), p(mn), p(en), p(stats))
        out.update({f"ad_{tag}_source": src, f"ad_{tag}_mean": mn, f"ad_{tag}_energy": en,
                    f"ad_{tag}_stats": stats})
        if lat is not None:
            out[f"ad_{tag}_latent"] = lat
    R.refd_mesh_free(m3)
    if write:
        np.savez_compressed(HERE / "nonsym.npz", **out)
    return out


def quartic_cases(R, write: bool = True) -> dict:
    """The nonlinear transport solve with the reference test's quartic response
    (tests/unit/test_heat_transport.cpp:30-76, 112-146) at L4: heat capacities of a month
    and of ten minutes, the test's conductance and ten times it. The local forcings b put
    each column's equilibrium between 200 and 320 K (seeded here instead of the test's
    keyed random stream); a sample of response evaluations pins the response itself."""
    m = R.refd_mesh_new(4, RADIUS)
    cnt = np.zeros(4, np.uint64)
    R.refd_mesh_counts(P_(m), p(cnt))
    n = int(cnt[0])
    rng = np.random.default_rng(20260930)
    radiative = 0.75 * 0.97 * 5.670374419e-8
    out = {}
    for ia, a in enumerate((0.04 + 0.37, 1.0e5 / 600.0)):
        target = 200.0 + 120.0 * rng.random(n)
        b = a * target + radiative * target ** 4
        out[f"b{ia}"] = b
        out[f"a{ia}"] = a
        h = rng.normal(0.0, 40.0, n)
        mean, slope = np.empty(n), np.empty(n)
        R.refd_quartic_response(n, a, p(b), p(h), p(mean), p(slope))
        out[f"probe_source{ia}"], out[f"probe_mean{ia}"], out[f"probe_slope{ia}"] = h, mean, slope
        for factor in (1.0, 10.0):
            K = factor * 0.5 * RADIUS * RADIUS
            floor, mean, src, stats = np.empty(n), np.empty(n), np.empty(n), np.empty(6)
            R.refd_solve_quartic(m, a, K, p(b), 1e-6, 1e-6, 4, p(floor), p(mean), p(src), p(stats))
            key = f"{ia}_{int(factor)}"
            out[f"K{key}"], out[f"floor{key}"], out[f"mean{key}"] = K, floor, mean
            out[f"source{key}"], out[f"stats{key}"] = src, stats
    if write:
        np.savez_compressed(HERE / "newton_quartic_L4.npz", **out)
    R.refd_mesh_free(m)
    return out


def mesh_arrays(R, m) -> dict:
    cnt = np.zeros(4, np.uint64)
    R.refd_mesh_counts(P_(m), p(cnt))
    n, e, d, k = (int(x) for x in cnt)
    a = dict(center=np.zeros((n, 3)), east=np.zeros((n, 3)), north=np.zeros((n, 3)), area_m2=np.zeros(n),
             source_vertex=np.zeros(n, np.uint32), edge_offset=np.zeros(n, np.uint32), edge_count=np.zeros(n, np.uint8),
             neighbor=np.zeros(d, np.uint32), edge=np.zeros(d, np.uint32), normal_east=np.zeros(d, np.float32),
             normal_north=np.zeros(d, np.float32), edge_first=np.zeros(e, np.uint32), edge_second=np.zeros(e, np.uint32),
             edge_length_m=np.zeros(e), edge_distance_m=np.zeros(e), corner_unit=np.zeros((k, 3)),
             corner=np.zeros(d, np.uint32))
    R.refd_mesh_cells(P_(m), *[p(a[x]) for x in ("center", "east", "north", "area_m2", "source_vertex", "edge_offset",
                                                 "edge_count")])
    R.refd_mesh_cell_edges(P_(m), *[p(a[x]) for x in ("neighbor", "edge", "normal_east", "normal_north")])
    R.refd_mesh_edges(P_(m), *[p(a[x]) for x in ("edge_first", "edge_second", "edge_length_m", "edge_distance_m")])
    R.refd_mesh_corners(P_(m), p(a["corner_unit"]), p(a["corner"]))
    off = np.zeros(n + 1, np.uint64)
    nb = np.zeros(d, np.uint64)
    a["graph_weight"] = np.zeros(d)
    a["graph_weight_sum"] = np.zeros(n)
    area = np.zeros(n)
    R.refd_graph(P_(m), p(area), p(off), p(nb), p(a["graph_weight"]), p(a["graph_weight_sum"]))
    return a


def sha(arr: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(arr).tobytes()).hexdigest()


def hierarchy(R, m) -> list[dict]:
    h = P(R.refd_hierarchy_new(P_(m)))
    out = []
    for i in range(int(R.refd_hierarchy_level_count(h))):
        s = np.zeros(4, np.uint64)
        R.refd_hierarchy_level_sizes(h, C.c_uint64(i), p(s))
        rows, nnz, na, nt = (int(x) for x in s)
        off, col = np.zeros(rows + 1, np.int64), np.zeros(nnz, np.int64)
        agg, tgt = np.zeros(max(na, 1), np.int64), np.zeros(max(nt, 1), np.int64)
        dg, val = np.zeros(rows), np.zeros(nnz)
        R.refd_hierarchy_level(h, C.c_uint64(i), p(off), p(col), p(agg), p(tgt), p(dg), p(val))
        out.append(dict(offset=off.astype(np.uint32), column=col.astype(np.uint32), aggregate=agg[:na].astype(np.uint32),
                        target=tgt[:nt]))
    R.refd_hierarchy_free(h)
    return out


def main(reference: Path, write: bool = True) -> dict:
    """Every fixture below; written to tests/golden/ when `write`, returned either way
    (file name -> arrays, or the digests' dictionary for golden.json)."""
    R = load(reference)
    made: dict = {}

    def save(name: str, **arrays):
        made[name] = arrays
        if write:
            np.savez_compressed(HERE / name, **arrays)

    rng = np.random.default_rng(20261203)
    meta = {"radius_m": RADIUS, "mesh_sha256": {}, "hierarchy_sha256": {}}

    # ---- meshes: full arrays at L0-L2, hashes up to L8 --------------------------------
    for level in range(0, 9):
        m = R.refd_mesh_new(level, RADIUS)
        a = mesh_arrays(R, m)
        meta["mesh_sha256"][str(level)] = {k: sha(v) for k, v in a.items()}
        if level <= 2:
            save(f"mesh_L{level}.npz", **a)
        if level >= 3:
            hl = hierarchy(R, m)
            meta["hierarchy_sha256"][str(level)] = [{k: sha(v) for k, v in lv.items()} | {"rows": int(len(lv["offset"]) - 1)}
                                                    for lv in hl]
        R.refd_mesh_free(P_(m))
        print("mesh", level, flush=True)

    # ---- operators at L4 (finite_volume.cpp) ------------------------------------------
    m = P(R.refd_mesh_new(4, RADIUS))
    a = mesh_arrays(R, m)
    n, e = len(a["area_m2"]), len(a["edge_length_m"])
    x64 = rng.standard_normal(n)
    f64 = rng.standard_normal(e)
    x32 = rng.standard_normal(n).astype(np.float32)
    f32 = rng.standard_normal(e).astype(np.float32)
    out = {"x64": x64, "flux64": f64, "x32": x32, "flux32": f32}
    for name, xin, dt in (("64", x64, np.float64), ("32", x32, np.float32)):
        lap, ge, gn = np.empty(n, dt), np.empty(n, dt), np.empty(n, dt)
        getattr(R, f"refd_laplacian_f{name}")(m, p(xin), p(lap))
        getattr(R, f"refd_gradient_f{name}")(m, p(xin), p(ge), p(gn))
        div = np.empty(n, dt)
        getattr(R, f"refd_divergence_f{name}")(m, p(f64 if name == "64" else f32), p(div))
        out.update({f"laplacian{name}": lap, f"east{name}": ge, f"north{name}": gn, f"divergence{name}": div})
    t = 288.0 + rng.normal(0, 10, n)
    ds = np.empty(n)
    R.refd_diffusion_source(m, 4e13, p(t), p(ds))
    out.update({"temperature": t, "diffusion_source": ds, "conductance": 4e13})
    save("operators_L4.npz", **out)

    # ---- Newton driver with a linear response at L4 (test_heat_transport.cpp:80-107 style)
    base = 250.0 + 50.0 * rng.random(n)
    slope = np.where(np.arange(n) % 5 == 0, 0.0, 0.01 + 0.2 * rng.random(n))
    K = 0.5 * RADIUS * RADIUS
    mean, src, stats = np.empty(n), np.empty(n), np.empty(6)
    R.refd_solve_linear(m, K, p(base), p(slope), 1e-6, 1e-6, 4, p(mean), p(src), p(stats))
    save("newton_L4.npz", base=base, slope=slope, conductance=K, cg_tolerance=1e-6,
                        newton_tolerance=1e-6, mean=mean, source=src, stats=stats)

    # insolation at L4 (substep_forcing.cpp) and its nodes
    ins = np.empty(n, np.float32)
    R.refd_insolation(m, 0, p(ins))
    nodes = np.empty(80)
    R.refd_insolation_nodes(0, p(nodes))
    save("insolation_L4.npz", insolation=ins, nodes=nodes.reshape(16, 5))
    R.refd_mesh_free(m)

    # ---- multigrid + PCG at L5 with the heat-step matrix ---------------------------------
    m = P(R.refd_mesh_new(5, RADIUS))
    a = mesh_arrays(R, m)
    n = len(a["area_m2"])
    C_heat, kappa, dt = 4e7, 1e6, 31_556_925.216 / 12.0
    K = C_heat * kappa
    s = np.full(n, dt / C_heat)
    lat = np.arcsin(a["center"][:, 2])
    t0 = 288.0 - 40.0 * np.sin(lat) ** 2 + rng.normal(0, 0.5, n)
    ins = np.empty(n, np.float32)
    R.refd_insolation(m, 0, p(ins))
    S = 0.7 * ins.astype(np.float64) - (203.3 + 2.09 * (t0 - 273.15))
    rhs = a["area_m2"] / s * t0 + a["area_m2"] * S
    diag = a["area_m2"] / s + K * a["graph_weight_sum"]
    off = -K * a["graph_weight"]
    h = P(R.refd_hierarchy_new(m))
    R.refd_hierarchy_set_matrix(h, p(diag), p(off))
    galerkin = {}
    for i in range(int(R.refd_hierarchy_level_count(h))):
        sz = np.zeros(4, np.uint64)
        R.refd_hierarchy_level_sizes(h, C.c_uint64(i), p(sz))
        rows, nnz, na, nt = (int(x) for x in sz)
        o, c = np.zeros(rows + 1, np.int64), np.zeros(nnz, np.int64)
        ag, tg = np.zeros(max(na, 1), np.int64), np.zeros(max(nt, 1), np.int64)
        dg, vl = np.zeros(rows), np.zeros(nnz)
        R.refd_hierarchy_level(h, C.c_uint64(i), p(o), p(c), p(ag), p(tg), p(dg), p(vl))
        galerkin[f"diag{i}"] = dg
        galerkin[f"off{i}"] = vl
    vrhs = rng.standard_normal(n) * 1e12
    vout = np.empty(n)
    R.refd_hierarchy_vcycle(h, m, p(vrhs), p(vout))
    R.refd_hierarchy_free(h)
    x = np.empty(n)
    it = R.refd_pcg(m, K, p(s), p(rhs), 1e-12, 2000, 1, p(x))
    save("heatstep_L5.npz", t0=t0, source=S, insolation=ins, heat_capacity=C_heat,
                        diffusivity=kappa, dt=dt, rhs=rhs, vcycle_rhs=vrhs, vcycle_out=vout, pcg_x=x,
                        pcg_iterations=it, pcg_tolerance=1e-12, **galerkin)
    R.refd_mesh_free(m)

    # ---- column radiation at N = 4 and N = 8 (the reference's maximum) -------------------
    g = R.refd_surface_gravity_earth()
    consts = np.zeros(6)
    R.refd_earth_like_constants(p(consts))
    cols = 256
    col_out = {"gravity": g, "constants": consts}
    for N in (4, 8):
        ps = 1e5 + rng.normal(0, 1500, cols)
        ts = 250.0 + 60.0 * rng.random(cols)
        sigma = 1.0 - (np.arange(N) + 0.5) / N
        temp = ts[None, :] * sigma[:, None] ** (287.04 * 6.5e-3 / g)
        q = np.empty((N, cols))
        for k in range(N):
            for c in range(cols):
                q[k, c] = 0.8 * R.refd_saturation_specific_humidity(temp[k, c], sigma[k] * ps[c])
        frac = rng.random((N, cols))
        frac[:, ::7] = 0.0                   # clear layers
        frac[0, 3::11] = 1.5                 # overcast (f capped at 1)
        ql = frac * consts[2] / (ps[None, :] / (g * N))
        eps, absb, fr, refl = (np.empty((N, cols)) for _ in range(4))
        sc = np.empty((5, cols))
        for c in range(cols):
            e1, a1, f1, r1, s1 = np.empty(N), np.empty(N), np.empty(N), np.empty(N), np.empty(5)
            rc = R.refd_column_radiation(N, p(np.ascontiguousarray(temp[:, c])), p(np.ascontiguousarray(q[:, c])),
                                         p(np.ascontiguousarray(ql[:, c])), float(ts[c]), float(ps[c]), g, p(consts),
                                         p(e1), p(a1), p(f1), p(r1), p(s1))
            assert rc == 0
            eps[:, c], absb[:, c], fr[:, c], refl[:, c], sc[:, c] = e1, a1, f1, r1, s1
        col_out.update({f"temperature{N}": temp, f"humidity{N}": q, f"cloud_water{N}": ql, f"surface_temperature{N}": ts,
                        f"surface_pressure{N}": ps, f"emissivity{N}": eps, f"absorbed{N}": absb, f"fraction{N}": fr,
                        f"reflectance{N}": refl, f"scalars{N}": sc})
    save("column.npz", **col_out)

    # ---- saturation (saturation.cpp) ------------------------------------------------------
    T = np.linspace(180.0, 320.0, 57)
    Pp = np.array([5e3, 2e4, 5e4, 8e4, 1e5])
    qs = np.array([[R.refd_saturation_specific_humidity(tt, pp) for pp in Pp] for tt in T])
    save("saturation.npz", temperature=T, pressure=Pp, qsat=qs)

    made["golden.json"] = meta
    if write:
        (HERE / "golden.json").write_text(json.dumps(meta, indent=1, sort_keys=True))
        print("golden fixtures written")
    return made


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    sys.path.insert(0, str(ROOT))
    from oracle.build import reference_root

    reference = reference_root(args[0] if args else None)
    if reference is None:
        raise SystemExit("name the reference checkout: make_golden.py <path> (or set PLANETSIM_REFERENCE)")
    if "--quartic" in sys.argv:   # only the nonlinear-transport fixture
        quartic_cases(load(reference))
        print("quartic fixture written")
    elif "--agglomeration" in sys.argv:   # only the agglomerated-graph fixture
        agglomeration_cases(load(reference))
        print("agglomeration fixture written")
    elif "--nonsym" in sys.argv:   # only the non-symmetric solves' fixture
        nonsym_cases(load(reference))
        print("nonsym fixture written")
    else:
        main(reference)
        quartic_cases(load(reference))
        agglomeration_cases(load(reference))
        nonsym_cases(load(reference))

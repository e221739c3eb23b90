"""The non-symmetric transport solves on the GPU against the reference's own (golden
vectors from the reference, tests/golden/make_golden.py --nonsym):

- block ILU(0) factor + solve: bit-identical to the reference's IncompleteLU;
- advection_diffusion_source: bit-identical, with and without the eddies' latent heat;
- solve_implicit_tracer on the agglomerated L3 graph (3 layers, column-balanced and
  divergent fluxes; 2 layers, eddies only) and the L3 mesh graph: the reference test's
  gates (mass conserved to 1e-13, non-negative, residual <= 1e-10, a uniform field kept
  to 1e-9 under balanced fluxes, no clipping) and the reference's solution to 1e-9 of the
  field (both solve to a 1e-12 relative residual, reduced in a different order);
- solve_implicit_advection_diffusion on the L3 graph (diffusion only, advection, advection
  with latent heat): the reference test's gates and the reference's H to 1e-5 W/m^2
  (both stop at 1e-6 W/m^2); a device response gives the host response's bits;
- at L5 (tracer on the agglomerated graph with 6 layers, the coupled solve on the mesh
  graph) against the oracle's restatements, themselves pinned bit-for-bit to the
  reference."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

CP = 1004.64
RADIUS = 6.371e6


def graph_of(planet):
    import planet_game_gb300 as pg

    g = pg.mesh_transport_graph(planet)
    return g.offset.astype(np.int64), g.neighbour.astype(np.int64), g.area_m2, g.weight


def full_fluxes(planet, half, layers):
    """Antisymmetric flows from their a < b entries ([layers][faces], CSR order)."""
    off, nb, _, _ = graph_of(planet)
    E = len(nb)
    rows = np.repeat(np.arange(len(off) - 1), np.diff(off))
    upper = np.nonzero(rows < nb)[0]
    rev = np.empty(E, dtype=np.int64)
    for k in range(E):
        b = nb[k]
        rev[k] = off[b] + int(np.nonzero(nb[off[b]:off[b + 1]] == rows[k])[0][0])
    out = np.zeros((layers, E))
    out[:, upper] = half
    out[:, rev[upper]] = -half
    return out.ravel()


@pytest.fixture(scope="module")
def planets():
    import planet_game_gb300 as pg

    return {"mesh": pg.make_icosphere(3, RADIUS), "agg": pg.agglomerated_transport_graph(3, RADIUS)}


def test_block_ilu_bit_identical(planets):
    import planet_game_gb300 as pg

    g = golden("nonsym.npz")
    off, nb, _, _ = graph_of(planets["mesh"])
    lu = pg.IncompleteLU(off, nb, g["ilu_diag"], g["ilu_off"], g["ilu_blocks"])
    assert np.array_equal(lu.solve(g["ilu_x"]), g["ilu_y"])
    with pytest.raises(pg.GB300Error, match="zero pivot"):
        pg.IncompleteLU(off, nb, np.zeros(len(g["ilu_diag"])), g["ilu_off"], g["ilu_blocks"])


def test_advection_diffusion_source_bit_identical(planets):
    import planet_game_gb300 as pg

    g = golden("nonsym.npz")
    p = planets["mesh"]
    _, _, area, weight = graph_of(p)
    flux = full_fluxes(p, g["flux"], 3)
    for tag, latent in (("dry", None), ("latent", g["src_latent"])):
        tr = pg.AdvectionDiffusion(3, 0.5 * RADIUS * RADIUS * weight, flux, CP, latent)
        eddy, adv = pg.advection_diffusion_source(p, tr, g["src_mean"], g["src_energy"])
        assert np.array_equal(eddy, g[f"src_eddy_{tag}"]) and np.array_equal(adv, g[f"src_adv_{tag}"])
    # energy conservation of the advective part
    assert abs(np.sum(area * adv)) <= 1e-12 * np.sum(np.abs(area * adv))


@pytest.mark.parametrize("tag", ["bal", "div", "eddy", "l3"])
def test_tracer_matches_the_reference(planets, tag):
    import planet_game_gb300 as pg

    g = golden("nonsym.npz")
    layers = int(g[f"tr_{tag}_layers"])
    p = planets["agg"] if int(g[f"tr_{tag}_agg"]) else planets["mesh"]
    _, nb, area, _ = graph_of(p)
    n = p.cell_count
    tr = pg.AdvectionDiffusion(layers, np.full(len(nb), float(g[f"tr_{tag}_eddy"])),
                               full_fluxes(p, g[f"tr_{tag}_flux"], layers), CP)
    mass = area * 100000.0 / (9.81 * layers)
    c0 = g[f"tr_{tag}_in"]
    r = pg.solve_implicit_tracer(p, tr, mass, c0, 2.63e6)
    ref, stats = g[f"tr_{tag}_out"], g[f"tr_{tag}_stats"]
    total = lambda c: np.sum(np.tile(mass, layers) * c)   # noqa: E731
    assert abs(total(r.tracer) - total(c0)) <= 1e-13 * total(c0)
    assert r.tracer.min() >= 0.0 and r.relative_residual <= 1e-10 and r.clipped_kg <= 1e-12 * total(c0)
    assert abs(r.iterations - stats[0]) <= 2
    assert r.column_divergence_kg_s == pytest.approx(stats[3], rel=1e-12, abs=1e-3)
    assert np.max(np.abs(r.tracer - ref)) <= 1e-9 * np.max(np.abs(ref))
    if tag == "bal":   # a uniform tracer stays uniform under column-balanced fluxes
        kept = pg.solve_implicit_tracer(p, tr, mass, np.full(layers * n, 0.01), 2.63e6)
        assert np.max(np.abs(kept.tracer / 0.01 - 1.0)) <= 1e-9
    if tag == "eddy":  # the eddies alone smooth
        assert np.ptp(r.tracer) < 0.5 * np.ptp(c0)


def column(g, source):
    """The reference test's column (test_advection_diffusion.cpp:73-104) on the GPU's
    quartic kernel: theta, its slope, s_l and ds_l/dh."""
    import planet_game_gb300 as pg

    q = pg.QuarticResponse(float(g["ad_a"]), g["ad_b"], hold_stride=0)
    x, s = (v.cpu().numpy() for v in pg.quartic_response(q, source))
    eps, phi = g["ad_eps"], g["ad_phi"]
    energy = np.concatenate([CP * x * (1.0 + e) + f for e, f in zip(eps, phi)])
    energy_slope = np.concatenate([CP * s * (1.0 + e) for e in eps])
    return x, s, energy, energy_slope


@pytest.mark.parametrize("tag", ["diff", "adv", "lat"])
def test_advection_diffusion_solve_matches_the_reference(planets, tag):
    import planet_game_gb300 as pg

    g = golden("nonsym.npz")
    p = planets["mesh"]
    _, nb, area, weight = graph_of(p)
    flux = full_fluxes(p, g["flux"], 3) if tag != "diff" else np.zeros(3 * len(nb))
    tr = pg.AdvectionDiffusion(3, 0.5 * RADIUS * RADIUS * weight, flux, CP,
                               g["ad_lat_latent"] if tag == "lat" else None)
    settings = {"cg_relative_tolerance": 1e-6, "newton_tolerance_W_m2": 1e-6}
    r = pg.solve_implicit_advection_diffusion(p, tr, g["ad_floor"], lambda h: column(g, h), settings=settings)
    stats = g[f"ad_{tag}_stats"]
    assert r.consistency_residual_W_m2 <= 1e-6
    assert abs(r.sum_W) <= 1e-12 * r.absolute_sum_W
    assert abs(r.newton_iterations - stats[0]) <= 1
    assert np.max(np.abs(r.source_W_m2 - g[f"ad_{tag}_source"])) <= 1e-5
    assert np.max(np.abs(r.mean_K - g[f"ad_{tag}_mean"])) <= 1e-6
    if tag == "adv":
        assert r.advective_absolute_sum_W > 0.1 * r.eddy_absolute_sum_W
    if tag == "diff":   # without fluxes it is the implicit transport solve
        q = pg.QuarticResponse(float(g["ad_a"]), g["ad_b"], hold_stride=0)
        heat = pg.solve_implicit_transport(p, 0.5 * RADIUS * RADIUS, g["ad_floor"], q, settings=settings)
        assert np.max(np.abs(r.source_W_m2 - heat.source_W_m2)) <= 1e-5


class _DeviceArray:
    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False), "version": 3,
                                         "stream": None}


def test_device_response_equals_host_response(planets):
    import torch

    import planet_game_gb300 as pg

    g = golden("nonsym.npz")
    p = planets["mesh"]
    _, _, _, weight = graph_of(p)
    tr = pg.AdvectionDiffusion(3, 0.5 * RADIUS * RADIUS * weight, full_fluxes(p, g["flux"], 3), CP)
    host = pg.solve_implicit_advection_diffusion(p, tr, g["ad_floor"], lambda h: column(g, h))

    def device_column(nodes, layers, source, mean, slope, energy, energy_slope, stream):
        h = torch.as_tensor(_DeviceArray(source, nodes), device="cuda").cpu().numpy()
        x, s, e, es = column(g, h)
        for ptr, values, count in ((mean, x, nodes), (slope, s, nodes), (energy, e, nodes * layers),
                                   (energy_slope, es, nodes * layers)):
            torch.as_tensor(_DeviceArray(ptr, count), device="cuda").copy_(torch.as_tensor(values))

    dev = pg.solve_implicit_advection_diffusion(p, tr, g["ad_floor"], device_column, device=True)
    assert dev.newton_iterations == host.newton_iterations
    assert np.array_equal(dev.source_W_m2, host.source_W_m2)


def test_invalid_inputs_are_refused(planets):
    import planet_game_gb300 as pg

    g = golden("nonsym.npz")
    p = planets["mesh"]
    _, nb, _, weight = graph_of(p)
    cond = 0.5 * RADIUS * RADIUS * weight
    cond[0] = -1.0
    tr = pg.AdvectionDiffusion(3, cond, np.zeros(3 * len(nb)), CP)
    with pytest.raises(ValueError, match="conductances"):
        pg.solve_implicit_advection_diffusion(p, tr, g["ad_floor"], lambda h: column(g, h))
    with pytest.raises(ValueError):
        pg.solve_implicit_tracer(p, tr, np.ones(p.cell_count + 1), np.zeros(3 * p.cell_count), 1.0)


def test_tracer_and_coupled_solve_against_the_oracle_at_l5():
    """Larger cases against the oracle's restatement (pinned bit-for-bit to the reference):
    the tracer on the L5 mesh's agglomerated graph with 6 layers, the coupled solve on the
    L5 graph; the tracer field to 1e-9, the coupled H to 1e-5 W/m^2."""
    import planet_game_gb300 as pg
    from oracle import oracle as O
    from planet_game_gb300 import workloads as W

    p = pg.agglomerated_transport_graph(5, RADIUS)
    g = pg.mesh_transport_graph(p)
    layers = 6
    flux = W.antisymmetric_layer_fluxes(g.offset, g.neighbour, layers, 2e9, seed=51, column_balanced=False)
    cond = np.full(len(g.neighbour), 2e8)
    mass = g.area_m2 * 100000.0 / (9.81 * layers)
    c0 = W.tracer_field(layers * p.cell_count, seed=52)
    r = pg.solve_implicit_tracer(p, pg.AdvectionDiffusion(layers, cond, flux, CP), mass, c0, 2.63e6)
    ref, stats = O.solve_implicit_tracer(g.offset, g.neighbour, layers, cond, flux, CP, mass, c0, 2.63e6)
    assert r.relative_residual <= 1e-10 and stats[1] <= 1e-10
    assert np.max(np.abs(r.tracer - ref)) <= 1e-9 * np.max(np.abs(ref))

    m = pg.make_icosphere(5, RADIUS)
    g5 = pg.mesh_transport_graph(m)
    flux5 = W.antisymmetric_layer_fluxes(g5.offset, g5.neighbour, 3, 5e9, seed=53, column_balanced=True)
    cond5 = 0.5 * RADIUS * RADIUS * g5.weight
    a, radiative = 3.0e5 / (30.0 * 86400.0), 0.75 * 0.97 * 5.670374419e-8
    b, floor = W.quartic_column(a, radiative, m.cell_count, seed=54)
    eps, phi = np.array([0.0, -0.08, -0.16]), np.array([3.0e4, 4.5e4, 7.0e4])

    def column(h):
        q = pg.QuarticResponse(a, b, radiative, hold_stride=0)
        x, s = (v.cpu().numpy() for v in pg.quartic_response(q, h))
        return x, s, np.concatenate([CP * x * (1.0 + e) + f for e, f in zip(eps, phi)]), \
            np.concatenate([CP * s * (1.0 + e) for e in eps])

    settings = {"cg_relative_tolerance": 1e-6, "newton_tolerance_W_m2": 1e-6}
    got = pg.solve_implicit_advection_diffusion(m, pg.AdvectionDiffusion(3, cond5, flux5, CP), floor, column,
                                                settings=settings)
    src, _, _, ostats = O.solve_implicit_advection_diffusion(O.OracleMesh(m.arrays()), 3, cond5, flux5, None, CP, a,
                                                             b, eps, phi, floor)
    assert got.consistency_residual_W_m2 <= 1e-6 and ostats[2] <= 1e-6
    assert np.max(np.abs(got.source_W_m2 - src)) <= 1e-5

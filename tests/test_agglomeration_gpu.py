"""The transport on the agglomerated graph (one mesh level coarser, nodes with their fine
cells' summed areas) on the GPU, against the oracle and the reference's own solve:

- the diffusion source and the group means are bit-identical to the oracle / the
  reference's loop (same summation order); group scatter is exact;
- a transport sub-step on the agglomerated L6 planet meets the solve's gates and matches
  the FP64 oracle to 2e-6 K (the step's bar); a batch mixing agglomerated and plain
  planets gives each the same bits as alone;
- the production pattern (fine-cell quartic response at the group's source, group means,
  the nonlinear solve on the agglomerated graph) matches the reference's own solve to
  1e-5 K and 1e-3 W/m^2, both stopping at 1e-6 W/m^2."""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SETTINGS = {"cg_relative_tolerance": 1e-6, "newton_tolerance_W_m2": 1e-6}


@pytest.fixture(scope="module")
def agg():
    import planet_game_gb300 as pg

    cache = {}

    def get(level, radius=6.371e6):
        if (level, radius) not in cache:
            cache[(level, radius)] = pg.agglomerated_transport_graph(level, radius)
        return cache[(level, radius)]

    return get


def test_diffusion_source_uses_the_group_areas(agg):
    import planet_game_gb300 as pg

    p = agg(5)
    a = p.arrays()
    t = 250.0 + 40.0 * np.random.default_rng(1).standard_normal(p.cell_count)
    got = pg.diffusion_source(p, 0.5 * 6.371e6 ** 2, t)
    ref = O.OracleMesh(a).diffusion_source(0.5 * 6.371e6 ** 2, t)
    assert np.array_equal(got, ref)
    assert not np.array_equal(a["graph_area_m2"], a["area_m2"])


def test_group_mean_and_scatter(agg, meshes):
    import planet_game_gb300 as pg

    p = agg(5)
    groups = p.group_of_cell()
    area = meshes(5).arrays()["area_m2"]
    graph_area = p.arrays()["graph_area_m2"]
    rng = np.random.default_rng(2)
    u, v = 280.0 + rng.standard_normal(p.fine_cell_count), rng.random(p.fine_cell_count)
    mu, mv = pg.group_mean(p, u, v)
    su, sv = np.zeros(p.cell_count), np.zeros(p.cell_count)
    for c in range(p.fine_cell_count):           # the reference's loop: members in cell order
        su[groups[c]] += area[c] * u[c]
        sv[groups[c]] += area[c] * v[c]
    assert np.array_equal(mu, su / graph_area) and np.array_equal(mv, sv / graph_area)
    assert np.array_equal(pg.group_mean(p, u), mu)
    h = rng.standard_normal(p.cell_count)
    assert np.array_equal(pg.group_scatter(p, h), h[groups])
    with pytest.raises(ValueError):
        pg.group_mean(p, u[:-1])
    with pytest.raises((ValueError, pg.GB300Error), match="agglomerated"):
        pg.group_scatter(meshes(4), np.zeros(meshes(4).cell_count))


@pytest.mark.parametrize("precision,method", [("fp64", "bicgstab"), ("mixed", "bicgstab"), ("mixed", "pcg")])
def test_transport_step_on_the_agglomerated_graph(agg, precision, method):
    import planet_game_gb300 as pg
    from planet_game_gb300 import workloads as W

    p = agg(6)
    inp = W.step_inputs(p, seed=6)
    t_new, H, rep = pg.transport_step(p, inp.t0, inp.source, inp.heat_capacity, inp.dt, inp.conductance,
                                      precision=precision, method=method)
    assert rep.status == 0 and rep.relative_residual <= 1e-10 and rep.closure <= 1e-12
    a = p.arrays()
    ref = O.OracleHierarchy(O.OracleMesh(a)).transport_step(inp.conductance, inp.heat_capacity, inp.dt, inp.t0,
                                                             inp.source, tol=1e-13)
    assert np.max(np.abs(t_new - ref["t_new"])) <= 2e-6
    s = inp.dt / inp.heat_capacity
    ga = a["graph_area_m2"]
    gain = np.sum(ga * (t_new - inp.t0) / s)
    assert abs(gain - np.sum(ga * inp.source)) <= 1e-12 * np.sum(np.abs(ga * inp.source))


def test_batch_of_agglomerated_and_plain_planets_equals_solo(agg, meshes):
    import planet_game_gb300 as pg
    from planet_game_gb300 import workloads as W

    ms = [agg(6), meshes(5), agg(4, 4.1e6), meshes(3)]
    inputs = [W.step_inputs(m, seed=20 + i) for i, m in enumerate(ms)]
    batch = pg.Batch(ms)
    outs, reps = batch.transport_step([i.t0 for i in inputs], [i.source for i in inputs], inputs[0].heat_capacity,
                                      inputs[0].dt, conductance=inputs[0].conductance, precision="mixed")
    for m, inp, out, rep in zip(ms, inputs, outs, reps):
        solo, _, srep = pg.transport_step(m, inp.t0, inp.source, inp.heat_capacity, inp.dt, inp.conductance,
                                          precision="mixed")
        assert rep.status == 0 and rep.iterations == srep.iterations
        assert np.array_equal(out, solo)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("factor", [1, 10])
def test_production_response_matches_the_reference(agg, factor, precision):
    import planet_game_gb300 as pg

    g = golden("agglomeration.npz")
    p = agg(5)
    a, b = float(g["qa"]), g["qb"]

    def response(h):
        mean_f, slope_f = O.quartic_response(a, b, pg.group_scatter(p, h))
        return pg.group_mean(p, mean_f, slope_f)

    r = pg.solve_implicit_transport(p, float(g[f"qK{factor}"]), g[f"qfloor{factor}"], response,
                                    settings=SETTINGS, precision=precision)
    assert r.consistency_residual_W_m2 <= 1e-6
    assert abs(r.sum_W) <= 1e-13 * r.absolute_sum_W and r.dissipation_W_K <= 0.0
    assert np.max(np.abs(r.mean_K - g[f"qmean{factor}"])) <= 1e-5
    assert np.max(np.abs(r.source_W_m2 - g[f"qsource{factor}"])) <= 1e-3
    assert abs(r.newton_iterations - g[f"qstats{factor}"][0]) <= 2

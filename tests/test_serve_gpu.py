"""The continuous-batching request loop: every served result equals the same step run
alone (bit for bit: planets never influence each other in a batch) and the oracle's solve
of the same step, lanes overlap, and HBM-budget admission evicts idle lanes without losing
requests."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def population():
    torch = pytest.importorskip("torch")
    from planet_game_gb300 import serve

    return serve.build_population(per_level=3, levels=(4, 5, 6), seed=5, device=torch.device("cuda", 0))


def test_served_results_equal_the_same_step_alone(population):
    import planet_game_gb300 as pg
    from planet_game_gb300 import serve
    from planet_game_gb300 import workloads as W

    trace = W.poisson_trace(120, 2000.0, seed=3, weights=((4, .4), (5, .4), (6, .2)), planets_per_level=3)
    reqs = serve.make_requests(trace, population, seed=4)
    srv = serve.Server(population, precision="mixed", keep_inputs=True, autotune=False)
    try:
        srv.run_trace(reqs, realtime=True)
    finally:
        srv.close()
    assert all(r.status == 0 for r in reqs)
    assert sum(l.rounds for l in srv.lanes.values()) < len(reqs)     # requests were batched together
    for r in reqs:
        p = population[r.level][r.planet]
        alone, _, rep = pg.transport_step(p.mesh, r.t_in, r.source, p.heat_capacity, p.dt, p.conductance,
                                          edge_conductance=p.edge_conductance, precision="mixed")
        assert rep.status == 0
        assert np.array_equal(alone, r.result)
    s = serve.summarize(reqs)
    assert s["ok"] == len(reqs) and s["p99_ms"] >= s["p50_ms"] > 0


def test_served_results_against_the_oracle(population):
    """Every result of a short trace through the tuned lanes against the oracle (the
    reference's FP64 PCG + SGS V-cycle solve, restated) from the same state and source."""
    from oracle import oracle as O
    from planet_game_gb300 import serve
    from planet_game_gb300 import workloads as W

    trace = W.poisson_trace(40, 2000.0, seed=31, weights=((4, .4), (5, .4), (6, .2)), planets_per_level=3)
    reqs = serve.make_requests(trace, population, seed=32)
    srv = serve.Server(population, precision="mixed", keep_inputs=True)
    try:
        srv.run_trace(reqs, realtime=True)
    finally:
        srv.close()
    assert all(r.status == 0 for r in reqs)
    oracles = {}
    for r in reqs:
        p = population[r.level][r.planet]
        if (r.level, r.planet) not in oracles:
            om = O.OracleMesh(p.mesh.arrays())
            oracles[(r.level, r.planet)] = (om, O.OracleHierarchy(om))
        om, h = oracles[(r.level, r.planet)]
        ref = h.transport_step(0.0, p.heat_capacity, p.dt, r.t_in, r.source, tol=1e-13,
                               edge_g=om.directed_conductance(p.edge_conductance))
        assert np.max(np.abs(r.result - ref["t_new"])) <= 2e-6


def test_tuned_lanes_equal_the_planet_alone_with_the_lane_tuning(population):
    """Lanes autotune at admission; a result equals the planet stepped alone in a one-planet
    batch that carries the lane's tuning."""
    import planet_game_gb300 as pg
    from planet_game_gb300 import serve
    from planet_game_gb300 import workloads as W

    trace = W.poisson_trace(60, 2000.0, seed=13, weights=((4, .4), (5, .4), (6, .2)), planets_per_level=3)
    reqs = serve.make_requests(trace, population, seed=14)
    srv = serve.Server(population, precision="mixed", keep_inputs=True)
    srv.prepare()
    assert set(srv.tunings) == {4, 5, 6}
    try:
        srv.run_trace(reqs, realtime=True)
    finally:
        srv.close()
    assert all(r.status == 0 for r in reqs)
    alone = {}
    for r in reqs:
        p = population[r.level][r.planet]
        key = (r.level, r.planet)
        if key not in alone:
            alone[key] = pg.Batch([p.mesh])
            alone[key].set_tuning(srv.tunings[r.level])
        out, reps = alone[key].transport_step([r.t_in], [r.source], p.heat_capacity, p.dt, conductance=p.conductance,
                                              edge_conductance=[p.edge_conductance], precision="mixed")
        assert reps[0].status == 0
        assert np.array_equal(out[0], r.result)


def test_budget_admission_evicts_idle_lanes(population):
    from planet_game_gb300 import serve
    from planet_game_gb300 import workloads as W

    trace = W.poisson_trace(60, 500.0, seed=8, weights=((4, .5), (5, .3), (6, .2)), planets_per_level=3)
    reqs = serve.make_requests(trace, population, seed=9)
    one_lane = max(sum(p.mesh.cell_count for p in population[l]) for l in (4, 5, 6)) * 700
    srv = serve.Server(population, budget_bytes=one_lane * 1.2, precision="mixed")
    try:
        srv.run_trace(reqs, realtime=True)
    finally:
        srv.close()
    assert all(r.status == 0 for r in reqs)
    assert srv.evictions > 0
    assert srv.resident_bytes <= one_lane * 1.2


def test_one_at_a_time_comparator_matches_the_oracle_gates(population):
    from planet_game_gb300 import serve
    from planet_game_gb300 import workloads as W

    trace = W.poisson_trace(12, 1000.0, seed=1, weights=((4, .5), (5, .5)), planets_per_level=3)
    reqs = serve.make_requests(trace, population, seed=2)
    serve.OneAtATime(population).run_trace(reqs, realtime=False)
    assert all(r.status == 0 for r in reqs)
    assert serve.summarize(reqs)["sub_steps_per_s"] > 0


def test_consecutive_traces_each_wait_for_all_of_their_own_requests(population):
    """The server's completion count runs across traces: a second trace on the same server
    returns only once every one of its own requests is done."""
    from planet_game_gb300 import serve
    from planet_game_gb300 import workloads as W

    srv = serve.Server(population, precision="mixed", autotune=False)
    try:
        first = serve.make_requests(W.poisson_trace(30, 5000.0, seed=21, weights=((4, .5), (5, .5)),
                                                    planets_per_level=3), population, seed=22)
        srv.run_trace(first, realtime=False)
        second = serve.make_requests(W.poisson_trace(90, 5000.0, seed=23, weights=((4, .3), (5, .3), (6, .4)),
                                                     planets_per_level=3), population, seed=24)
        srv.run_trace(second, realtime=False)
        assert all(r.status == 0 and r.done_s >= 0.0 for r in first + second)
    finally:
        srv.close()

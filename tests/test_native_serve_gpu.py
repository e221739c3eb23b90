"""The library's own serving loop (psgb_server_*, the C++ request loop a caller of the
drop-in uses) on the GPU: a short Poisson trace, each result bit-identical to the planet
stepped alone from the same state and to the Python loop over the same batch entry points
(both untuned, so both run the default smoother)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_native_loop_equals_the_planet_alone_and_the_python_loop():
    torch = pytest.importorskip("torch")
    import planet_game_gb300 as pg
    from planet_game_gb300 import serve
    from planet_game_gb300 import workloads as W

    dev = torch.device("cuda", 0)
    pop = serve.build_population(per_level=2, levels=(4, 5, 6), seed=21, device=dev)
    initial = {(l, i): p.state.cpu().numpy() for l, ps in pop.items() for i, p in enumerate(ps)}
    trace = W.poisson_trace(48, 2000.0, seed=22, weights=((4, .4), (5, .4), (6, .2)), planets_per_level=2)
    reqs = serve.make_requests(trace, pop, seed=23)

    native = {}
    with serve.NativeServer(budget_bytes=150e9, precision="mixed", autotune=False) as srv:
        ids = {key: srv.add_planet(key[0], pop[key[0]][key[1]].radius, pop[key[0]][key[1]].heat_capacity,
                                   pop[key[0]][key[1]].dt, pop[key[0]][key[1]].conductance, t0,
                                   pop[key[0]][key[1]].edge_conductance)
               for key, t0 in initial.items()}
        pending = [(k, srv.submit(ids[(r.level, r.planet)], r.source)) for k, r in enumerate(reqs)]
        for k, rid in pending:
            r = reqs[k]
            out, rep = srv.wait(rid, ids[(r.level, r.planet)], timeout_s=120.0)
            assert rep.solve.status == 0 and rep.closure <= 1e-12
            native[k] = out
        stats = srv.stats()
    assert stats["completed"] == len(reqs) and stats["p99_ms"] >= stats["p50_ms"] > 0

    # the planet alone, its requests in order from its initial state
    state = dict(initial)
    for k, r in enumerate(reqs):
        p = pop[r.level][r.planet]
        alone, _, rep = pg.transport_step(p.mesh, state[(r.level, r.planet)], r.source, p.heat_capacity, p.dt,
                                          p.conductance, edge_conductance=p.edge_conductance, precision="mixed")
        assert rep.status == 0
        assert np.array_equal(native[k], alone)
        state[(r.level, r.planet)] = alone

    # the Python loop over the same trace and starting states
    for key, t0 in initial.items():
        pop[key[0]][key[1]].state = torch.from_numpy(t0).to(dev)
    again = serve.make_requests(trace, pop, seed=23)
    py = serve.Server(pop, precision="mixed", autotune=False)
    try:
        py.run_trace(again, realtime=False)
    finally:
        py.close()
    for k, r in enumerate(again):
        assert r.status == 0
        assert np.array_equal(native[k], r.result)

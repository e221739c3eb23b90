"""The L8 multi-right-hand-side case: one 655,362-cell planet, 32 right-hand sides
S_j = S + N(0, 5^2) W/m^2, solved in one batch of 32 instances of the planet, in plain
FP64 (variant A) and with the FP32 inner solve inside FP64 refinement (variant B).

Bars: every solve meets ||b - A x|| <= 1e-10 ||b|| and closure <= 1e-12; the two variants
agree to 1e-6 K (both are 1e-10-residual solutions of the same system, ~300 K values:
measured 3e-7 K); two of the 32 agree with the FP64 CPU oracle (PCG to 1e-13) to 2e-6 K,
the transport step's bar."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

RHS = 32


@pytest.fixture(scope="module")
def l8():
    import planet_game_gb300 as pg
    from planet_game_gb300 import workloads as W

    m = pg.make_icosphere(8, 6.371e6)
    inp = W.step_inputs(m, seed=8)
    sources = W.perturbed_sources(inp.source, RHS, seed=9)
    return m, inp, sources


def test_variants_a_and_b_meet_the_gates_and_agree(l8):
    import planet_game_gb300 as pg

    m, inp, sources = l8
    batch = pg.Batch([m] * RHS)
    out = {}
    for precision in ("fp64", "mixed"):
        t, reps = batch.transport_step([inp.t0] * RHS, list(sources), inp.heat_capacity, inp.dt,
                                       conductance=inp.conductance, precision=precision)
        for r in reps:
            assert r.status == 0 and r.relative_residual <= 1e-10 and r.closure <= 1e-12
        out[precision] = (np.array(t), reps)
    (ta, ra), (tb, rb) = out["fp64"], out["mixed"]
    assert np.max(np.abs(ta - tb)) <= 1e-6
    assert all(r.refinements >= 2 for r in rb)                   # FP32 inner: refinement at work
    print("A refinements", {r.refinements for r in ra}, "inner", sum(r.iterations for r in ra),
          "| B refinements", {r.refinements for r in rb}, "inner", sum(r.iterations for r in rb))
    # against the FP64 CPU oracle on two of the right-hand sides
    om = O.OracleMesh(m.arrays())
    h = O.OracleHierarchy(om)
    for j in (0, RHS - 1):
        ref = h.transport_step(inp.conductance, inp.heat_capacity, inp.dt, inp.t0, sources[j], tol=1e-13)
        assert np.max(np.abs(ta[j] - ref["t_new"])) <= 2e-6
        assert np.max(np.abs(tb[j] - ref["t_new"])) <= 2e-6

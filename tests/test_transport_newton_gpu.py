"""The implicit transport solve with a general (host) tile response, against the reference's
own solve_implicit_transport (golden vectors from the reference, tests/golden/make_golden.py):
the quartic response of the reference's test (heat capacities of a month and of ten minutes,
the test's conductance and ten times it) and its linear response.

Tolerances: both solves stop at max |h - K lap T(h)| <= 1e-6 W/m^2, so the temperatures
agree to well below 1e-5 K and the applied transport to 1e-3 W/m^2 (values ~1e2); the
reference test's gates hold exactly as written there (test_heat_transport.cpp:103-106,
140-144)."""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SETTINGS = {"cg_relative_tolerance": 1e-6, "newton_tolerance_W_m2": 1e-6}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case,factor", [(0, 1), (0, 10), (1, 1), (1, 10)])
def test_quartic_response_matches_the_reference(meshes, case, factor, precision):
    import planet_game_gb300 as pg

    g = golden("newton_quartic_L4.npz")
    key = f"{case}_{factor}"
    a, b, K = float(g[f"a{case}"]), g[f"b{case}"], float(g[f"K{key}"])
    floor = g[f"floor{key}"]
    m = meshes(4)
    calls = []

    def response(h):
        calls.append(1)
        return O.quartic_response(a, b, h)

    r = pg.solve_implicit_transport(m, K, floor, response, settings=SETTINGS, precision=precision)
    ref_stats = g[f"stats{key}"]
    # the reference test's gates
    assert r.consistency_residual_W_m2 <= 1e-6
    assert abs(r.sum_W) <= 1e-13 * r.absolute_sum_W
    assert r.dissipation_W_K <= 0.0
    assert np.all(r.mean_K[::7] <= 273.15)
    before, _ = O.quartic_response(a, b, np.zeros(m.cell_count))
    assert np.ptp(r.mean_K) <= np.ptp(before)
    # against the reference's own solve
    assert np.max(np.abs(r.mean_K - g[f"mean{key}"])) <= 1e-5
    assert np.max(np.abs(r.source_W_m2 - g[f"source{key}"])) <= 1e-3
    assert abs(r.newton_iterations - ref_stats[0]) <= 2
    assert len(calls) >= r.newton_iterations + 1


def test_linear_response_matches_the_reference(meshes):
    import planet_game_gb300 as pg

    g = golden("newton_L4.npz")
    base, slope = g["base"], g["slope"]
    m = meshes(4)
    r = pg.solve_implicit_transport(m, float(g["conductance"]), np.full(m.cell_count, -np.inf),
                                    lambda h: (base + slope * h, slope.copy()), settings=SETTINGS)
    assert r.newton_iterations <= 3 and r.consistency_residual_W_m2 <= 1e-6
    assert abs(r.sum_W) <= 1e-13 * r.absolute_sum_W and r.dissipation_W_K <= 0.0
    assert np.max(np.abs(r.mean_K - g["mean"])) <= 1e-5
    assert np.max(np.abs(r.source_W_m2 - g["source"])) <= 1e-3


def test_errors_reach_the_caller(meshes):
    import planet_game_gb300 as pg

    m = meshes(4)
    floor = np.zeros(m.cell_count)
    with pytest.raises(ValueError, match="conductance"):
        pg.solve_implicit_transport(m, 0.0, floor, lambda h: (h, h))

    class Boom(RuntimeError):
        pass

    def failing(h):
        raise Boom("tile solve failed")

    with pytest.raises(Boom):
        pg.solve_implicit_transport(m, 1e12, floor, failing)

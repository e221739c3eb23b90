"""GPU column radiation (K12) against the reference (N = 4, 8 golden columns) and the
oracle's N-layer restatement (N = 10 config columns). FP64; the only differences come
from the device's expm1/log1p versus the host libm (a few ulps): rtol 1e-13."""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NAMES = ("emissivity", "absorbed", "fraction", "reflectance", "scalars")


def constants_from(g):
    import planet_game_gb300 as pg

    c = g["constants"]
    return pg.column_constants(dry_optical_depth=c[0], vapour_absorption_m2_kg=c[1], in_cloud_water_path_kg_m2=c[2],
                               effective_radius_m=c[3], cloud_asymmetry=c[4], cloud_longwave_absorption_m2_kg=c[5],
                               reference_pressure_Pa=101_325.0, gravity_m_s2=float(g["gravity"]),
                               stefan_boltzmann=5.670374419e-8)


@pytest.mark.parametrize("layers", [4, 8])
def test_column_matches_reference_golden(layers):
    import planet_game_gb300 as pg

    g = golden("column.npz")
    outs = pg.column_radiation(constants_from(g), g[f"temperature{layers}"], g[f"humidity{layers}"],
                               g[f"cloud_water{layers}"], g[f"surface_temperature{layers}"],
                               g[f"surface_pressure{layers}"])
    for got, name in zip(outs, NAMES):
        np.testing.assert_allclose(got, g[f"{name}{layers}"], rtol=1e-13, atol=1e-300, err_msg=name)


def test_ten_layer_columns_on_l6_against_oracle(meshes):
    import planet_game_gb300 as pg
    from planet_game_gb300 import workloads as W

    m = meshes(6)
    inp = W.step_inputs(m, seed=6)
    col = W.column_profiles(inp.t0, 10, seed=6)
    k = pg.column_constants(**W.EARTH_COLUMN)
    outs = pg.column_radiation(k, col.temperature, col.humidity, col.cloud_water, col.surface_temperature,
                               col.surface_pressure)
    ref = O.column_radiation(W.column_constant_vector(), col.temperature, col.humidity, col.cloud_water,
                             col.surface_temperature, col.surface_pressure)
    for got, want, name in zip(outs, ref, NAMES):
        np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-300, err_msg=name)
    # identities: fractions recovered from the cloud water, energy budget of the column
    np.testing.assert_allclose(outs[2], col.cloud_fraction, rtol=1e-12)
    up_surface = W.STEFAN_BOLTZMANN * col.surface_temperature**4
    emission = outs[0] * W.STEFAN_BOLTZMANN * col.temperature**4
    # absorbed + OLR + surface down = surface up + 2 * emission (each layer emits up and down)
    lhs = outs[1].sum(0) + outs[4][1] + outs[4][0]
    rhs = up_surface + 2.0 * emission.sum(0)
    np.testing.assert_allclose(lhs, rhs, rtol=1e-12)


def test_column_edge_cases():
    import planet_game_gb300 as pg
    from planet_game_gb300 import workloads as W

    k = pg.column_constants(**W.EARTH_COLUMN)
    n, L = 5, 3
    t = np.full((L, n), 250.0)
    q = np.array([[0.0, -1e-3, 1e-3, 0.0, 0.01]] * L)      # negative humidity counts as zero
    ql = np.array([[0.0, -1.0, 10.0, 1e-6, 0.0]] * L)      # overcast layer caps f at 1
    outs = pg.column_radiation(k, t, q, ql, np.full(n, 280.0), np.full(n, 1e5))
    ref = O.column_radiation(W.column_constant_vector(), t, q, ql, np.full(n, 280.0), np.full(n, 1e5))
    for got, want in zip(outs, ref):
        np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-300)
    assert np.all(outs[2][:, 2] == 1.0) and np.all(outs[2][:, 0] == 0.0) and np.all(outs[2][:, 1] == 0.0)
    empty = pg.column_radiation(k, np.zeros((L, 0)), np.zeros((L, 0)), np.zeros((L, 0)), np.zeros(0), np.zeros(0))
    assert all(o.size == 0 for o in empty)

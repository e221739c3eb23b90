"""The synthetic workload generators (CPU): spherical harmonics, column profiles, the
planet mix and the serving trace."""
import numpy as np

from conftest import rel_l2


def test_real_harmonics_addition_theorem():
    from planet_game_gb300 import workloads as W

    rng = np.random.default_rng(0)
    u = rng.standard_normal((500, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    Y, _, _ = W.real_harmonics(16, u)
    for l in range(17):
        np.testing.assert_allclose((Y[l] ** 2).sum(0), (2 * l + 1) / (4 * np.pi), rtol=1e-12)


def test_harmonic_gradient_against_finite_differences():
    from planet_game_gb300 import workloads as W

    rng = np.random.default_rng(1)
    u = rng.standard_normal((200, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    coef = W.harmonic_coefficients(16, 3)
    R = 6.371e6
    f, e, n, _ = W._gradient3(coef, 16, u, R)
    east = np.stack([-u[:, 1], u[:, 0], np.zeros(len(u))], 1)
    east /= np.linalg.norm(east, axis=1)[:, None]
    north = np.cross(u, east)
    h = 1e-6

    def fval(v):
        v = v / np.linalg.norm(v, axis=1)[:, None]
        return W._gradient3(coef, 16, v, R)[0]

    fe = (fval(u + h * east) - fval(u - h * east)) / (2 * h * R)
    fn = (fval(u + h * north) - fval(u - h * north)) / (2 * h * R)
    assert np.abs(fe - e).max() <= 1e-8 * np.abs(e).max()
    assert np.abs(fn - n).max() <= 1e-8 * np.abs(n).max()


def test_operators_converge_to_harmonic_fields(meshes):
    """Second-order convergence of the (oracle) operators towards the analytic values,
    the property the GPU operators are gated on."""
    from oracle import oracle as O
    from planet_game_gb300 import workloads as W

    errs = []
    for level in (4, 5, 6):
        m = meshes(level)
        a = m.arrays()
        om = O.OracleMesh(a)
        F = W.harmonic_field(a, m.radius_m, 16, 0)
        w = a["area_m2"]
        ge, gn = om.gradient(F.value)
        errs.append((rel_l2(om.laplacian(F.value), F.laplacian, w), rel_l2(ge, F.east, w),
                     rel_l2(om.divergence(F.edge_flux), F.laplacian, w)))
    for coarse, fine in zip(errs, errs[1:]):
        for c, f in zip(coarse, fine):
            assert f < 0.4 * c   # order ~2: a factor ~4 per level


def test_column_profiles():
    from planet_game_gb300 import workloads as W

    ts = np.array([300.0, 250.0, 220.0])
    col = W.column_profiles(ts, 10, seed=4)
    assert col.temperature.shape == (10, 3)
    assert np.all(np.diff(col.temperature, axis=0) < 0)       # lapse rate: colder aloft
    sigma = 1.0 - (np.arange(10) + 0.5) / 10
    q_sat = W.saturation_specific_humidity(col.temperature, sigma[:, None] * 1e5)
    np.testing.assert_allclose(col.humidity, 0.8 * q_sat)
    assert np.all((col.cloud_fraction >= 0) & (col.cloud_fraction < 1))
    # 6.5 K/km: T = Ts - 6.5e-3 z with z hypsometric for that profile
    z = (ts[None, :] - col.temperature) / 6.5e-3
    assert np.all(z[-1] > 12e3) and np.all(z[0] < 600)


def test_planet_mix_and_trace():
    from planet_game_gb300 import workloads as W

    mix = W.planet_mix(2026)
    assert len(mix) == 64
    cells = sum(10 * 4**p.level + 2 for p in mix)
    assert cells == 2_252_928
    assert all(3e6 <= p.radius <= 9e6 for p in mix)
    trace = W.poisson_trace(2000, 500.0, seed=1)
    assert len(trace) == 2000
    gaps = np.diff([r.arrival_s for r in trace])
    assert abs(np.mean(gaps) - 1 / 500.0) < 0.1 / 500.0
    share = np.mean([r.level == 4 for r in trace])
    assert abs(share - 0.30) < 0.04


def test_lognormal_diffusivity_is_per_edge():
    from planet_game_gb300 import workloads as W

    k = W.lognormal_edge_diffusivity(100_000, seed=3)
    assert abs(np.median(k) / 1e6 - 1) < 0.02
    assert abs(np.std(np.log(k)) - 0.5) < 0.01


def test_reverse_entries_and_antisymmetric_fluxes(meshes):
    import planet_game_gb300 as pg
    from planet_game_gb300 import workloads as W

    g = pg.mesh_transport_graph(meshes(3))
    off, nb = g.offset.astype(np.int64), g.neighbour.astype(np.int64)
    rows = np.repeat(np.arange(len(off) - 1), np.diff(off))
    rev = W.reverse_entries(g.offset, g.neighbour)
    assert np.array_equal(nb[rev], rows) and np.array_equal(rows[rev], nb)
    for balanced in (True, False):
        f = W.antisymmetric_layer_fluxes(g.offset, g.neighbour, 3, 1e9, seed=5, column_balanced=balanced)
        F = f.reshape(3, len(nb))
        assert np.array_equal(F[:, rev], -F)
        column = np.abs(F.sum(axis=0)).max()
        assert (column <= 1e-6 * 1e9) if balanced else (column > 1.0)


def test_default_lanes_split_the_highest_level():
    from types import SimpleNamespace

    import planet_game_gb300 as pg

    ms = [SimpleNamespace(subdivision=l) for l in (4, 7, 5, 6, 7, 4)]
    assert pg.default_lanes(ms) == [[0, 2, 3, 5], [1, 4]]
    assert pg.default_lanes([SimpleNamespace(subdivision=l) for l in (5, 6, 5)]) == [[0, 1, 2]]
    assert pg.default_lanes([SimpleNamespace(subdivision=8)]) == [[0]]
    # the highest level's planets in lanes of at most four, split evenly
    mix = [SimpleNamespace(subdivision=l) for l in [4, 5, 6] + [7] * 8]
    assert pg.default_lanes(mix) == [[0, 1, 2], [3, 5, 7, 9], [4, 6, 8, 10]]
    mix = [SimpleNamespace(subdivision=l) for l in [4, 6] + [7] * 5]
    assert pg.default_lanes(mix) == [[0, 1], [2, 4, 6], [3, 5]]
    assert pg.default_lanes(mix, top_lane_planets=8) == [[0, 1], [2, 3, 4, 5, 6]]

"""The CPU oracle (oracle/planetsim_oracle.cpp) pinned against the reference's own
outputs (golden vectors written by tests/golden/make_golden.py from the reference
sources). Operators, diffusion source, Galerkin values, the SGS V-cycle, PCG and the
Newton driver are bit-identical; column radiation agrees to the last ulps of libm."""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O


@pytest.fixture(scope="module")
def L4(meshes):
    return O.OracleMesh(meshes(4).arrays())


@pytest.fixture(scope="module")
def L5(meshes):
    return O.OracleMesh(meshes(5).arrays())


def test_operators_f64_bit_identical(L4):
    g = golden("operators_L4.npz")
    assert np.array_equal(L4.laplacian(g["x64"]), g["laplacian64"])
    e, n = L4.gradient(g["x64"])
    assert np.array_equal(e, g["east64"]) and np.array_equal(n, g["north64"])
    assert np.array_equal(L4.divergence(g["flux64"]), g["divergence64"])
    assert np.array_equal(L4.diffusion_source(float(g["conductance"]), g["temperature"]), g["diffusion_source"])


def test_operators_f32_bit_identical(L4):
    g = golden("operators_L4.npz")
    assert np.array_equal(L4.laplacian(g["x32"]), g["laplacian32"])
    e, n = L4.gradient(g["x32"])
    assert np.array_equal(e, g["east32"]) and np.array_equal(n, g["north32"])
    assert np.array_equal(L4.divergence(g["flux32"]), g["divergence32"])


def test_galerkin_values_and_vcycle_bit_identical(L5):
    g = golden("heatstep_L5.npz")
    a = L5.a
    s = float(g["dt"]) / float(g["heat_capacity"])
    K = float(g["heat_capacity"]) * float(g["diffusivity"])
    h = O.OracleHierarchy(L5)
    h.set_matrix(a["area_m2"] / s + K * a["graph_weight_sum"], -K * a["graph_weight"])
    for lvl in range(h.levels()):
        d, o = h.values(lvl)
        assert np.array_equal(d, g[f"diag{lvl}"]), lvl
        assert np.array_equal(o, g[f"off{lvl}"]), lvl
    assert np.array_equal(h.vcycle_sgs(g["vcycle_rhs"]), g["vcycle_out"])


def test_pcg_bit_identical(L5):
    g = golden("heatstep_L5.npz")
    s = float(g["dt"]) / float(g["heat_capacity"])
    K = float(g["heat_capacity"]) * float(g["diffusivity"])
    h = O.OracleHierarchy(L5)
    x, it = h.pcg(K, np.full(L5.n, s), g["rhs"], float(g["pcg_tolerance"]), 2000)
    assert it == int(g["pcg_iterations"])
    assert np.array_equal(x, g["pcg_x"])


def test_newton_driver_bit_identical(L4):
    g = golden("newton_L4.npz")
    mean, src, stats = L4.solve_implicit_transport_linear(float(g["conductance"]), g["base"], g["slope"],
                                                          float(g["cg_tolerance"]), float(g["newton_tolerance"]))
    assert np.array_equal(mean, g["mean"])
    assert np.array_equal(src, g["source"])
    assert np.array_equal(stats, g["stats"])
    # the reference test's gates (test_heat_transport.cpp:103-106)
    assert stats[0] <= 3 and stats[2] <= 1e-6 and abs(stats[3]) <= 1e-13 * stats[4] and stats[5] <= 0.0


@pytest.mark.parametrize("layers", [4, 8])
def test_column_radiation_matches_reference(layers):
    g = golden("column.npz")
    k = np.concatenate([g["constants"], [101_325.0, float(g["gravity"]), 5.670374419e-8]])
    outs = O.column_radiation(k, g[f"temperature{layers}"], g[f"humidity{layers}"], g[f"cloud_water{layers}"],
                              g[f"surface_temperature{layers}"], g[f"surface_pressure{layers}"])
    for got, name in zip(outs, ("emissivity", "absorbed", "fraction", "reflectance", "scalars")):
        np.testing.assert_allclose(got, g[f"{name}{layers}"], rtol=1e-14, atol=1e-300, err_msg=name)


def test_saturation_matches_reference():
    from planet_game_gb300 import workloads as W

    g = golden("saturation.npz")
    T, P = np.meshgrid(g["temperature"], g["pressure"], indexing="ij")
    q_oracle = np.vectorize(O.saturation_specific_humidity)(T, P)
    assert np.array_equal(q_oracle, g["qsat"])
    np.testing.assert_allclose(W.saturation_specific_humidity(T, P), g["qsat"], rtol=1e-14)


def test_bicgstab_and_pcg_agree(L5):
    """The D1 bridge of the reference (test_advection_diffusion.cpp:166-191): the
    BiCGSTAB and PCG paths solve the same SPD system."""
    g = golden("heatstep_L5.npz")
    s = float(g["dt"]) / float(g["heat_capacity"])
    K = float(g["heat_capacity"]) * float(g["diffusivity"])
    h = O.OracleHierarchy(L5)
    xb, _ = h.bicgstab(K, np.full(L5.n, s), g["rhs"], 1e-12)
    np.testing.assert_allclose(xb, g["pcg_x"], rtol=1e-9)


def test_planted_oracle_mistake_is_caught(L4):
    """A mistake planted in the oracle's inputs (a flipped weight) must break parity."""
    g = golden("operators_L4.npz")
    a = dict(L4.a)
    w = a["edge_length_m"].copy()
    w[7] *= 1.0 + 1e-12
    a["edge_length_m"] = w
    bad = O.OracleMesh(a)
    assert not np.array_equal(bad.laplacian(g["x64"]), g["laplacian64"])


@pytest.mark.parametrize("case", [0, 1])
def test_quartic_response_bit_identical(case):
    """The oracle's quartic tile response equals the reference's (solve_column_surface)."""
    g = golden("newton_quartic_L4.npz")
    mean, slope = O.quartic_response(float(g[f"a{case}"]), g[f"b{case}"], g[f"probe_source{case}"])
    assert np.array_equal(mean, g[f"probe_mean{case}"])
    assert np.array_equal(slope, g[f"probe_slope{case}"])


@pytest.mark.parametrize("case,factor", [(0, 1), (0, 10), (1, 1), (1, 10)])
def test_nonlinear_newton_driver_bit_identical(L4, case, factor):
    """The oracle's restatement of solve_implicit_transport with the quartic response is
    the reference's, bit for bit, and meets the reference test's gates
    (test_heat_transport.cpp:140-144)."""
    g = golden("newton_quartic_L4.npz")
    key = f"{case}_{factor}"
    floor, mean, src, stats = L4.solve_implicit_transport_quartic(float(g[f"K{key}"]), float(g[f"a{case}"]),
                                                                  g[f"b{case}"])
    assert np.array_equal(floor, g[f"floor{key}"])
    assert np.array_equal(mean, g[f"mean{key}"])
    assert np.array_equal(src, g[f"source{key}"])
    assert np.array_equal(stats, g[f"stats{key}"])
    assert stats[2] <= 1e-6 and abs(stats[3]) <= 1e-13 * stats[4] and stats[5] <= 0.0
    assert np.all(mean[::7] <= 273.15)


# ---- the non-symmetric pieces against the reference (tests/golden/nonsym.npz) ---------

def _graph(planet):
    import planet_game_gb300 as pg

    g = pg.mesh_transport_graph(planet)
    return g.offset, g.neighbour, g.area_m2, g.weight


def _full_fluxes(offset, neighbour, half, layers):
    from planet_game_gb300 import workloads as W

    off, nb = offset.astype(np.int64), neighbour.astype(np.int64)
    rows = np.repeat(np.arange(len(off) - 1), np.diff(off))
    upper = np.nonzero(rows < nb)[0]
    rev = W.reverse_entries(offset, neighbour)
    out = np.zeros((layers, len(nb)))
    out[:, upper] = half
    out[:, rev[upper]] = -half
    return out.ravel()


def test_oracle_block_ilu_bit_identical_to_the_reference(meshes):
    g = golden("nonsym.npz")
    off, nb, _, _ = _graph(meshes(3))
    lu = O.OracleIlu(off, nb, g["ilu_diag"], g["ilu_off"], g["ilu_blocks"])
    assert not lu.zero_pivot
    assert np.array_equal(lu.solve(g["ilu_x"]), g["ilu_y"])


def test_oracle_advection_source_bit_identical_to_the_reference(meshes):
    g = golden("nonsym.npz")
    off, nb, area, weight = _graph(meshes(3))
    flux = _full_fluxes(off, nb, g["flux"], 3)
    for tag, latent in (("dry", None), ("latent", g["src_latent"])):
        eddy, adv = O.advection_source(off, nb, area, 3, 0.5 * 6.371e6 ** 2 * weight, flux, latent, g["src_mean"],
                                       g["src_energy"])
        assert np.array_equal(eddy, g[f"src_eddy_{tag}"]) and np.array_equal(adv, g[f"src_adv_{tag}"])


@pytest.mark.parametrize("tag", ["bal", "div", "eddy", "l3"])
def test_oracle_tracer_bit_identical_to_the_reference(meshes, tag):
    import planet_game_gb300 as pg

    g = golden("nonsym.npz")
    layers = int(g[f"tr_{tag}_layers"])
    planet = pg.agglomerated_transport_graph(3, 6.371e6) if int(g[f"tr_{tag}_agg"]) else meshes(3)
    off, nb, area, _ = _graph(planet)
    flux = _full_fluxes(off, nb, g[f"tr_{tag}_flux"], layers)
    cond = np.full(len(nb), float(g[f"tr_{tag}_eddy"]))
    mass = area * 100000.0 / (9.81 * layers)
    out, stats = O.solve_implicit_tracer(off, nb, layers, cond, flux, 1004.64, mass, g[f"tr_{tag}_in"], 2.63e6)
    assert np.array_equal(out, g[f"tr_{tag}_out"])
    assert np.array_equal(stats, g[f"tr_{tag}_stats"])


@pytest.mark.parametrize("tag", ["diff", "adv", "lat"])
def test_oracle_advection_diffusion_bit_identical_to_the_reference(meshes, tag):
    g = golden("nonsym.npz")
    m = meshes(3)
    off, nb, area, weight = _graph(m)
    flux = _full_fluxes(off, nb, g["flux"], 3) if tag != "diff" else np.zeros(3 * len(nb))
    om = O.OracleMesh(m.arrays())
    src, mean, energy, stats = O.solve_implicit_advection_diffusion(
        om, 3, 0.5 * 6.371e6 ** 2 * weight, flux, g["ad_lat_latent"] if tag == "lat" else None, 1004.64,
        float(g["ad_a"]), g["ad_b"], g["ad_eps"], g["ad_phi"], g["ad_floor"])
    assert np.array_equal(stats, g[f"ad_{tag}_stats"])
    assert np.array_equal(src, g[f"ad_{tag}_source"]) and np.array_equal(mean, g[f"ad_{tag}_mean"])
    assert np.array_equal(energy, g[f"ad_{tag}_energy"])


@pytest.mark.parametrize("factor", [1, 10])
def test_oracle_group_response_solve_bit_identical_to_the_reference(meshes, factor):
    """The production pattern on the L5 agglomeration (fine-cell quartic at the group's
    source, group means, the nonlinear solve) against the reference's own solve."""
    import planet_game_gb300 as pg

    g = golden("agglomeration.npz")
    p = pg.agglomerated_transport_graph(5, 6.371e6)
    om = O.OracleMesh(p.arrays())
    mean, src, stats = om.solve_implicit_transport_group_quartic(
        p.group_of_cell(), meshes(5).arrays()["area_m2"], float(g[f"qK{factor}"]), float(g["qa"]), g["qb"],
        g[f"qfloor{factor}"])
    assert np.array_equal(mean, g[f"qmean{factor}"]) and np.array_equal(src, g[f"qsource{factor}"])
    assert np.array_equal(stats, g[f"qstats{factor}"])

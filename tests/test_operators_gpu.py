"""GPU finite-volume operators (K1-K3) and diffusion source through the C-ABI,
against the reference's golden vectors and the CPU oracle."""
import numpy as np
import pytest

from conftest import golden, rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_operators_match_oracle_bit_for_bit(meshes):
    """Same mesh, same inputs: gradient, divergence and diffusion_source follow the
    reference's operation order exactly; the Laplacian uses the precomputed l/d weight."""
    import planet_game_gb300 as pg

    g = golden("operators_L4.npz")
    m = meshes(4)
    a = m.arrays()
    om = O.OracleMesh(a)
    e, n = pg.gradient(m, g["x64"])
    eo, no = om.gradient(g["x64"])
    assert np.array_equal(e, eo) and np.array_equal(n, no)
    assert np.array_equal(pg.divergence(m, g["flux64"]), om.divergence(g["flux64"]))
    K = float(g["conductance"])
    assert np.array_equal(pg.diffusion_source(m, K, g["temperature"]), om.diffusion_source(K, g["temperature"]))
    rows = np.repeat(np.arange(m.cell_count), a["edge_count"].astype(int))
    scale = np.bincount(rows, np.abs(g["x64"][a["neighbor"]] - g["x64"][rows]) * a["graph_weight"]) / a["area_m2"]
    assert np.all(np.abs(pg.laplacian(m, g["x64"]) - om.laplacian(g["x64"])) <= 2e-15 * scale)
    e32, n32 = pg.gradient(m, g["x32"])
    eo32, no32 = om.gradient(g["x32"])
    assert np.array_equal(e32, eo32) and np.array_equal(n32, no32)
    assert np.array_equal(pg.divergence(m, g["flux32"]), om.divergence(g["flux32"]))
    lap32, lapo32 = pg.laplacian(m, g["x32"]), om.laplacian(g["x32"])
    assert np.all(np.abs(lap32 - lapo32) <= np.spacing(np.abs(lapo32)))


def test_operators_match_reference_golden(meshes):
    """Against the reference's own outputs (computed on the x86 build host). The host
    mesh is bit-identical there; on another host's libm its geometry may differ in the
    last bits, so the comparison is to 1e-12 of each output's scale."""
    import planet_game_gb300 as pg

    g = golden("operators_L4.npz")
    m = meshes(4)

    def close(got, want):
        return np.max(np.abs(got - want)) <= 1e-12 * np.max(np.abs(want))

    e, n = pg.gradient(m, g["x64"])
    assert close(e, g["east64"]) and close(n, g["north64"])
    assert close(pg.divergence(m, g["flux64"]), g["divergence64"])
    assert close(pg.laplacian(m, g["x64"]), g["laplacian64"])
    assert close(pg.diffusion_source(m, float(g["conductance"]), g["temperature"]), g["diffusion_source"])
    e32, n32 = pg.gradient(m, g["x32"])
    assert np.max(np.abs(e32 - g["east32"])) <= 2 * np.spacing(np.max(np.abs(g["east32"])))


def test_host_mesh_on_this_host_matches_reference(meshes):
    """Integer topology identical to the reference's; floating-point geometry within a few
    ulps (bit-identical on the reference's own build host, where the CPU suite checks it)."""
    import hashlib

    ref = golden("golden.json")["mesh_sha256"]["6"]
    a = meshes(6).arrays()
    for key in ("source_vertex", "edge_offset", "edge_count", "neighbor", "edge", "edge_first", "edge_second",
                "corner"):
        assert hashlib.sha256(np.ascontiguousarray(a[key]).tobytes()).hexdigest() == ref[key], key
    np.testing.assert_allclose(a["area_m2"].sum(), 4 * np.pi * 6.371e6**2, rtol=1e-12)


@pytest.mark.parametrize("level", [5, 6])
def test_harmonic_sweep_against_oracle_and_analytic(meshes, level):
    """The L6 operator sweep: 8 seeded fields, sums of real spherical harmonics l <= 16."""
    import planet_game_gb300 as pg
    from planet_game_gb300 import workloads as W

    m = meshes(level)
    a = m.arrays()
    om = O.OracleMesh(a)
    analytic_gate = {5: (2.5e-2, 6.5e-2, 1.3e-2), 6: (6.5e-3, 2.2e-2, 3.2e-3)}[level]
    for seed in range(8):
        F = W.harmonic_field(a, m.radius_m, 16, seed)
        lap, (ge, gn), div = pg.laplacian(m, F.value), pg.gradient(m, F.value), pg.divergence(m, F.edge_flux)
        np.testing.assert_allclose(lap, om.laplacian(F.value), rtol=0, atol=1e-13 * np.abs(lap).max())
        assert np.array_equal(ge, om.gradient(F.value)[0]) and np.array_equal(gn, om.gradient(F.value)[1])
        assert np.array_equal(div, om.divergence(F.edge_flux))
        w = a["area_m2"]
        assert rel_l2(lap, F.laplacian, w) < analytic_gate[0]
        assert rel_l2(ge, F.east, w) < analytic_gate[1] and rel_l2(gn, F.north, w) < analytic_gate[1]
        assert rel_l2(div, F.laplacian, w) < analytic_gate[2]


def test_conservation_and_constant_fields(meshes):
    import planet_game_gb300 as pg

    m = meshes(6)
    a = m.arrays()
    rng = np.random.default_rng(5)
    phi = rng.standard_normal(m.cell_count)
    lap = pg.laplacian(m, phi)
    gross = np.sum(a["area_m2"] * np.abs(lap))
    assert abs(np.sum(a["area_m2"] * lap)) <= 1e-13 * gross
    assert np.sum(a["area_m2"] * phi * lap) < 0.0
    flux = rng.standard_normal(m.edge_count)
    div = pg.divergence(m, flux)
    assert abs(np.sum(a["area_m2"] * div)) <= 1e-13 * np.sum(a["area_m2"] * np.abs(div))
    assert np.all(pg.laplacian(m, np.full(m.cell_count, 3.5)) == 0.0)
    e, n = pg.gradient(m, np.full(m.cell_count, 3.5))
    assert np.all(e == 0.0) and np.all(n == 0.0)


def test_device_pointer_path_matches_host_path(meshes):
    torch = pytest.importorskip("torch")
    import planet_game_gb300 as pg

    m = meshes(5)
    rng = np.random.default_rng(9)
    phi = rng.standard_normal(m.cell_count)
    host = pg.laplacian(m, phi)
    dev = pg.laplacian(m, torch.from_numpy(phi).cuda())
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy(), host)
    f32 = torch.from_numpy(phi.astype(np.float32)).cuda()
    e, n = pg.gradient(m, f32)
    e_h, n_h = pg.gradient(m, phi.astype(np.float32))
    assert np.array_equal(e.cpu().numpy(), e_h) and np.array_equal(n.cpu().numpy(), n_h)


@pytest.mark.parametrize("substep", [0, 5])
def test_insolation_kernel_matches_the_reference(meshes, substep):
    """The sub-step-mean insolation kernel: within one FP32 ulp of the reference at L4
    (sub-step 0, golden) and of the host restatement (another sub-step); zero only where
    the host's is."""
    m = meshes(4)
    gpu = m.substep_mean_insolation_gpu(substep)
    host = m.substep_mean_insolation(substep)
    ulp = np.spacing(np.abs(host).astype(np.float32))
    assert np.all(np.abs(gpu - host) <= ulp)
    assert np.array_equal(gpu == 0.0, host == 0.0)
    if substep == 0:
        ref = golden("insolation_L4.npz")["insolation"]
        assert np.all(np.abs(gpu - ref) <= np.spacing(np.abs(ref).astype(np.float32)))


def test_insolation_kernel_on_device_memory(meshes):
    import torch

    m = meshes(6)
    out = torch.empty(m.cell_count, dtype=torch.float32, device="cuda")
    m.substep_mean_insolation_gpu(3, out)
    host = m.substep_mean_insolation(3)
    assert np.all(np.abs(out.cpu().numpy() - host) <= np.spacing(np.abs(host).astype(np.float32)))

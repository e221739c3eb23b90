"""The agglomerated transport graph against the reference's (golden vectors from
agglomerated_transport_graph, heat_transport.cpp:456-539): the group of every fine cell,
the coarse graph's CSR and weights, and the groups' summed areas, bit for bit at L0, L1,
L3 and L5 and through SHA-256 digests of the same arrays at L6-L8; plus the reference
test's own checks (test_heat_transport.cpp:173-211):
every cell covered once, areas summing to the sphere's to 1e-12, symmetric positive
weights, about four cells per group. Host-built, no GPU."""
import numpy as np
import pytest

from conftest import golden

LEVELS = (0, 1, 3, 5)


@pytest.fixture(scope="module")
def planets():
    import planet_game_gb300 as pg

    return {level: pg.agglomerated_transport_graph(level, 6.371e6) for level in LEVELS}


@pytest.mark.parametrize("level", LEVELS)
def test_groups_and_graph_bit_identical(planets, level):
    import planet_game_gb300 as pg

    g = golden("agglomeration.npz")
    p = planets[level]
    graph = pg.mesh_transport_graph(p)
    assert p.cell_count == len(g[f"area{level}"])
    assert np.array_equal(p.group_of_cell(), g[f"group{level}"])
    assert np.array_equal(graph.area_m2, g[f"area{level}"])
    assert np.array_equal(graph.offset.astype(np.uint32), g[f"offset{level}"])
    assert np.array_equal(graph.neighbour.astype(np.uint32), g[f"neighbour{level}"])
    assert np.array_equal(graph.weight, g[f"weight{level}"])
    assert np.array_equal(graph.weight_sum, g[f"weight_sum{level}"])


def test_reference_checks_at_l5(planets, meshes):
    import planet_game_gb300 as pg

    p = planets[5]
    fine = meshes(5)
    graph = pg.mesh_transport_graph(p)
    groups = p.group_of_cell()
    assert p.fine_cell_count == fine.cell_count == len(groups)
    assert groups.max() < p.cell_count and np.all(np.bincount(groups, minlength=p.cell_count) > 0)
    mesh_area = fine.arrays()["area_m2"].sum()
    assert abs(graph.area_m2.sum() - mesh_area) <= 1e-12 * mesh_area
    # the groups' areas are the fine cells' summed in fine-cell order
    sums = np.zeros(p.cell_count)
    for c, a in zip(groups, fine.arrays()["area_m2"]):
        sums[c] += a
    assert np.array_equal(sums, graph.area_m2)
    for node in range(p.cell_count):
        for k in range(graph.offset[node], graph.offset[node + 1]):
            other = int(graph.neighbour[k])
            back = graph.neighbour[graph.offset[other]:graph.offset[other + 1]] == node
            assert other != node and graph.weight[k] > 0.0
            assert np.any(back & (graph.weight[graph.offset[other]:graph.offset[other + 1]] == graph.weight[k]))
    assert 3.9 < fine.cell_count / p.cell_count < 4.1


def test_level0_is_the_mesh_itself(planets, meshes):
    p = planets[0]
    assert p.subdivision == 0 and p.cell_count == meshes(0).cell_count == p.fine_cell_count
    assert np.array_equal(p.group_of_cell(), np.arange(p.cell_count, dtype=np.uint32))
    assert np.array_equal(p.arrays()["graph_area_m2"], meshes(0).arrays()["area_m2"])


def test_plain_planet_has_no_groups(meshes):
    with pytest.raises(ValueError):
        meshes(2).group_of_cell()


def test_nonsymmetric_inputs_are_checked_before_the_library(planets):
    """The C ABI takes bare pointers: the Python layer refuses arrays of the wrong size."""
    import numpy as np

    import planet_game_gb300 as pg

    p = planets[3]
    E, n = p.directed_edge_count, p.cell_count
    good = pg.AdvectionDiffusion(2, np.ones(E), np.zeros(2 * E))
    good.check(p)
    for bad in (pg.AdvectionDiffusion(2, np.ones(E - 1), np.zeros(2 * E)),
                pg.AdvectionDiffusion(2, np.ones(E), np.zeros(E)),
                pg.AdvectionDiffusion(2, np.ones(E), np.zeros(2 * E), eddy_latent_W_m2=np.zeros(n + 1))):
        with pytest.raises(ValueError):
            bad.check(p)
    with pytest.raises(ValueError):
        pg.solve_implicit_tracer(p, good, np.ones(n), np.ones(2 * n - 1), 1.0)
    with pytest.raises(ValueError):
        pg.advection_diffusion_source(p, good, np.ones(n), np.ones(n))


@pytest.mark.parametrize("level", [6, 7, 8])
def test_large_agglomerations_match_the_reference_digests(level):
    """L6-L8 (the sizes the workloads use) against SHA-256 digests of the reference's
    groups, graph and areas (tests/golden/agglomeration_sha256.json)."""
    import hashlib
    import json
    from pathlib import Path

    import planet_game_gb300 as pg

    want = json.loads((Path(__file__).parent / "golden" / "agglomeration_sha256.json").read_text())[str(level)]
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()   # noqa: E731
    p = pg.agglomerated_transport_graph(level, 6.371e6)
    g = pg.mesh_transport_graph(p)
    assert p.cell_count == want["nodes"]
    assert sha(p.group_of_cell()) == want["group"]
    assert sha(g.area_m2) == want["area"]
    assert sha(g.offset.astype(np.uint32)) == want["offset"]
    assert sha(g.neighbour.astype(np.uint32)) == want["neighbour"]
    assert sha(g.weight) == want["weight"] and sha(g.weight_sum) == want["weight_sum"]

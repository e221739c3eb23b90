"""Host mesh and hierarchy builders against the reference (golden vectors).

The reference's make_icosphere and build_hierarchy outputs are pinned as full arrays
(L0-L2) and SHA-256 digests (L0-L8); the GB300 library's host builders must reproduce
them bit for bit (cell order, adjacency, FP64 geometry, FP32 normals, aggregates,
coarse patterns, Galerkin targets)."""
import hashlib

import numpy as np
import pytest

from conftest import golden


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("level", [0, 1, 2])
def test_mesh_arrays_bit_identical(meshes, level):
    ref = golden(f"mesh_L{level}.npz")
    mine = meshes(level).arrays()
    for key in ref.files:
        assert mine[key].dtype == ref[key].dtype, key
        assert mine[key].tobytes() == ref[key].tobytes(), key


@pytest.mark.parametrize("level", [3, 4, 5, 6, 7, 8])
def test_mesh_digests_bit_identical(meshes, level):
    ref = golden("golden.json")["mesh_sha256"][str(level)]
    mine = meshes(level).arrays()
    bad = [k for k, h in ref.items() if sha(mine[k]) != h]
    assert not bad, f"arrays differing from the reference at L{level}: {bad}"


@pytest.mark.parametrize("level", [3, 4, 5, 6, 7, 8])
def test_hierarchy_structure_bit_identical(meshes, level):
    ref = golden("golden.json")["hierarchy_sha256"][str(level)]
    m = meshes(level)
    assert len(m.level_rows) == len(ref)
    for i, lv in enumerate(ref):
        mine = m.hierarchy_level(i)
        assert m.level_rows[i] == lv["rows"]
        for key in ("offset", "column", "aggregate", "target"):
            assert sha(mine[key]) == lv[key], (level, i, key)


def test_mesh_counts_and_pentagons(meshes):
    for level in range(0, 7):
        m = meshes(level)
        a = m.arrays()
        assert m.cell_count == 10 * 4**level + 2
        assert m.edge_count == 3 * m.cell_count - 6
        assert int((a["edge_count"] == 5).sum()) == 12
        np.testing.assert_allclose(a["area_m2"].sum(), 4 * np.pi * 6.371e6**2, rtol=1e-12)


def test_insolation_matches_reference(meshes):
    ref = golden("insolation_L4.npz")
    mine = meshes(4).substep_mean_insolation(0)
    ulp = np.spacing(np.abs(ref["insolation"]).astype(np.float32))
    assert np.all(np.abs(mine - ref["insolation"]) <= ulp)


def test_radius_scales_geometry_only(meshes):
    a = meshes(4).arrays()
    b = meshes(4, 4.5e6).arrays()
    for key in ("neighbor", "edge", "edge_first", "edge_second", "source_vertex", "edge_offset"):
        assert np.array_equal(a[key], b[key])
    assert np.allclose(b["area_m2"] / a["area_m2"], (4.5e6 / 6.371e6) ** 2, rtol=1e-12)


def test_invalid_mesh_arguments():
    import planet_game_gb300 as pg

    with pytest.raises(ValueError):
        pg.make_icosphere(3, -1.0)
    with pytest.raises(ValueError):
        pg.make_icosphere(3, float("nan"))
    with pytest.raises(ValueError):
        pg.make_icosphere(40, 6.371e6)


@pytest.mark.parametrize("level", [4, 5, 6])
def test_integer_structure_depends_on_the_level_only(level):
    """The hierarchy is built from unit conductances: its integer structure (columns,
    aggregates, targets) and the graph's CSR are the same for every radius of a level,
    while the geometric weights differ in the last bits."""
    import planet_game_gb300 as pg

    ms = [pg.make_icosphere(level, r) for r in (3.1e6, 6.371e6, 8.9e6)]
    for m in ms[1:]:
        assert m.level_rows == ms[0].level_rows
        for i in range(len(m.level_rows)):
            a, b = ms[0].hierarchy_level(i), m.hierarchy_level(i)
            for key in ("offset", "column", "aggregate", "target"):
                assert np.array_equal(a[key], b[key]), (level, i, key)
        ga, gb = pg.mesh_transport_graph(ms[0]), pg.mesh_transport_graph(m)
        assert np.array_equal(ga.offset, gb.offset) and np.array_equal(ga.neighbour, gb.neighbour)
        assert np.allclose(ga.weight, gb.weight, rtol=1e-15, atol=0)

"""The oracle's own restatement of the reference's mesh builder (oracle/mesh_oracle.cpp),
which the CPU legs of the benchmark use to build their planets without the product
library, against the reference's meshes: full arrays at L0-L2, SHA-256 digests of every
array at L3-L7 (the digests the product's builder is pinned to)."""
import hashlib

import numpy as np
import pytest

from conftest import golden


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("level", [0, 1, 2])
def test_oracle_mesh_arrays_are_the_reference_ones(level):
    from oracle import oracle as O

    ref = golden(f"mesh_L{level}.npz")
    mine = O.icosphere(level, float(golden("golden.json")["radius_m"]))
    for key in ref.files:
        assert mine[key].dtype == ref[key].dtype, key
        assert mine[key].tobytes() == ref[key].tobytes(), key


@pytest.mark.parametrize("level", [3, 4, 5, 6, 7])
def test_oracle_mesh_digests_are_the_reference_ones(level):
    from oracle import oracle as O

    ref = golden("golden.json")["mesh_sha256"][str(level)]
    mine = O.icosphere(level, float(golden("golden.json")["radius_m"]))
    bad = [k for k, h in ref.items() if sha(mine[k]) != h]
    assert not bad, f"arrays differing from the reference at L{level}: {bad}"


def test_oracle_mesh_is_the_product_mesh_at_another_radius(meshes):
    from oracle import oracle as O

    a = O.icosphere(4, 4.2e6)
    b = meshes(4, 4.2e6).arrays()
    for key in a:
        assert np.array_equal(a[key], b[key]), key


def test_oracle_insolation_is_the_reference_one():
    from oracle import oracle as O

    ref = golden("insolation_L4.npz")
    mine = O.substep_mean_insolation(O.icosphere(4, 6.371e6)["center"], ref["nodes"])
    assert mine.dtype == ref["insolation"].dtype
    assert np.array_equal(mine, ref["insolation"])

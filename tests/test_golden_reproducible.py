"""The committed golden fixtures come from the reference itself: where the reference's
sources are present, its code (compiled where it lies by oracle/Makefile.ref, driven by
oracle/ref_driver.cpp through tests/golden/make_golden.py's loader) is run again and must
give the committed values bit for bit: the L0-L2 meshes' arrays, the L3-L8 meshes' and
hierarchies' digests, the agglomerated graphs at L0/L1/L3/L5 and their L6-L8 digests, the
non-symmetric solves' fixture (block ILU(0), advection source, tracer, coupled solve), the
quartic-response transport solves, and every fixture of the main set (operators, the
linear Newton solve, insolation, the L5 heat step with its Galerkin values, V-cycle and PCG,
column radiation, saturation, the digests).
Skipped where the reference is absent (the GPU host)."""
import importlib.util
import json
import re
import shutil
from pathlib import Path

import numpy as np
import pytest

from conftest import golden

ROOT = Path(__file__).resolve().parents[1]


def _reference() -> Path | None:
    from oracle.build import reference_root

    return reference_root()


@pytest.fixture(scope="module")
def maker():
    ref = _reference()
    if ref is None or shutil.which("make") is None or shutil.which("g++") is None:
        pytest.skip("reference sources or a compiler not present")
    spec = importlib.util.spec_from_file_location("make_golden", ROOT / "tests" / "golden" / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg, mg.load(ref)


@pytest.mark.parametrize("level", [0, 1, 2])
def test_mesh_fixtures_are_the_reference_meshes(maker, level):
    mg, R = maker
    m = mg.P(R.refd_mesh_new(level, mg.RADIUS))
    try:
        fresh = mg.mesh_arrays(R, m)
    finally:
        R.refd_mesh_free(m)
    committed = golden(f"mesh_L{level}.npz")
    assert sorted(fresh) == sorted(committed.files)
    for key, value in fresh.items():
        assert np.array_equal(value, committed[key]), key


@pytest.mark.parametrize("level", [3, 5, 7])
def test_mesh_and_hierarchy_digests_are_the_reference_ones(maker, level):
    mg, R = maker
    meta = golden("golden.json")
    m = mg.P(R.refd_mesh_new(level, mg.RADIUS))
    try:
        digests = {k: mg.sha(v) for k, v in mg.mesh_arrays(R, m).items()}
        levels = mg.hierarchy(R, m)
    finally:
        R.refd_mesh_free(m)
    assert digests == meta["mesh_sha256"][str(level)]
    want = meta["hierarchy_sha256"][str(level)]
    assert len(levels) == len(want)
    for lv, w in zip(levels, want):
        assert {k: mg.sha(v) for k, v in lv.items()} | {"rows": len(lv["offset"]) - 1} == w


def _agglomeration(mg, R, level):
    m = mg.P(R.refd_mesh_new(level, mg.RADIUS))
    try:
        counts = np.zeros(3, np.uint64)
        R.refd_agglomeration_counts(m, mg.p(counts))
        n, d, f = (int(x) for x in counts)
        area, wsum, w = np.empty(n), np.empty(n), np.empty(d)
        off, nb, groups = np.empty(n + 1, np.uint64), np.empty(d, np.uint64), np.empty(f, np.uint64)
        R.refd_agglomeration(m, mg.p(area), mg.p(off), mg.p(nb), mg.p(w), mg.p(wsum), mg.p(groups))
    finally:
        R.refd_mesh_free(m)
    return {"area": area, "offset": off.astype(np.uint32), "neighbour": nb.astype(np.uint32), "weight": w,
            "weight_sum": wsum, "group": groups.astype(np.uint32)}


@pytest.mark.parametrize("level", [1, 3, 5])
def test_agglomeration_fixture_is_the_reference_one(maker, level):
    mg, R = maker
    fresh = _agglomeration(mg, R, level)
    committed = golden("agglomeration.npz")
    for key, value in fresh.items():
        assert np.array_equal(value, committed[f"{key}{level}"]), key


def test_agglomeration_digest_at_l6_is_the_reference_one(maker):
    mg, R = maker
    fresh = _agglomeration(mg, R, 6)
    want = json.loads((ROOT / "tests" / "golden" / "agglomeration_sha256.json").read_text())["6"]
    assert len(fresh["area"]) == want["nodes"]
    for key, value in fresh.items():
        assert mg.sha(value) == want[key], key


@pytest.mark.parametrize("name,fixture", [("nonsym_cases", "nonsym.npz"), ("quartic_cases", "newton_quartic_L4.npz")])
def test_solve_fixtures_are_the_reference_ones(maker, name, fixture):
    mg, R = maker
    fresh = getattr(mg, name)(R, write=False)
    committed = golden(fixture)
    assert sorted(fresh) == sorted(committed.files)
    for key, value in fresh.items():
        assert np.array_equal(np.asarray(value), committed[key]), key


def test_main_fixtures_are_the_reference_ones(maker):
    mg, R = maker
    ref = _reference()
    made = mg.main(ref, write=False)
    assert made.pop("golden.json") == golden("golden.json")
    for name, arrays in made.items():
        committed = golden(name)
        assert sorted(arrays) == sorted(committed.files), name
        for key, value in arrays.items():
            assert np.array_equal(np.asarray(value), committed[key]), (name, key)

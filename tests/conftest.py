"""Shared fixtures. `-m gpu` tests need a GPU and the in-tree CUDA library; the CPU suite
(`-m "not gpu"`) checks the oracle against the reference's golden vectors, the host
builders, the C-ABI surface and the multi-process host logic."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and runs the sm_103a kernels")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Compile the library and the oracle in-tree (incremental)."""
    from oracle import build as oracle_build
    from planet_game_gb300 import build

    build.build_library()
    oracle_build.build_oracle()
    yield


def golden(name: str):
    if name.endswith(".json"):
        return json.loads((GOLDEN / name).read_text())
    return np.load(GOLDEN / name)


@pytest.fixture(scope="session")
def meshes():
    """Host-built meshes by level (no GPU needed to build them)."""
    import planet_game_gb300 as pg

    cache = {}

    def get(level: int, radius: float = 6.371e6):
        key = (level, radius)
        if key not in cache:
            cache[key] = pg.make_icosphere(level, radius)
        return cache[key]

    return get


def rel_l2(x, y, w=None):
    w = np.ones_like(y) if w is None else w
    return float(np.sqrt(np.sum(w * (x - y) ** 2) / np.sum(w * y**2)))

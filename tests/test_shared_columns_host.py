"""The fine level's columns shared per distinct graph of a batch, checked on the host
(tests/cpp/shared_columns_check.cpp): read through each tile's shift they give every row
of every planet the same columns as the per-planet layout, and each distinct graph is
held once. On the GPU, batches holding planets of one mesh level (which share a graph)
give each planet's solve bit for bit (tests/test_solver_gpu.py)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_shared_columns_equal_the_per_planet_columns(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "shared_columns_check"
    csrc = ROOT / "planet_game_gb300" / "csrc"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(csrc), str(ROOT / "tests" / "cpp" / "shared_columns_check.cpp"),
                    str(csrc / "host" / "shared_columns.cpp"), "-o", str(exe)], check=True, capture_output=True,
                   text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and out.stdout.strip() == "OK", out.stdout + out.stderr

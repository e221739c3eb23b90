"""The block ILU(0) structure's host builder (level schedules, the IKJ update list, the
shared-memory solve's records) checked on random patterns by a small C++ program compiled
here against the library's host source (tests/cpp/ilu_pattern_check.cpp). No GPU."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_ilu_pattern_schedules_and_update_list(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "ilu_pattern_check"
    csrc = ROOT / "planet_game_gb300" / "csrc"
    subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-I", str(csrc),
                    str(ROOT / "tests" / "cpp" / "ilu_pattern_check.cpp"), str(csrc / "host" / "ilu_pattern.cpp"),
                    "-o", str(exe)], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == "OK", out.stdout + out.stderr

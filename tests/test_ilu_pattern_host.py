"""Host builders checked by small C++ programs compiled here against the library's host
sources (tests/cpp/): the block ILU(0) structure (level schedules, the IKJ update list, the
shared-memory solve's records) on random patterns, and the spread coarse tail's block
layout. No GPU."""
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


def test_spread_tail_block_layout(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "tail_blocks_check"
    csrc = ROOT / "planet_game_gb300" / "csrc"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(csrc), str(ROOT / "tests" / "cpp" / "tail_blocks_check.cpp"),
                    str(csrc / "host" / "tail_blocks.cpp"), "-o", str(exe)], check=True, capture_output=True,
                   text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and out.stdout.strip() == "OK", out.stdout + out.stderr

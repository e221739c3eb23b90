"""The C++ shim of the integration guide (its first cpp block) compiles against the reference's own headers and this
library's C header: the drop-in a maintainer adds is real code, not a sketch. Needs the
reference sources (found through oracle/Makefile.ref, or PLANETSIM_REFERENCE); skipped
where they are absent."""
import os
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def reference_root() -> Path | None:
    env = os.environ.get("PLANETSIM_REFERENCE")
    if env:
        return Path(env)
    m = re.search(r"^REF \?= (\S+)$", (ROOT / "oracle" / "Makefile.ref").read_text(), re.M)
    return Path(m.group(1)) if m else None


def test_shim_compiles_against_the_reference_headers(tmp_path):
    ref = reference_root()
    if ref is None or not (ref / "sim" / "planet" / "surface" / "heat_transport.hpp").exists():
        pytest.skip("reference sources not present")
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    text = (ROOT / "INTEGRATION.md").read_text()
    blocks = re.findall(r"```cpp\n(.*?)```", text, re.S)
    assert blocks, "the integration guide has no C++ shim"
    src = tmp_path / "planetsim_gb300_adapter.cpp"
    src.write_text(blocks[0] + "\nint main() { return 0; }\n")
    proc = subprocess.run(["g++", "-std=c++20", "-fsyntax-only", "-I", str(ref), "-I", str(ROOT / "include"),
                           str(src)], capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr[-4000:]

"""Build recipes of the checker (test infrastructure, never the product path).

``build_oracle()`` compiles the CPU restatement (``planetsim_oracle.cpp``,
``nonsym_oracle.cpp``, ``mesh_oracle.cpp``) into ``oracle/lib/libplanetsim_oracle.so``.
``build_reference_driver(reference)`` compiles the reference's own sources, unmodified and
where they lie, with ``oracle/ref_driver.cpp`` into ``oracle/_ref/`` (``Makefile.ref``),
and records the checkout it used in ``oracle/_ref/REFERENCE`` so that the tests and
fixture scripts that re-run the reference find it again.

``reference_root()`` locates the checkout: an explicit path, else the
``PLANETSIM_REFERENCE`` environment variable, else the recorded build; ``None`` where
the reference's sources are absent (the GPU host).
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
ROOT = ORACLE_DIR.parent
ORACLE_LIB = ORACLE_DIR / "lib" / "libplanetsim_oracle.so"
REF_OUT = ORACLE_DIR / "_ref"
REFERENCE_RECORD = REF_OUT / "REFERENCE"


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)


def _has_sources(path: Path) -> bool:
    return (path / "sim" / "planet" / "surface" / "heat_transport.cpp").is_file()


def reference_root(explicit: str | Path | None = None) -> Path | None:
    """The reference checkout to compile or re-run, or None when its sources are absent."""
    candidates = [explicit, os.environ.get("PLANETSIM_REFERENCE")]
    if REFERENCE_RECORD.exists():
        candidates.append(REFERENCE_RECORD.read_text().strip())
    for c in candidates:
        if c and _has_sources(Path(c)):
            return Path(c)
    return None


def build_oracle(force: bool = False) -> Path:
    """Compile the CPU oracle into oracle/lib/."""
    srcs = [ORACLE_DIR / "planetsim_oracle.cpp", ORACLE_DIR / "nonsym_oracle.cpp", ORACLE_DIR / "mesh_oracle.cpp"]
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    if force or _stale(ORACLE_LIB, srcs + [ORACLE_DIR / "oracle_abi.hpp"]):
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread", *map(str, srcs),
              "-o", str(tmp)])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_reference_driver(reference: str | Path) -> Path:
    """Compile the reference's own sources at `reference` into oracle/_ref/."""
    ref = Path(reference)
    if not _has_sources(ref):
        raise FileNotFoundError(f"no reference sources under {ref}")
    _run(["make", "-s", "-f", str(ORACLE_DIR / "Makefile.ref"), f"REF={ref}", f"OUT={REF_OUT}",
          f"-j{os.cpu_count() or 4}", "-C", str(ROOT)])
    REFERENCE_RECORD.write_text(str(ref) + "\n")
    return REF_OUT / "libref_driver.so"

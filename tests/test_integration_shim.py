"""The C++ shim of the integration guide (its first cpp block) compiles against the reference's own headers and this
library's C header: the drop-in a maintainer adds is real code, not a sketch. Needs the
reference sources (PLANETSIM_REFERENCE, or the checkout oracle/build.py compiled); skipped
where they are absent."""
import os
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def reference_root() -> Path | None:
    from oracle.build import reference_root as located

    return located()


# Takes the address of every adapter function, so that the compiler emits them and the
# link below has to resolve every C entry point they call.
USES = """
namespace {
using namespace planetsim;
using G = const TransportGraph&;
void* const adapter_functions[] = {
    reinterpret_cast<void*>(static_cast<TransportGraph (*)(const PlanetMesh&)>(&gb300::mesh_transport_graph)),
    reinterpret_cast<void*>(&gb300::agglomerated_transport_graph),
    reinterpret_cast<void*>(&gb300::laplacian<double>),
    reinterpret_cast<void*>(&gb300::laplacian<float>),
    reinterpret_cast<void*>(&gb300::solve_implicit_transport),
    reinterpret_cast<void*>(&gb300::advection_diffusion_source),
    reinterpret_cast<void*>(&gb300::solve_implicit_tracer),
    reinterpret_cast<void*>(&gb300::solve_implicit_advection_diffusion),
};
}  // namespace
extern "C" void* const* planetsim_gb300_adapter_functions() { return adapter_functions; }
"""


def _shim_source(tmp_path: Path) -> Path:
    text = (ROOT / "INTEGRATION.md").read_text()
    blocks = re.findall(r"```cpp\n(.*?)```", text, re.S)
    assert blocks, "the integration guide has no C++ shim"
    src = tmp_path / "planetsim_gb300_adapter.cpp"
    src.write_text(blocks[0] + USES)
    return src


def test_shim_compiles_against_the_reference_headers(tmp_path):
    ref = reference_root()
    if ref is None or not (ref / "sim" / "planet" / "surface" / "heat_transport.hpp").exists():
        pytest.skip("reference sources not present")
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    src = _shim_source(tmp_path)
    proc = subprocess.run(["g++", "-std=c++20", "-fsyntax-only", "-I", str(ref), "-I", str(ROOT / "include"),
                           str(src)], capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr[-4000:]


def test_shim_links_against_this_library(tmp_path):
    """The adapter compiled to an object and linked, with no undefined symbol left, against
    libplanetsim_gb300.so (its C entry points) and the reference's own build (the graph
    constructors it hands back to): every psgb_* call the shim makes names an entry point
    the library exports."""
    ref = reference_root()
    if ref is None or shutil.which("g++") is None:
        pytest.skip("reference sources or a compiler not present")
    ref_lib = ROOT / "oracle" / "_ref" / "libref_driver.so"
    if not ref_lib.exists():
        from oracle import build as ob

        ob.build_reference_driver(ref)
    from planet_game_gb300 import build

    lib = build.build_library()
    src = _shim_source(tmp_path)
    obj = tmp_path / "adapter.o"
    proc = subprocess.run(["g++", "-std=c++20", "-O1", "-fPIC", "-I", str(ref), "-I", str(ROOT / "include"), "-c",
                           str(src), "-o", str(obj)], capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr[-4000:]
    undefined = subprocess.run(["nm", "--undefined-only", str(obj)], capture_output=True, text=True).stdout
    called = sorted({line.split()[-1] for line in undefined.splitlines() if line.split()[-1].startswith("psgb_")})
    assert len(called) >= 10, called
    out = tmp_path / "libadapter.so"
    proc = subprocess.run(["g++", "-shared", "-o", str(out), str(obj), "-Wl,--no-undefined", "-L", str(lib.parent),
                           "-lplanetsim_gb300", str(ref_lib), f"-Wl,-rpath,{lib.parent}"],
                          capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr[-4000:]
    exported = subprocess.run(["nm", "-D", "--defined-only", str(lib)], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in exported.splitlines()}
    assert set(called) <= exported

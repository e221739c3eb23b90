"""The native serving loop (psgb_server_*) on a host without a GPU:

- its host logic (serve_core.cpp), compiled here with a fake device backend
  (tests/cpp/serve_check.cpp): per-planet request order, continuous batching (one round
  steps every planet of a lane with queued work; lanes step side by side), the memory
  budget (least recently used idle lane evicted with its states copied back; a lane larger
  than the budget refused; lanes taking turns when one waits for memory), concurrent
  producers, failures reported per request, timeouts and shutdown;
- its device side (serve.cpp) with the CUDA runtime and the batch entry points replaced by
  host stand-ins (tests/cpp/serve_gpu_lane_check.cpp): the lanes' layout of states and
  sources, stored per-edge conductances, tuning once per level and reused after eviction,
  states surviving eviction, per-request solve statuses, failed rounds keeping the state,
  and everything freed with the server;
- the C entry points and their Python wrapper (serve.NativeServer): argument checks, and a
  lane that cannot reach a GPU failing its requests with the CUDA status instead of
  hanging."""
import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_serving_loop_host_logic(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "serve_check"
    csrc = ROOT / "planet_game_gb300" / "csrc"
    subprocess.run(["g++", "-std=c++17", "-O1", "-pthread", "-I", str(csrc), str(ROOT / "tests" / "cpp" / "serve_check.cpp"),
                    str(csrc / "serve_core.cpp"), "-o", str(exe)], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == "OK", out.stdout + out.stderr


def test_serving_loop_device_side_with_host_stand_ins(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    cuda_include = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"
    if not (cuda_include / "cuda_runtime.h").exists():
        pytest.skip("no CUDA headers")
    exe = tmp_path / "serve_gpu_lane_check"
    csrc = ROOT / "planet_game_gb300" / "csrc"
    subprocess.run(["g++", "-std=c++17", "-O1", "-pthread", "-I", str(csrc), "-I", str(cuda_include),
                    str(ROOT / "tests" / "cpp" / "serve_gpu_lane_check.cpp"), str(csrc / "serve.cpp"),
                    str(csrc / "serve_core.cpp"), "-o", str(exe)], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == "OK", out.stdout + out.stderr


def _server(lib, capi, budget=1e9):
    cfg = capi.ServerConfig()
    cfg.budget_bytes, cfg.bytes_per_cell, cfg.autotune, cfg.device = budget, 0.0, 0, 0
    lib.psgb_solve_options_default(C.byref(cfg.options))
    srv = C.c_void_p()
    return lib.psgb_server_create(C.byref(cfg), C.byref(srv)), srv


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def test_server_entry_points_check_their_arguments():
    from planet_game_gb300 import capi

    lib = capi.load()
    assert _server(lib, capi, budget=0.0)[0] == capi.ERR_INVALID_ARGUMENT
    code, srv = _server(lib, capi)
    assert code == capi.OK
    try:
        t0 = np.full(162, 280.0)
        pid = C.c_uint32()
        bad = capi.StepParams(4e7, -1.0, 4e13, None, 0)
        assert lib.psgb_server_add_planet(srv, 2, 6.371e6, C.byref(bad), _ptr(t0), C.byref(pid)) == \
            capi.ERR_INVALID_ARGUMENT
        hot = t0.copy()
        hot[5] = np.nan
        good = capi.StepParams(4e7, 2.6e6, 4e13, None, 0)
        assert lib.psgb_server_add_planet(srv, 2, 6.371e6, C.byref(good), _ptr(hot), C.byref(pid)) == \
            capi.ERR_INVALID_ARGUMENT
        assert lib.psgb_server_add_planet(srv, 2, 6.371e6, C.byref(good), _ptr(t0), C.byref(pid)) == capi.OK
        rid = C.c_uint64()
        assert lib.psgb_server_submit(srv, 7, _ptr(np.zeros(162)), C.byref(rid)) == capi.ERR_INVALID_ARGUMENT
        assert lib.psgb_server_wait(srv, 12345, 0.0, None, None) == capi.ERR_INVALID_ARGUMENT
        out = np.empty(162)
        assert lib.psgb_server_state(srv, pid, _ptr(out)) == capi.OK and np.array_equal(out, t0)
    finally:
        lib.psgb_server_destroy(srv)


def test_server_without_a_gpu_fails_requests_cleanly():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("checks the path where no GPU can be reached")
    from planet_game_gb300 import capi

    lib = capi.load()
    code, srv = _server(lib, capi)
    assert code == capi.OK
    try:
        t0 = np.full(162, 280.0)
        pid = C.c_uint32()
        params = capi.StepParams(4e7, 2.6e6, 4e13, None, 0)
        assert lib.psgb_server_add_planet(srv, 2, 6.371e6, C.byref(params), _ptr(t0), C.byref(pid)) == capi.OK
        rid = C.c_uint64()
        assert lib.psgb_server_submit(srv, pid, _ptr(np.zeros(162)), C.byref(rid)) == capi.OK
        assert lib.psgb_server_wait(srv, rid, 60.0, None, None) == capi.ERR_CUDA
        assert lib.psgb_last_error()
        # the level's lane exists now: its planets are fixed
        assert lib.psgb_server_add_planet(srv, 2, 6.371e6, C.byref(params), _ptr(t0), C.byref(pid)) == \
            capi.ERR_INVALID_ARGUMENT
        stats = capi.ServerStats()
        assert lib.psgb_server_stats_get(srv, C.byref(stats)) == capi.OK
        assert (stats.submitted, stats.failed, stats.completed, stats.resident_lanes) == (1, 1, 0, 0)
    finally:
        lib.psgb_server_destroy(srv)


def test_python_wrapper_of_the_native_server():
    from planet_game_gb300 import capi
    from planet_game_gb300.serve import NativeServer

    with NativeServer(budget_bytes=1e9, autotune=False) as srv:
        t0 = np.linspace(250.0, 300.0, 162)
        pid = srv.add_planet(2, 6.371e6, 4e7, 2.6e6, 4e13, t0)
        assert np.array_equal(srv.state(pid), t0)
        with pytest.raises(ValueError):
            srv.add_planet(2, 6.371e6, 4e7, 2.6e6, 4e13, t0[:-1])
        with pytest.raises(ValueError):
            srv.submit(pid, np.zeros(10))
        with pytest.raises(capi.GB300Error):
            srv.add_planet(2, 6.371e6, 4e7, 0.0, 4e13, t0)
        stats = srv.stats()
        assert stats["planets"] == 1 and stats["submitted"] == 0
        srv.reset_stats()

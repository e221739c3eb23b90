#!/usr/bin/env python
"""Benchmark of the GB300 implicit heat-transport sub-step (PlanetSim).

Workload (default, `--workload batch`): the batched uneven-planet sub-step - 64 planets
(16 x L4, 24 x L5, 16 x L6, 8 x L7; 2,252,928 cells), radius U(3e6, 9e6) m, per-edge
diffusivity lognormal (median 1e6 m^2/s, sigma 0.5), the config-0 state and sources;
FP32 multigrid-preconditioned BiCGSTAB inside FP64 iterative refinement to a 1e-10
relative residual, all 64 planets solved together in the concatenated block layout. A
step is one sub-step of every planet; the metric is sub-steps/s (planets x steps / s).

`--workload l8` times the L8 plain-FP64 drop-in solve (one planet) instead.

Reported beside it, in the same JSON line: the plain one-planet-at-a-time FP64 GPU
solve of the same planets (the drop-in comparator), the end-to-end rate through the
C-ABI with host buffers, the dominant kernel's roofline (CUDA events on its launching
stream during a profiled pass over the same steps, algorithmic bytes counted on the
device), a CPU baseline (the oracle's port of the reference's FP64 PCG solve, one
host core, a bounded sample) and the SM clocks sampled during the timed region.

`--impl reference` times the reference algorithm on the host cores instead (the oracle
port, all cores, one process per core), on the same workload, metric and unit.

Multi-GPU (`torchrun ... --gpus N`): planets are independent, so every rank solves its
own replica of the workload with no data-path collective ("replicas only"); the value
is the units of all ranks over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

MEASURED_PEAKS = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0
TRAFFIC_FILE = ROOT / "profiles" / "traffic.json"


# ---- distributed helpers -----------------------------------------------------------------

def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def init_dist(world: int, backend: str):
    if world <= 1:
        return None
    import torch.distributed as dist

    dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(value: float, dist, device=None) -> float:
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ---- clocks ---------------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = [line.split(",") for line in Path(self.file.name).read_text().splitlines() if line.strip()]
        os.unlink(self.file.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, flag in zip(names, r[5:9]):
                if flag.strip().lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks() -> tuple[float, str]:
    if MEASURED_PEAKS.exists():
        return float(json.loads(MEASURED_PEAKS.read_text())["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


# ---- workloads ---------------------------------------------------------------------------------

def make_workload(kind: str, seed: int):
    """Planets and their inputs (host numpy)."""
    import planet_game_gb300 as pg
    from planet_game_gb300 import workloads as W

    planets = []
    if kind == "batch":
        for i, spec in enumerate(W.planet_mix(seed)):
            m = pg.make_icosphere(spec.level, spec.radius)
            kappa = W.lognormal_edge_diffusivity(m.edge_count, spec.seed)
            inp = W.step_inputs(m, spec.seed, edge_diffusivity=kappa)
            planets.append((m, inp))
    elif kind == "l8":
        m = pg.make_icosphere(8, W.EARTH_RADIUS)
        planets.append((m, W.step_inputs(m, seed)))
    else:
        raise SystemExit(f"unknown workload {kind}")
    return planets


def smoother_desc(tuning) -> str:
    if tuning is None:
        return "damped Jacobi 2+2 on every level, omega 0.8 (untuned)"
    if isinstance(tuning, list):
        return " | ".join(f"lane {k}: {smoother_desc(t)}" for k, t in enumerate(tuning))
    per = ", ".join(f"L{l}: {a}+{b}" for l, (a, b) in enumerate(zip(tuning["pre_sweeps"], tuning["post_sweeps"])))
    return f"damped Jacobi, autotuned sweeps per level ({per}), omega {tuning['jacobi_omega']}"


def precision_for(kind: str) -> str:
    return "mixed" if kind == "batch" else "fp64"


SOLVER = dict(method="bicgstab", tolerance=1e-10, inner_tolerance=1e-4, poll=4)


# ---- the GB300 arm ---------------------------------------------------------------------------------

def run_gb300(args, rank, world, local_rank):
    import torch

    import planet_game_gb300 as pg
    from planet_game_gb300 import capi

    torch.cuda.set_device(local_rank)
    dist = init_dist(world, "nccl")
    dev = torch.device("cuda", local_rank)
    planets = make_workload(args.workload, args.seed)
    meshes = [m for m, _ in planets]
    cells = sum(m.cell_count for m in meshes)
    prec = precision_for(args.workload)
    # the planets of the mix's highest level in a lane of their own (pg.default_lanes):
    # they need the most Krylov iterations, and the lanes run side by side
    batch = pg.LaneBatch(meshes)
    batch.concurrent = not args.serial_lanes
    t0_d = [torch.from_numpy(inp.t0).to(dev) for _, inp in planets]
    s_d = [torch.from_numpy(inp.source).to(dev) for _, inp in planets]
    out_d = [torch.empty_like(t) for t in t0_d]
    heat = [inp.heat_capacity for _, inp in planets]
    dt = [inp.dt for _, inp in planets]
    cond = [inp.conductance for _, inp in planets]
    edge_g = [inp.edge_conductance for _, inp in planets] if planets[0][1].edge_conductance is not None else None
    if edge_g is not None:      # per-edge conductances live with the batch; steps refer to them
        batch.set_edge_conductance(edge_g)
        edge_g = "stored"
    lib = capi.load()

    def step(t0, src, out):
        _, reps = batch.transport_step(t0, src, heat, dt, conductance=cond, edge_conductance=edge_g, out=out,
                                       precision=prec, **SOLVER)
        return reps

    # per-level launch shapes and sweeps picked by the autotuner (setup, not timed)
    tuning = None
    if args.tuning_in:
        tuning = json.loads(Path(args.tuning_in).read_text())
        batch.set_tuning(tuning)
    elif not args.no_autotune:
        tuning = batch.autotune(t0_d, s_d, heat, dt, conductance=cond, edge_conductance=edge_g, precision=prec,
                                **SOLVER)
    if args.tuning_out and tuning is not None and rank == 0:
        Path(args.tuning_out).write_text(json.dumps(tuning))
    for _ in range(args.warmup):
        reps = step(t0_d, s_d, out_d)
    torch.cuda.synchronize()
    bad = [r for r in reps if r.status != 0 or r.relative_residual > 1e-10 or r.closure > 1e-12]
    if bad:
        raise SystemExit(f"solve failed its gates: {bad[0]}")

    # timed region: inputs resident in HBM
    stream = torch.cuda.current_stream()
    launches0 = lib.psgb_launch_count()
    with ClockSampler(local_rank) as clocks:
        barrier(dist)
        torch.cuda.synchronize()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        iters = []
        for _ in range(args.steps):
            torch.cuda.nvtx.range_push("timed_step")     # ncu --nvtx-include "timed_step/" selects these launches
            reps = step(t0_d, s_d, out_d)
            torch.cuda.nvtx.range_pop()
            iters.append(sum(r.iterations * m.cell_count for r, m in zip(reps, meshes)))
        end.record(stream)
        torch.cuda.synchronize()
        barrier(dist)
    launches = lib.psgb_launch_count() - launches0
    elapsed = max_over_ranks(start.elapsed_time(end) / 1e3, dist, dev)
    units = len(meshes) * args.steps * world
    value = units / elapsed
    clock = clocks.summary()
    refinements = [r.refinements for r in reps]

    # end to end: host buffers, copies inside the timed region
    t0_h = [inp.t0 for _, inp in planets]
    s_h = [inp.source for _, inp in planets]
    out_h = [np.empty_like(x) for x in t0_h]
    barrier(dist)
    torch.cuda.synchronize()
    t_e2e = time.perf_counter()
    for _ in range(args.steps):
        step(t0_h, s_h, out_h)
    torch.cuda.synchronize()
    e2e_elapsed = max_over_ranks(time.perf_counter() - t_e2e, dist, dev)
    e2e = {"value": units / e2e_elapsed, "unit": "sub-steps/s", "h2d_bytes_per_step": cells * 16,
           "d2h_bytes_per_step": cells * 8}

    # profiled pass: the dominant kernel family timed with events on its stream
    import ctypes as C

    peak, peak_kind = peaks()
    traffic_all = json.loads(TRAFFIC_FILE.read_text()) if TRAFFIC_FILE.exists() else {}

    def profile_family(family: bytes, kernel: str) -> dict:
        ms, nl, nbytes = C.c_double(), C.c_uint64(), C.c_uint64()
        batch.concurrent = False      # one launch at a time between a family's events
        capi.check(lib.psgb_profile_begin(family))
        for _ in range(args.steps):
            step(t0_d, s_d, out_d)
        capi.check(lib.psgb_profile_end(C.byref(ms), C.byref(nl), C.byref(nbytes)))
        batch.concurrent = not args.serial_lanes
        achieved = nbytes.value / (ms.value / 1e3) / 1e9 if ms.value > 0 else None
        traffic = (traffic_all.get(args.workload) or {}).get(family.decode())
        return {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "peak_kind": peak_kind,
                "unit": "GB/s", "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                "launches": int(nl.value), "avg_launch_us": ms.value * 1e3 / max(1, nl.value),
                "bytes_per_launch": nbytes.value / max(1, nl.value), "share_of_step": ms.value / args.steps / (elapsed * 1e3 / args.steps)}

    if args.schedule == "persistent":
        roofline = profile_family(b"persistent", "k_persistent_solve (whole refined solve; Jacobi-sweep bytes)")
        roofline_coarse = None
    else:
        roofline = profile_family(b"smooth", "k_smooth / k_prolong_smooth / k_smooth_zero on the fine level")
        roofline_coarse = profile_family(b"smooth_coarse", "k_smooth / k_prolong_smooth on the coarse levels")

    # the plain one-planet-at-a-time FP64 GPU drop-in on the same planets
    plain = None
    if rank == 0 and not args.skip_plain:
        for i, (m, inp) in enumerate(planets):   # warm the solo batches
            pg.transport_step(m, t0_d[i], s_d[i], inp.heat_capacity, inp.dt, inp.conductance,
                              edge_conductance=inp.edge_conductance, precision="fp64", **SOLVER)
        torch.cuda.synchronize()
        tp = time.perf_counter()
        plain_iters = 0
        for i, (m, inp) in enumerate(planets):
            _, _, r = pg.transport_step(m, t0_d[i], s_d[i], inp.heat_capacity, inp.dt, inp.conductance,
                                        edge_conductance=inp.edge_conductance, precision="fp64", **SOLVER)
            plain_iters += r.iterations
            if r.status != 0:
                raise SystemExit(f"plain FP64 solve failed: {r}")
        torch.cuda.synchronize()
        plain = {"value": len(planets) / (time.perf_counter() - tp), "unit": "sub-steps/s",
                 "krylov_iterations": plain_iters, "solver": "FP64 AMG-BiCGSTAB, one planet per call"}

    serving = serving_point(args, dev, rate=args.serve_rate, count=args.serve_requests) \
        if (rank == 0 and not args.skip_serve) else None
    cpu = cpu_baseline(planets, args) if (rank == 0 and not args.skip_cpu) else None
    if rank == 0:
        line = {
            "metric": "sub-steps/s at 1e-10 relative residual",
            "value": value,
            "unit": "sub-steps/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": elapsed * 1e3 / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32 inner, f64 refinement" if prec == "mixed" else "f64",
            "data": "synthetic",
            "config": {
                "workload": ("64 uneven planets (16xL4, 24xL5, 16xL6, 8xL7; 2,252,928 cells), per-edge lognormal "
                             "diffusivity, one batched sub-step per step" if args.workload == "batch"
                             else "one L8 planet (655,362 cells), plain FP64 drop-in solve"),
                "planets": len(meshes), "cells": cells, "precision": prec, "krylov": "BiCGSTAB",
                "lanes": [sorted({meshes[i].subdivision for i in lane}) for lane in batch.lanes],
                "smoother": smoother_desc(tuning), "tuning": tuning, "tolerance": 1e-10,
                "krylov_iterations_per_step": sum(r.iterations for r in reps), "refinements_last_step": max(refinements),
                "krylov_iterations_per_planet": {"min": min(r.iterations for r in reps),
                                                 "median": float(np.median([r.iterations for r in reps])),
                                                 "max": max(r.iterations for r in reps)},
                "cell_iterations_per_s": statistics.mean(iters) * world / (elapsed / args.steps),
                "l2": "working set larger than the 129 MB L2 (no flush needed)" if cells > 1_000_000 else
                      "working set may be L2 resident",
                "plain_fp64_one_at_a_time": plain,
                "parallelism": f"replicas x{world}",
            },
            "e2e": e2e,
            "serving": serving,
            "roofline": roofline,
            "roofline_coarse_sweeps": roofline_coarse,
            "cpu_baseline": cpu,
            "clocks": clock,
            "gpu_launches": int(launches),
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


# ---- serving ------------------------------------------------------------------------------------

SERVE_POPULATION = {4: 16, 5: 16, 6: 16, 7: 8, 8: 4}


def serving_point(args, dev, rate: float, count: int, population=None) -> dict:
    """A seeded Poisson trace of `count` requests over L4-L8 (30/30/20/15/5 %) at `rate`
    requests/s, served by the continuous-batching loop (mixed precision) and by the plain
    FP64 one-at-a-time drop-in, with p50/p99 latency from arrival to result on the host."""
    import torch

    from planet_game_gb300 import serve
    from planet_game_gb300 import workloads as W

    out = {"requests": count, "offered_per_s": rate, "population": {f"L{k}": v for k, v in SERVE_POPULATION.items()},
           "budget_gb": 150}
    for name in ("continuous_batching_mixed", "one_at_a_time_fp64"):
        pop = build_serve_population(dev)
        trace = W.poisson_trace(count, rate, seed=args.seed + 1, planets_per_level=max(SERVE_POPULATION.values()))
        trace = [W.Request(r.arrival_s, r.level, r.planet % SERVE_POPULATION[r.level]) for r in trace]
        reqs = serve.make_requests(trace, pop, seed=args.seed + 2)
        if name.startswith("continuous"):
            srv = serve.Server(pop, budget_bytes=150e9, precision="mixed", **SOLVER_SERVE)
            srv.prepare()                                                      # admit and tune the lanes
            warm = serve.make_requests(trace[:40], pop, seed=args.seed + 3)   # record graphs
            srv.run_trace(warm, realtime=False)
            srv.completed = 0
            try:
                srv.run_trace(reqs, realtime=True)
            finally:
                srv.close()
        else:
            srv = serve.OneAtATime(pop, **SOLVER_SERVE)
            warm = serve.make_requests(trace[:40], pop, seed=args.seed + 3)
            srv.run_trace(warm, realtime=False)
            srv.run_trace(reqs, realtime=True)
        torch.cuda.synchronize()
        summary = serve.summarize(reqs)
        if summary["ok"] != count:
            raise SystemExit(f"serving: {count - summary['ok']} requests failed")
        out[name] = summary
    a, b = out["continuous_batching_mixed"], out["one_at_a_time_fp64"]
    out["speedup_sub_steps_per_s"] = a["sub_steps_per_s"] / b["sub_steps_per_s"]
    if getattr(args, "native_serve", False):
        out["continuous_batching_native"] = native_serving_point(args, dev, rate, count)
    return out


def native_serving_point(args, dev, rate: float, count: int) -> dict:
    """The same trace through the library's own serving loop (psgb_server_*): lanes and
    their threads in C++, host arrays in and out; latency from submission to completion as
    the loop records it, after a warm-up that admits and tunes every lane."""
    from planet_game_gb300 import serve
    from planet_game_gb300 import workloads as W

    pop = build_serve_population(dev)
    trace = W.poisson_trace(count, rate, seed=args.seed + 1, planets_per_level=max(SERVE_POPULATION.values()))
    trace = [W.Request(r.arrival_s, r.level, r.planet % SERVE_POPULATION[r.level]) for r in trace]
    reqs = serve.make_requests(trace, pop, seed=args.seed + 2)
    warm = serve.make_requests(trace[:40], pop, seed=args.seed + 3)
    srv = serve.NativeServer(budget_bytes=150e9, precision="mixed", **SOLVER_SERVE)
    try:
        ids = {}
        for level, planets in pop.items():
            for i, p in enumerate(planets):
                ids[(level, i)] = srv.add_planet(level, p.radius, p.heat_capacity, p.dt, p.conductance,
                                                 p.state.cpu().numpy(), p.edge_conductance)
        for level in pop:   # admit and tune every lane
            pid = ids[(level, 0)]
            srv.wait(srv.submit(pid, np.zeros(pop[level][0].mesh.cell_count)), pid)
        for r in warm:
            pid = ids[(r.level, r.planet)]
            srv.wait(srv.submit(pid, r.source), pid)
        srv.reset_stats()
        t_start = time.perf_counter()
        pending = []
        for r in reqs:
            delay = r.arrival_s - (time.perf_counter() - t_start)
            if delay > 0:
                time.sleep(delay)
            pid = ids[(r.level, r.planet)]
            pending.append((r, srv.submit(pid, r.source), pid))
        for r, rid, pid in pending:
            r.result, rep = srv.wait(rid, pid)
            r.status = rep.solve.status
        elapsed = time.perf_counter() - t_start
        stats = srv.stats()
    finally:
        srv.close()
    return {"requests": count, "sub_steps_per_s": count / elapsed, "p50_ms": stats["p50_ms"],
            "p99_ms": stats["p99_ms"], "ok": int(sum(r.status == 0 for r in reqs)),
            "latency": "submission to completion, recorded by the loop"}


SOLVER_SERVE = dict(method="bicgstab", tolerance=1e-10, inner_tolerance=1e-4, poll=4)


def build_serve_population(dev):
    from planet_game_gb300 import serve

    pop = {}
    for level, n in SERVE_POPULATION.items():
        pop.update(serve.build_population(n, levels=(level,), seed=100 + level, device=dev))
    return pop


def run_serve_sweep(args, rank, local_rank):
    """The full offered-rate sweep (50 -> 5000 requests/s), one JSON line."""
    import torch

    if rank != 0:
        return
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    points = [serving_point(args, dev, rate, args.serve_requests) for rate in (50.0, 200.0, 1000.0, 5000.0)]
    best = max(points, key=lambda p: p["continuous_batching_mixed"]["sub_steps_per_s"])
    print(json.dumps({"metric": "served sub-steps/s and p50/p99 at 1e-10 relative residual", "unit": "sub-steps/s",
                      "value": best["continuous_batching_mixed"]["sub_steps_per_s"], "n_gpus": 1,
                      "higher_is_better": True, "data": "synthetic", "sweep": points}))


# ---- the rows that widen the hot path -------------------------------------------------------

class _DeviceArray:
    """A raw device pointer as a CUDA array (torch.as_tensor without a copy)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False), "version": 3,
                                         "stream": None}


def _median_ms(fn, repeats: int = 5) -> float:
    import statistics

    import torch

    fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(repeats):
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        times.append((time.perf_counter() - t) * 1e3)
    return statistics.median(times)


def run_next(args, rank, local_rank):
    """GPU timings of the widened rows on the cases oracle/time_reference.py times with the
    reference's CPU code (same shapes, same seeds): the implicit tracer on the L7 mesh's
    agglomerated graph (10 layers), the transport step on the L8 mesh's agglomerated graph,
    the L8 sub-step-mean insolation, the coupled advection-diffusion solve on the L6 graph
    (3 layers, the reference test's column on the GPU). Host arrays in and out (as the
    reference's calls), device-resident where noted. One JSON line."""
    import torch

    import planet_game_gb300 as pg
    from planet_game_gb300 import workloads as W

    if rank != 0:
        return
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    R, CP = W.EARTH_RADIUS, 1004.64
    out = {"metric": "ms per call of the widened rows (median of 5)", "unit": "ms", "n_gpus": 1, "data": "synthetic"}
    # the mesh builder (host, all cores): the first L8 mesh of the process, then another radius
    t = time.perf_counter()
    pg.make_icosphere(8, R)
    out["mesh_l8_first_ms"] = (time.perf_counter() - t) * 1e3
    t = time.perf_counter()
    pg.make_icosphere(8, 0.5 * R)
    out["mesh_l8_radius_ms"] = (time.perf_counter() - t) * 1e3
    out["host_cores"] = os.cpu_count()
    # tracer
    p7 = pg.agglomerated_transport_graph(7, R)
    g7 = pg.mesh_transport_graph(p7)
    n7, layers = p7.cell_count, 10
    flux = W.antisymmetric_layer_fluxes(g7.offset, g7.neighbour, layers, 2e9, seed=71, column_balanced=False)
    cond = np.full(len(g7.neighbour), 2e8)
    mass = g7.area_m2 * 100000.0 / (9.81 * layers)
    tracer = W.tracer_field(layers * n7, seed=72)
    tr_h = pg.AdvectionDiffusion(layers, cond, flux, CP)
    res = {}
    out["tracer_ms"] = _median_ms(lambda: res.update(r=pg.solve_implicit_tracer(p7, tr_h, mass, tracer, 2.63e6)))
    out["tracer_iterations"] = res["r"].iterations
    out["tracer_rows"] = layers * n7
    tr_d = pg.AdvectionDiffusion(layers, torch.as_tensor(cond, device=dev), torch.as_tensor(flux, device=dev), CP)
    mass_d, tracer_d = torch.as_tensor(mass, device=dev), torch.as_tensor(tracer, device=dev)
    out["tracer_resident_ms"] = _median_ms(lambda: pg.solve_implicit_tracer(p7, tr_d, mass_d, tracer_d, 2.63e6))
    # agglomerated transport step (plain FP64 and mixed)
    p8 = pg.agglomerated_transport_graph(8, R)
    t0, source = W.agglomerated_step_inputs(p8.cell_count, seed=81)
    for prec in ("fp64", "mixed"):
        rep = {}
        out[f"agglomerated_{prec}_ms"] = _median_ms(lambda: rep.update(r=pg.transport_step(
            p8, t0, source, W.HEAT_CAPACITY, W.SUBSTEP_S, W.HEAT_CAPACITY * W.DIFFUSIVITY, precision=prec)[2]))
        out[f"agglomerated_{prec}_iterations"] = rep["r"].iterations
    out["agglomerated_nodes"] = p8.cell_count
    # insolation at L8
    m8 = pg.make_icosphere(8, R)
    ins = torch.empty(m8.cell_count, dtype=torch.float32, device=dev)
    out["insolation_resident_ms"] = _median_ms(lambda: m8.substep_mean_insolation_gpu(0, ins))
    out["insolation_ms"] = _median_ms(lambda: m8.substep_mean_insolation_gpu(0))
    # coupled advection-diffusion on the L6 graph, the column on the GPU
    m6 = pg.make_icosphere(6, R)
    g6 = pg.mesh_transport_graph(m6)
    n6 = m6.cell_count
    flux6 = W.antisymmetric_layer_fluxes(g6.offset, g6.neighbour, 3, 5e9, seed=61, column_balanced=True)
    cond6 = 0.5 * R * R * g6.weight
    a, radiative = 3.0e5 / (30.0 * 86400.0), 0.75 * 0.97 * pg.api.STEFAN_BOLTZMANN_W_M2_K4
    b, floor = W.quartic_column(a, radiative, n6, seed=62)
    eps = torch.tensor([0.0, -0.08, -0.16], dtype=torch.float64, device=dev)[:, None]
    phi = torch.tensor([3.0e4, 4.5e4, 7.0e4], dtype=torch.float64, device=dev)[:, None]
    q = pg.QuarticResponse(a, torch.as_tensor(b, device=dev), radiative, hold_stride=0)

    def column(nodes, nl, src, mean, slope, energy, energy_slope, stream):
        h = torch.as_tensor(_DeviceArray(src, nodes), device=dev)
        x, s = pg.quartic_response(q, h)
        torch.as_tensor(_DeviceArray(mean, nodes), device=dev).copy_(x)
        torch.as_tensor(_DeviceArray(slope, nodes), device=dev).copy_(s)
        torch.as_tensor(_DeviceArray(energy, nodes * nl), device=dev).view(nl, nodes).copy_(CP * x * (1.0 + eps) + phi)
        torch.as_tensor(_DeviceArray(energy_slope, nodes * nl), device=dev).view(nl, nodes).copy_(CP * s * (1.0 + eps))

    tr6 = pg.AdvectionDiffusion(3, cond6, flux6, CP)
    settings = {"cg_relative_tolerance": 1e-6, "newton_tolerance_W_m2": 1e-6}
    ad = {}
    out["advection_ms"] = _median_ms(lambda: ad.update(r=pg.solve_implicit_advection_diffusion(
        m6, tr6, floor, column, settings=settings, device=True)))
    out["advection_newton"], out["advection_linear"] = ad["r"].newton_iterations, ad["r"].linear_iterations
    print(json.dumps(out))


# ---- CPU baseline and the reference arm ------------------------------------------------------

def _oracle_solve(payload):
    """One planet's sub-step by the oracle's port of the reference (FP64 PCG + SGS V-cycle)."""
    arrays, inp, edge_g, tol = payload
    from oracle import oracle as O

    om = O.OracleMesh(arrays)
    h = O.OracleHierarchy(om)
    t = time.perf_counter()
    out = h.transport_step(inp["conductance"], inp["heat_capacity"], inp["dt"], inp["t0"], inp["source"], tol=tol,
                           edge_g=None if edge_g is None else om.directed_conductance(edge_g))
    return time.perf_counter() - t, out["iterations"]


def _payload(m, inp):
    return (m.arrays(), {"conductance": inp.conductance, "heat_capacity": inp.heat_capacity, "dt": inp.dt,
                         "t0": inp.t0, "source": inp.source}, inp.edge_conductance, 1e-10)


def cpu_baseline(planets, args):
    """A bounded sample on one host core: every planet of the mix once (about 10-30 s)."""
    from oracle import oracle as O  # noqa: F401  (the checker; timed here as the CPU baseline)

    total, iters = 0.0, 0
    for m, inp in planets:
        dt, it = _oracle_solve(_payload(m, inp))
        total += dt
        iters += it
    return {"value": len(planets) / total, "unit": "sub-steps/s", "cores": 1, "kind": "port",
            "sample": f"all {len(planets)} planets of the workload once, one core, FP64 PCG + SGS V-cycle to 1e-10 "
                      "(the oracle's restatement of the reference's solve: bit-identical solutions, within 1% of the "
                      "reference's own speed where both compile)",
            "pcg_iterations": iters}


def run_reference(args, rank, world):
    if rank != 0:
        return
    import multiprocessing as mp

    planets = make_workload(args.workload, args.seed)
    payloads = [_payload(m, inp) for m, inp in planets]
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(processes=cores) as pool:
        for _ in range(args.warmup):
            pool.map(_oracle_solve, payloads, chunksize=1)
        t = time.perf_counter()
        for _ in range(args.steps):
            results = pool.map(_oracle_solve, payloads, chunksize=1)
        elapsed = time.perf_counter() - t
    value = len(planets) * args.steps / elapsed
    line = {
        "impl": "reference",
        "metric": "sub-steps/s at 1e-10 relative residual",
        "value": value,
        "unit": "sub-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": elapsed * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "same planets and inputs as the GB300 arm", "planets": len(planets),
                   "cells": sum(m.cell_count for m, _ in planets), "pcg_iterations": sum(r[1] for r in results)},
        "cpu_baseline": {"value": value, "unit": "sub-steps/s", "cores": cores, "kind": "port",
                         "sample": "every planet of the workload per step, one process per core (the oracle's "
                                   "restatement of the reference's FP64 PCG + SGS solve: bit-identical solutions, "
                                   "within 1% of the reference's own speed where both compile)"},
        "e2e": {"value": value, "unit": "sub-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=["batch", "l8", "serve", "next"], default="batch")
    ap.add_argument("--serve-rate", type=float, default=5000.0)
    ap.add_argument("--serve-requests", type=int, default=2000)
    ap.add_argument("--skip-serve", action="store_true")
    ap.add_argument("--native-serve", action="store_true",
                    help="serving: also run the trace through the library's own loop (psgb_server_*)")
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="uniform 2+2 Jacobi sweeps, default launch shapes")
    ap.add_argument("--tuning-out", help="write the autotuned settings (JSON) here")
    ap.add_argument("--tuning-in", help="use these settings (JSON from --tuning-out) instead of autotuning; "
                                        "profiling runs use it, since timings under a profiler are not the real ones")
    ap.add_argument("--serial-lanes", action="store_true",
                    help="step the lanes one after another (profiling runs: the profiler serialises kernels anyway)")
    ap.add_argument("--schedule", choices=["auto", "kernels", "persistent"], default="auto",
                    help="persistent: one cooperative kernel per solve; kernels: one kernel per phase")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    SOLVER["schedule"] = SOLVER_SERVE["schedule"] = args.schedule
    rank, world, local_rank = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "serve":
        run_serve_sweep(args, rank, local_rank)
        return
    if args.workload == "next":
        run_next(args, rank, local_rank)
        return
    run_gb300(args, rank, world, local_rank)


if __name__ == "__main__":
    main()

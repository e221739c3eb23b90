#!/usr/bin/env python
"""Benchmark of the GB300 implicit heat-transport sub-step (PlanetSim).

Workload (default, `--workload batch`): the batched uneven-planet sub-step - 64 planets
(16 x L4, 24 x L5, 16 x L6, 8 x L7; 2,252,928 cells), radius U(3e6, 9e6) m, per-edge
diffusivity lognormal (median 1e6 m^2/s, sigma 0.5), the config-0 state and sources;
FP32 multigrid-preconditioned BiCGSTAB inside FP64 iterative refinement to a 1e-10
relative residual, all 64 planets solved together in the concatenated block layout. A
step is one sub-step of every planet; the metric is sub-steps/s (planets x steps / s).

Reported beside it, in the same JSON line:
* `e2e`: the same through the C-ABI with host buffers, copies inside the timed region;
* `reassembled`: the same with the matrix, its Galerkin coarse values and the coarsest
  inverses assembled again on every step (the timed step otherwise reuses them while C,
  dt and the conductances are unchanged);
* `oracle_error`: every planet's T and H against the oracle (the reference's FP64 PCG +
  SGS V-cycle solve, restated) on the same inputs;
* `plain_fp64_one_at_a_time`: the same planets solved one per call in plain FP64, tuned
  per level as the batch is (and untuned);
* `serving`: the served workload (a Poisson trace over L4-L8) swept over offered rates
  50 -> 5000 requests/s through the continuous-batching loop and the tuned plain FP64
  one-at-a-time comparator, with p50/p99 latency; `headline_served` is its saturated point;
* `roofline` (the fine-level Jacobi sweeps) and `kernels` (every profiled kernel family:
  algorithmic GB/s from bytes counted on the device over CUDA-event kernel time);
* `cpu_baseline`: the oracle's port of the reference's solve on one host core.

Other workloads: `l8` (one L8 planet, plain FP64), `l8rhs` (one L8 planet with 32 right-hand
sides, plain FP64 and mixed, in one multi-RHS block), `ops` (the L6 operator sweep, L6 solve
and 10-layer column radiation), `serve` (the serving sweep alone), `next` (the widened rows).

`--impl reference` times the reference algorithm on the host cores instead (the oracle's
port, all cores, one process per core) on the same workload, metric and unit; it builds
its planets with the oracle's own mesh builder, without the product library.

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

WORKLOAD_NAMES = {
    "batch": "64 uneven planets (16xL4, 24xL5, 16xL6, 8xL7; 2,252,928 cells), per-edge lognormal diffusivity, "
             "one batched sub-step per step",
    "l8": "one L8 planet (655,362 cells), plain FP64 drop-in solve",
}


def make_workload(kind: str, seed: int):
    """Planets and their inputs (host numpy), meshes from the product's builder."""
    import planet_game_gb300 as pg
    from planet_game_gb300 import workloads as W

    planets = []
    if kind == "batch":
        for spec in W.planet_mix(seed):
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


def oracle_workload(kind: str, seed: int):
    """The same planets and inputs built by the oracle alone (its restatement of the
    reference's mesh builder and sub-step insolation, the reference's own orbit nodes from
    the committed fixture): the CPU arms never load the product library."""
    from oracle import oracle as O
    from planet_game_gb300 import workloads as W   # numpy only: no library is loaded

    nodes = np.load(ROOT / "tests" / "golden" / "insolation_L4.npz")["nodes"]
    out = []
    if kind == "batch":
        for spec in W.planet_mix(seed):
            a = O.icosphere(spec.level, spec.radius)
            kappa = W.lognormal_edge_diffusivity(len(a["edge_length_m"]), spec.seed)
            out.append((a, W.step_inputs_from(a["center"], O.substep_mean_insolation(a["center"], nodes), spec.seed,
                                              kappa)))
    elif kind == "l8":
        a = O.icosphere(8, W.EARTH_RADIUS)
        out.append((a, W.step_inputs_from(a["center"], O.substep_mean_insolation(a["center"], nodes), seed)))
    else:
        raise SystemExit(f"unknown workload {kind}")
    return out


def smoother_desc(tuning) -> str:
    if tuning is None:
        return "damped Jacobi 2+2 on every level, omega 0.8 (untuned)"
    if isinstance(tuning, list):
        return " | ".join(f"lane {k}: {smoother_desc(t)}" for k, t in enumerate(tuning))
    per = ", ".join(f"L{l}: {a}+{b}" + (f" x{k}" if k > 1 else "") for l, (a, b, k) in
                    enumerate(zip(tuning["pre_sweeps"], tuning["post_sweeps"],
                                  tuning.get("block_sweeps", [1] * len(tuning["pre_sweeps"])))))
    scale = tuning.get("coarse_correction", 1.0)
    return (f"damped Jacobi, autotuned sweeps per level ({per}), omega {tuning['jacobi_omega']}"
            + (f", coarse-grid correction x{scale}" if scale != 1.0 else ""))


def precision_for(kind: str) -> str:
    return "mixed" if kind == "batch" else "fp64"


SOLVER = dict(method="bicgstab", tolerance=1e-10, inner_tolerance=1e-4, poll=4)


def static_config(kind: str, planets: int, cells: int) -> dict:
    """The workload's description, the same in both arms' lines."""
    return {"workload": WORKLOAD_NAMES[kind], "planets": planets, "cells": cells, "tolerance": 1e-10}


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
    # the planets of the mix's highest level in lanes of their own, at most four each
    # (pg.default_lanes): they need the most Krylov iterations, and the lanes run side by side
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

    def step(t0, src, out, h=None):
        _, reps = batch.transport_step(t0, src, heat, dt, conductance=cond, edge_conductance=edge_g, out=out,
                                       transport_out=h, precision=prec, **SOLVER)
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

    def timed(steps: int):
        """`steps` steps bracketed by a barrier and device synchronisation, CUDA events on
        the stream the steps are ordered on; max over ranks."""
        stream = torch.cuda.current_stream()
        barrier(dist)
        torch.cuda.synchronize()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        its = []
        for _ in range(steps):
            torch.cuda.nvtx.range_push("timed_step")     # ncu --nvtx-include "timed_step/" selects these launches
            r = step(t0_d, s_d, out_d)
            torch.cuda.nvtx.range_pop()
            its.append(sum(x.iterations * m.cell_count for x, m in zip(r, meshes)))
        end.record(stream)
        torch.cuda.synchronize()
        barrier(dist)
        return max_over_ranks(start.elapsed_time(end) / 1e3, dist, dev), r, its

    # timed region: inputs resident in HBM
    launches0 = lib.psgb_launch_count()
    with ClockSampler(local_rank) as clocks:
        elapsed, reps, iters = timed(args.steps)
    launches = lib.psgb_launch_count() - launches0
    units = len(meshes) * args.steps * world
    value = units / elapsed
    clock = clocks.summary()
    refinements = [r.refinements for r in reps]

    # end to end: pinned host buffers (numpy views of page-locked memory), copies inside the
    # timed region
    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
        view = t.numpy()
        view[:] = a
        return view

    t0_h = [pinned(inp.t0) for _, inp in planets]
    s_h = [pinned(inp.source) for _, inp in planets]
    out_h = [pinned(np.zeros_like(x)) for x in t0_h]
    barrier(dist)
    torch.cuda.synchronize()
    t_e2e = time.perf_counter()
    for _ in range(args.steps):
        step(t0_h, s_h, out_h)
    torch.cuda.synchronize()
    e2e_elapsed = max_over_ranks(time.perf_counter() - t_e2e, dist, dev)
    e2e = {"value": units / e2e_elapsed, "unit": "sub-steps/s", "h2d_bytes_per_step": cells * 16,
           "d2h_bytes_per_step": cells * 8}

    # the same steps with the matrix assembled again every step (as the reference does)
    batch.set_reassembly(True)
    step(t0_d, s_d, out_d)
    re_elapsed, re_reps, _ = timed(args.steps)
    batch.set_reassembly(False)
    reassembled = {"value": units / re_elapsed, "unit": "sub-steps/s", "ms_per_step": re_elapsed * 1e3 / args.steps,
                   "what": "every step assembles the fine matrix from C, dt and the per-edge conductances, the "
                           "Galerkin values of every coarse level and the coarsest levels' inverses on the device; "
                           "the headline steps reuse them while those parameters are unchanged",
                   "same_iterations": [r.iterations for r in re_reps] == [r.iterations for r in reps]}

    # every planet's result against the oracle (FP64 PCG + SGS V-cycle, tight tolerance)
    oracle_error = None
    if rank == 0 and not args.skip_cpu:
        h_d = [torch.empty_like(t) for t in t0_d]
        step(t0_d, s_d, out_d, h_d)
        torch.cuda.synchronize()
        oracle_error = oracle_errors(planets, [o.cpu().numpy() for o in out_d], [h.cpu().numpy() for h in h_d])

    # profiled pass: kernel families timed with events on their stream, bytes counted on the device
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
        achieved = nbytes.value / (ms.value / 1e3) / 1e9 if ms.value > 0 and nbytes.value > 0 else None
        per_launch = nbytes.value / max(1, nl.value)
        # DRAM bytes per algorithmic byte of the family's dominant kernel, from a committed
        # ncu capture of a few launches, applied to this run's algorithmic bytes per launch
        entry = (traffic_all.get(args.workload) or {}).get(family.decode())
        traffic = source = None
        if isinstance(entry, dict) and per_launch > 0:
            traffic = entry["dram_per_algorithmic"] * per_launch
            source = (f"ncu dram__bytes_read+write per algorithmic byte of {entry['kernel']} "
                      f"({entry['launches']} launches, {entry['summary']}) x this run's algorithmic bytes per launch")
        return {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "peak_kind": peak_kind,
                "unit": "GB/s", "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                "traffic_source": source,
                "launches": int(nl.value), "avg_launch_us": ms.value * 1e3 / max(1, nl.value),
                "bytes_per_launch": per_launch,
                "share_of_step": ms.value / args.steps / (elapsed * 1e3 / args.steps)}

    kernels = {}
    if args.schedule == "persistent":
        roofline = profile_family(b"persistent", "k_persistent_solve (whole refined solve; Jacobi-sweep bytes)")
    else:
        roofline = profile_family(b"smooth", "k_smooth / k_prolong_smooth / k_smooth_zero on the fine level")
        for fam, desc in PROFILED_FAMILIES:
            kernels[fam] = profile_family(fam.encode(), desc)

    # the plain one-planet-at-a-time FP64 GPU drop-in on the same planets
    plain = None
    if rank == 0 and not args.skip_plain:
        plain = plain_comparator(planets, t0_d, s_d, torch)

    serving = serving_sweep(args, dev) if (rank == 0 and not args.skip_serve) else None
    cpu = cpu_baseline(planets, args) if (rank == 0 and not args.skip_cpu) else None
    if rank == 0:
        config = static_config(args.workload, len(meshes), cells)
        config.update({
            "precision": prec, "krylov": "BiCGSTAB", "parallelism": f"replicas x{world}",
            "lanes": [sorted({meshes[i].subdivision for i in lane}) for lane in batch.lanes],
            "smoother": smoother_desc(tuning), "tuning": tuning,
            "krylov_iterations_per_step": sum(r.iterations for r in reps), "refinements_last_step": max(refinements),
            "krylov_iterations_per_planet": {"min": min(r.iterations for r in reps),
                                             "median": float(np.median([r.iterations for r in reps])),
                                             "max": max(r.iterations for r in reps)},
            "cell_iterations_per_s": statistics.mean(iters) * world / (elapsed / args.steps),
            "l2": "working set larger than the 129 MB L2 (no flush needed)" if cells > 1_000_000 else
                  "working set may be L2 resident",
            "matrix": "assembled once and reused while C, dt and the conductances are unchanged (as in a run of "
                      "sub-steps with constant coefficients); `reassembled` times the same steps assembling it "
                      "every step",
            "plain_fp64_one_at_a_time": plain,
        })
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
            "config": config,
            "e2e": e2e,
            "reassembled": reassembled,
            "oracle_error": oracle_error,
            "headline_served": serving.get("headline") if serving else None,
            "serving": serving,
            "roofline": roofline,
            "kernels": kernels,
            "cpu_baseline": cpu,
            "clocks": clock,
            "gpu_launches": int(launches),
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


# Kernel families profiled beside the headline roofline (psgb_profile_begin names).
PROFILED_FAMILIES = (
    ("smooth_coarse", "k_smooth / k_smooth_block / k_prolong_smooth on the coarse levels"),
    ("residual", "k_residual, fine level"),
    ("residual_coarse", "k_residual, coarse levels"),
    ("restrict", "k_restrict_zero from the fine level"),
    ("restrict_coarse", "k_restrict_zero between coarse levels"),
    ("dense", "k_dense_solve (coarsest levels)"),
    ("krylov_spmv", "k_bicg_v / k_bicg_t (SpMV with fused dots)"),
    ("krylov_vector", "k_bicg_init / p / s / x (vector updates with fused dots)"),
    ("refine", "k_outer_init / residual / update (FP64 refinement)"),
    ("step", "k_step_rhs / k_step_finish (right-hand side, flux form, closure sums)"),
)


def plain_comparator(planets, t0_d, s_d, torch) -> dict:
    """The planets one per call in plain FP64: tuned once per level (api.TunedSolo), and
    through the untuned single-planet entry point."""
    import planet_game_gb300 as pg

    out = {"unit": "sub-steps/s", "solver": "FP64 AMG-BiCGSTAB, one planet per call"}
    solo = pg.TunedSolo(precision="fp64", **SOLVER)
    for name, fn in (
        ("untuned", lambda i, m, inp: pg.transport_step(m, t0_d[i], s_d[i], inp.heat_capacity, inp.dt,
                                                        inp.conductance, edge_conductance=inp.edge_conductance,
                                                        precision="fp64", **SOLVER)[2]),
        ("tuned", lambda i, m, inp: solo.step(m, t0_d[i], s_d[i], inp.heat_capacity, inp.dt, inp.conductance,
                                              edge_conductance=inp.edge_conductance)[1]),
    ):
        for i, (m, inp) in enumerate(planets):   # warm: batches, tunings, graphs
            fn(i, m, inp)
        torch.cuda.synchronize()
        tp = time.perf_counter()
        its = 0
        for i, (m, inp) in enumerate(planets):
            r = fn(i, m, inp)
            its += r.iterations
            if r.status != 0:
                raise SystemExit(f"plain FP64 solve failed: {r}")
        torch.cuda.synchronize()
        out[name] = {"value": len(planets) / (time.perf_counter() - tp), "krylov_iterations": its}
    out["value"] = out["tuned"]["value"]
    out["tunings_per_level"] = {f"L{k[0]}": smoother_desc(t) for k, t in solo.tunings.items()}
    return out


def oracle_errors(planets, t_gpu, h_gpu) -> dict:
    """Max |T_gpu - T_oracle| and |H_gpu - H_oracle| over every planet, the oracle (the
    reference's FP64 PCG + SGS V-cycle solve, restated) to a 1e-13 relative residual on
    the same inputs, its solves spread over the host cores (spawned processes)."""
    import multiprocessing as mp

    payloads = [(m.arrays(), inp_dict(inp), inp.edge_conductance, 1e-13) for m, inp in planets]
    with mp.get_context("spawn").Pool(processes=max(1, min(len(payloads), os.cpu_count() or 1))) as pool:
        results = pool.map(_oracle_solve_full, payloads, chunksize=1)
    rows = []
    for (m, _), tg, hg, (tn, h) in zip(planets, t_gpu, h_gpu, results):
        rows.append((m.subdivision, float(np.max(np.abs(tg - tn))), float(np.max(np.abs(tn))),
                     float(np.max(np.abs(hg - h))), float(np.max(np.abs(h)))))
    worst = max(range(len(rows)), key=lambda k: rows[k][1])
    per_level = {}
    for lvl, dt_, _, dh, _ in rows:
        e = per_level.setdefault(f"L{lvl}", {"max_abs_T_K": 0.0, "max_abs_H_W_m2": 0.0})
        e["max_abs_T_K"] = max(e["max_abs_T_K"], dt_)
        e["max_abs_H_W_m2"] = max(e["max_abs_H_W_m2"], dh)
    return {"planets": len(rows), "oracle": "FP64 PCG + SGS V-cycle (the reference's solve, restated), relative "
                                            "residual 1e-13, same inputs",
            "max_abs_T_K": max(r[1] for r in rows), "max_rel_T": max(r[1] / r[2] for r in rows),
            "max_abs_H_W_m2": max(r[3] for r in rows), "max_rel_H": max(r[3] / r[4] for r in rows),
            "worst_planet": {"index": worst, "level": rows[worst][0], "abs_T_K": rows[worst][1]},
            "per_level": per_level}


# ---- serving ------------------------------------------------------------------------------------

SERVE_POPULATION = {4: 16, 5: 16, 6: 16, 7: 8, 8: 4}
SERVE_RATES = (50.0, 200.0, 1000.0, 5000.0)
SOLVER_SERVE = dict(method="bicgstab", tolerance=1e-10, inner_tolerance=1e-4, poll=4)


def build_serve_population(dev):
    from planet_game_gb300 import serve

    pop = {}
    for level, n in SERVE_POPULATION.items():
        pop.update(serve.build_population(n, levels=(level,), seed=100 + level, device=dev))
    return pop


def serve_trace(args, rate: float, count: int):
    from planet_game_gb300 import workloads as W

    trace = W.poisson_trace(count, rate, seed=args.seed + 1, planets_per_level=max(SERVE_POPULATION.values()))
    return [W.Request(r.arrival_s, r.level, r.planet % SERVE_POPULATION[r.level]) for r in trace]


def requests_at(args, rate: float) -> int:
    """The serving configuration's 2,000 requests a point, fewer at the lowest rate (500 at
    50 requests/s: 10 s of offered traffic, where both arms keep up and only the latency
    differs)."""
    return min(args.serve_requests, max(500, int(10 * rate)))


def serving_sweep(args, dev, rates=SERVE_RATES) -> dict:
    """A seeded Poisson trace over L4-L8 (30/30/20/15/5 %) at each offered rate, served by
    the continuous-batching loop (mixed precision, lanes tuned at admission) and by the
    plain FP64 one-at-a-time comparator (one-planet batches tuned per level); latency from
    arrival to result on the host. Both arms see the same requests and sources."""
    import torch

    from planet_game_gb300 import serve

    out = {"population": {f"L{k}": v for k, v in SERVE_POPULATION.items()}, "budget_gb": 150,
           "latency": "arrival to result on the host (host source in, host temperature out)", "points": []}
    pop_b = build_serve_population(dev)
    pop_o = build_serve_population(dev)
    srv = serve.Server(pop_b, budget_bytes=150e9, precision="mixed", **SOLVER_SERVE)
    one = serve.OneAtATime(pop_o, tuned=True, **SOLVER_SERVE)
    try:
        # both arms tuned ahead of traffic on the same representative sources
        srv.prepare(sources=serve.typical_sources(pop_b, seed=args.seed + 5))   # admit and tune every lane
        typical_o = serve.typical_sources(pop_o, seed=args.seed + 5)
        for level, planets in pop_o.items():             # one-planet batches and per-level tunings
            for p, src in zip(planets, typical_o[level]):
                one.solo.batch_of(p.mesh, p.state, torch.from_numpy(src).to(p.state.device), p.heat_capacity, p.dt,
                                  p.conductance, p.edge_conductance)
        warm = serve_trace(args, 5000.0, 60)
        srv.run_trace(serve.make_requests(warm, pop_b, seed=args.seed + 3), realtime=False)   # record graphs
        one.run_trace(serve.make_requests(warm, pop_o, seed=args.seed + 3), realtime=False)
        for rate in rates:
            count = requests_at(args, rate)
            trace = serve_trace(args, rate, count)
            reqs_b = serve.make_requests(trace, pop_b, seed=args.seed + 2)
            srv.completed = 0
            srv.run_trace(reqs_b, realtime=True)
            reqs_o = serve.make_requests(trace, pop_o, seed=args.seed + 2)
            one.run_trace(reqs_o, realtime=True)
            torch.cuda.synchronize()
            a, b = serve.summarize(reqs_b), serve.summarize(reqs_o)
            if a["ok"] != count or b["ok"] != count:
                raise SystemExit(f"serving at {rate}/s: {count - a['ok']} + {count - b['ok']} requests failed")
            out["points"].append({"offered_per_s": rate, "requests": count, "continuous_batching_mixed": a,
                                  "one_at_a_time_fp64_tuned": b,
                                  "speedup_sub_steps_per_s": a["sub_steps_per_s"] / b["sub_steps_per_s"]})
        out["tunings"] = {f"L{k}": smoother_desc(t) for k, t in sorted(srv.tunings.items())}
    finally:
        srv.close()
    if getattr(args, "native_serve", False):
        out["continuous_batching_native"] = native_serving_point(args, dev, rates[-1], requests_at(args, rates[-1]))
    top = out["points"][-1]
    out["headline"] = {"offered_per_s": top["offered_per_s"], "requests": top["requests"],
                       "served_sub_steps_per_s": top["continuous_batching_mixed"]["sub_steps_per_s"],
                       "plain_fp64_tuned_sub_steps_per_s": top["one_at_a_time_fp64_tuned"]["sub_steps_per_s"],
                       "ratio": top["speedup_sub_steps_per_s"], "target_ratio": 5.0,
                       "p50_ms": top["continuous_batching_mixed"]["p50_ms"],
                       "p99_ms": top["continuous_batching_mixed"]["p99_ms"],
                       "plain_p50_ms": top["one_at_a_time_fp64_tuned"]["p50_ms"],
                       "plain_p99_ms": top["one_at_a_time_fp64_tuned"]["p99_ms"]}
    return out


def native_serving_point(args, dev, rate: float, count: int) -> dict:
    """The same trace through the library's own serving loop (psgb_server_*): lanes and
    their threads in C++, host arrays in and out; latency from submission to completion as
    the loop records it, after a warm-up that admits and tunes every lane."""
    from planet_game_gb300 import serve

    pop = build_serve_population(dev)
    reqs = serve.make_requests(serve_trace(args, rate, count), pop, seed=args.seed + 2)
    warm = serve.make_requests(serve_trace(args, 5000.0, 60), pop, seed=args.seed + 3)
    srv = serve.NativeServer(budget_bytes=150e9, precision="mixed", **SOLVER_SERVE)
    try:
        ids = {}
        for level, planets in pop.items():
            for i, p in enumerate(planets):
                ids[(level, i)] = srv.add_planet(level, p.radius, p.heat_capacity, p.dt, p.conductance,
                                                 p.state.cpu().numpy(), p.edge_conductance)
        typical = serve.typical_sources(pop, seed=args.seed + 5)
        for level in pop:   # admit and tune every lane, on a representative source
            pid = ids[(level, 0)]
            srv.wait(srv.submit(pid, typical[level][0]), pid)
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
    return {"requests": count, "offered_per_s": rate, "sub_steps_per_s": count / elapsed, "p50_ms": stats["p50_ms"],
            "p99_ms": stats["p99_ms"], "ok": int(sum(r.status == 0 for r in reqs)),
            "latency": "submission to completion, recorded by the loop"}


def run_serve_sweep(args, rank, local_rank):
    """The serving sweep alone, one JSON line."""
    import torch

    if rank != 0:
        return
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    sweep = serving_sweep(args, dev)
    print(json.dumps({"metric": "served sub-steps/s and p50/p99 at 1e-10 relative residual", "unit": "sub-steps/s",
                      "value": sweep["headline"]["served_sub_steps_per_s"], "n_gpus": 1, "higher_is_better": True,
                      "data": "synthetic", "serving": sweep}))


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


# ---- config 1: operators, L6 solve, column radiation ---------------------------------------------

OPS_REPS = 7


def _event_median_us(fn, flush, reps: int | None = None) -> float:
    """Median device time of fn() in microseconds, CUDA events on the current stream, the
    L2 flushed (a write of a buffer larger than L2) before every timed launch."""
    import torch

    stream = torch.cuda.current_stream()
    fn()
    times = []
    for _ in range(reps or OPS_REPS):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b) * 1e3)
    return float(statistics.median(times))


def operator_bytes(a: dict) -> dict:
    """Algorithmic FP64 bytes per cell of the operator kernels, each array counted once:
    Laplacian: columns 24, weights 48, area 8, field 8, out 8; gradient: columns 24,
    degree 1, distances 48, FP32 normals 48, the 2x2 normal matrix 32, field 8, out 16;
    divergence: edge ids 24, orientation and degree 2, area 8, out 8, and per undirected
    edge its flux and length (16 B, E/N of them per cell)."""
    n, e = len(a["area_m2"]), len(a["edge_length_m"])
    return {"laplacian": 96.0, "gradient": 177.0, "divergence": 42.0 + 16.0 * e / n}


def column_point(args, m, flush, peak, dev) -> dict:
    """Column radiation over 10 layers (1000 -> 100 hPa) for every cell of `m`: time,
    algorithmic GB/s ((7N + 7) x 8 B a column at N = 10), error against the oracle's N-layer
    restatement and the oracle's one-core time."""
    import torch

    import planet_game_gb300 as pg
    from oracle import oracle as O
    from planet_game_gb300 import workloads as W

    inp = W.step_inputs(m, args.seed)
    col = W.column_profiles(inp.t0, 10, seed=args.seed)
    k = pg.column_constants(**W.EARTH_COLUMN)
    ins = [torch.from_numpy(np.ascontiguousarray(v)).to(dev) for v in
           (col.temperature, col.humidity, col.cloud_water, col.surface_temperature, col.surface_pressure)]
    res = {}
    us = _event_median_us(lambda: res.update(o=pg.column_radiation(k, *ins)), flush)
    n = m.cell_count
    per_cell = (7 * 10 + 7) * 8.0
    gbs = per_cell * n / (us * 1e-6) / 1e9
    got = [o.cpu().numpy() for o in res["o"]]
    t = time.perf_counter()
    ref = O.column_radiation(W.column_constant_vector(), col.temperature, col.humidity, col.cloud_water,
                             col.surface_temperature, col.surface_pressure)
    cpu_s = time.perf_counter() - t
    rel = max(float(np.max(np.abs(g - r_) / np.maximum(np.abs(r_), 1e-300))) for g, r_ in zip(got, ref))
    return {"cells": n, "layers": 10, "us": us, "bytes_per_cell": per_cell, "achieved_GBs": gbs,
            "frac": gbs / peak, "max_rel_vs_oracle": rel,
            "cpu_baseline": {"seconds": cpu_s, "cores": 1, "kind": "port"}, "gpu_over_cpu": cpu_s / (us * 1e-6)}


def run_ops(args, rank, local_rank):
    """The L6 operator sweep on 8 seeded fields (sums of real spherical harmonics l <= 16):
    gradient, divergence of the exact edge-normal flux of the gradient, Laplacian; then the
    config-0 implicit solve on L6 in plain FP64; then column radiation over 10 layers for
    every L6 cell. Each kernel's time (CUDA events, L2 flushed before every launch),
    algorithmic GB/s and fraction of the measured HBM bandwidth, its error against the
    analytic fields and against the oracle, and the oracle's time on one host core. The
    operator kernels are also timed on the L8 mesh (655,362 cells), whose arrays exceed
    what a flushed L2 would hide."""
    import torch

    import planet_game_gb300 as pg
    from oracle import oracle as O
    from planet_game_gb300 import workloads as W

    if rank != 0:
        return
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    peak, peak_kind = peaks()
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)      # 256 MB > L2
    R = W.EARTH_RADIUS
    out = {"metric": "config 1 (L6 operator sweep, L6 solve, 10-layer column radiation)", "n_gpus": 1,
           "data": "synthetic", "peak_GBs": peak, "peak_kind": peak_kind,
           "timing": "median of 7 launches, CUDA events, L2 flushed before each"}

    def rel_l2(x, y, w):
        return float(np.sqrt(np.sum(w * (x - y) ** 2) / np.sum(w * y ** 2)))

    for level in args.ops_levels:
        m = pg.make_icosphere(level, R)
        a = m.arrays()
        om = O.OracleMesh(a)
        per_cell = operator_bytes(a)
        n = m.cell_count
        fields = [W.harmonic_field(a, R, 16, seed) for seed in range(8 if level == 6 else 1)]
        res = {"cells": n, "fields": len(fields), "kernels": {}}
        x_d = [torch.from_numpy(F.value).to(dev) for F in fields]
        f_d = [torch.from_numpy(F.edge_flux).to(dev) for F in fields]
        kern = {
            "laplacian": lambda k: pg.laplacian(m, x_d[k]),
            "gradient": lambda k: pg.gradient(m, x_d[k]),
            "divergence": lambda k: pg.divergence(m, f_d[k]),
        }
        for name, fn in kern.items():
            us = statistics.median(_event_median_us(lambda: fn(k), flush) for k in range(len(fields)))
            gbs = per_cell[name] * n / (us * 1e-6) / 1e9
            res["kernels"][name] = {"us": us, "bytes_per_cell": per_cell[name], "achieved_GBs": gbs,
                                    "frac": gbs / peak}
        if level == 6:
            w = a["area_m2"]
            errs = {"laplacian_vs_oracle": 0.0, "gradient_vs_oracle": 0.0, "divergence_vs_oracle": 0.0,
                    "laplacian_vs_analytic_rel_l2": 0.0, "gradient_vs_analytic_rel_l2": 0.0,
                    "divergence_vs_analytic_rel_l2": 0.0}
            cpu_s = 0.0
            for k, F in enumerate(fields):
                lap = pg.laplacian(m, x_d[k]).cpu().numpy()
                ge, gn = (t.cpu().numpy() for t in pg.gradient(m, x_d[k]))
                div = pg.divergence(m, f_d[k]).cpu().numpy()
                t = time.perf_counter()
                lo, (eo, no), do = om.laplacian(F.value), om.gradient(F.value), om.divergence(F.edge_flux)
                cpu_s += time.perf_counter() - t
                errs["laplacian_vs_oracle"] = max(errs["laplacian_vs_oracle"], float(np.max(np.abs(lap - lo)) / np.max(np.abs(lo))))
                errs["gradient_vs_oracle"] = max(errs["gradient_vs_oracle"], float(max(np.max(np.abs(ge - eo)), np.max(np.abs(gn - no))) / np.max(np.abs(eo))))
                errs["divergence_vs_oracle"] = max(errs["divergence_vs_oracle"], float(np.max(np.abs(div - do)) / np.max(np.abs(do))))
                errs["laplacian_vs_analytic_rel_l2"] = max(errs["laplacian_vs_analytic_rel_l2"], rel_l2(lap, F.laplacian, w))
                errs["gradient_vs_analytic_rel_l2"] = max(errs["gradient_vs_analytic_rel_l2"],
                                                          rel_l2(ge, F.east, w), rel_l2(gn, F.north, w))
                errs["divergence_vs_analytic_rel_l2"] = max(errs["divergence_vs_analytic_rel_l2"], rel_l2(div, F.laplacian, w))
            res["errors"] = errs
            gpu_us = sum(v["us"] for v in res["kernels"].values()) * len(fields)
            res["cpu_baseline"] = {"seconds": cpu_s, "cores": 1, "kind": "port",
                                   "sample": "the oracle's gradient, divergence and Laplacian of the 8 fields"}
            res["gpu_over_cpu"] = cpu_s / (gpu_us * 1e-6)
        out[f"operators_L{level}"] = res

        # column radiation over 10 layers for every cell of this level
        out[f"column_L{level}"] = column_point(args, m, flush, peak, dev)
    if 6 not in args.ops_levels:
        print(json.dumps(out))
        return
    # the config-0 solve on L6, plain FP64, one planet per call (tuned)
    m = pg.make_icosphere(6, R)
    inp = W.step_inputs(m, args.seed)
    t0, src = torch.from_numpy(inp.t0).to(dev), torch.from_numpy(inp.source).to(dev)
    solo = pg.TunedSolo(precision="fp64", **SOLVER)
    rep = {}
    ms = _median_ms(lambda: rep.update(r=solo.step(m, t0, src, inp.heat_capacity, inp.dt, inp.conductance)))
    t_new = rep["r"][0].cpu().numpy()
    om = O.OracleMesh(m.arrays())
    tight = O.OracleHierarchy(om).transport_step(inp.conductance, inp.heat_capacity, inp.dt, inp.t0, inp.source,
                                                 tol=1e-13)
    t = time.perf_counter()
    base = O.OracleHierarchy(om).transport_step(inp.conductance, inp.heat_capacity, inp.dt, inp.t0, inp.source,
                                                tol=1e-10)
    cpu_s = time.perf_counter() - t
    r = rep["r"][1]
    out["solve_L6"] = {"ms": ms, "iterations": r.iterations, "relative_residual": r.relative_residual,
                       "closure": r.closure, "max_abs_T_vs_oracle_K": float(np.max(np.abs(t_new - tight["t_new"]))),
                       "cpu_baseline": {"seconds": cpu_s, "cores": 1, "kind": "port", "pcg_iterations": base["iterations"]},
                       "gpu_over_cpu": cpu_s / (ms * 1e-3)}

    print(json.dumps(out))


# ---- config 2: one L8 planet, 32 right-hand sides --------------------------------------------------

def run_l8rhs(args, rank, local_rank):
    """One L8 planet (655,362 cells), 32 sub-steps with sources S_j = S + N(0, 5^2) W/m^2,
    solved as one block (psgb_transport_step_multi: every sweep reads the matrix once for
    all 32) in plain FP64 (variant A) and FP32 inner + FP64 refinement (variant B), beside
    the same 32 sub-steps one per call through the plain FP64 drop-in; each sub-step's error
    against the FP64 CPU oracle (PCG + SGS V-cycle to 1e-13, all host cores), refinement
    counts and inner iterations, the block's fine-level sweep bytes per second."""
    import ctypes as C

    import torch

    import planet_game_gb300 as pg
    from oracle import oracle as O
    from planet_game_gb300 import capi
    from planet_game_gb300 import workloads as W

    if rank != 0:
        return
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    rhs = 32
    m = pg.make_icosphere(8, W.EARTH_RADIUS)
    inp = W.step_inputs(m, args.seed)
    sources = W.perturbed_sources(inp.source, rhs, seed=args.seed + 1)
    t0 = torch.from_numpy(inp.t0).to(dev)
    src = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in sources]
    lib = capi.load()
    peak, peak_kind = peaks()
    # per precision, the planet's settings autotuned on a one-planet batch (setup, not
    # timed): the block step and the one-at-a-time comparator use the same tuning
    tunings = {}
    if not args.no_autotune:
        tb = pg.Batch([m])
        for precision in ("fp64", "mixed"):
            if precision == "fp64" or precision in args.l8rhs_variants:
                tunings[precision] = tb.autotune([t0], [src[0]], [inp.heat_capacity], [inp.dt],
                                                 conductance=[inp.conductance], precision=precision, **SOLVER)
        del tb
    out = {"metric": "sub-steps/s of 32 sub-steps of one L8 planet at 1e-10 relative residual", "unit": "sub-steps/s",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "data": "synthetic", "higher_is_better": True,
           "config": {"workload": "one L8 planet (655,362 cells), 32 right-hand sides S + N(0, 5^2) W/m^2",
                      "cells": m.cell_count, "rhs": rhs, "tolerance": 1e-10, "krylov": "BiCGSTAB",
                      "smoother": {p: smoother_desc(t) for p, t in tunings.items()} or smoother_desc(None),
                      "tuning": tunings or None}}
    results = {}
    for name, precision in (("A_fp64", "fp64"), ("B_mixed", "mixed")):
        if precision not in args.l8rhs_variants:
            continue
        m.set_tuning(tunings.get(precision))
        step = lambda: pg.transport_step_multi(m, t0, src, inp.heat_capacity, inp.dt, inp.conductance,
                                               precision=precision, **SOLVER)
        for _ in range(args.warmup):
            t_new, _, reps = step()
        stream = torch.cuda.current_stream()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(args.steps):
            t_new, _, reps = step()
        b.record(stream)
        torch.cuda.synchronize()
        sec = a.elapsed_time(b) / 1e3
        ms, nl, nbytes = C.c_double(), C.c_uint64(), C.c_uint64()
        capi.check(lib.psgb_profile_begin(b"smooth"))
        step()
        capi.check(lib.psgb_profile_end(C.byref(ms), C.byref(nl), C.byref(nbytes)))
        achieved = nbytes.value / (ms.value / 1e3) / 1e9 if ms.value > 0 else None
        results[name] = [x.cpu().numpy() for x in t_new]
        out[name] = {"value": rhs * args.steps / sec, "ms_per_block": sec * 1e3 / args.steps,
                     "refinements": sorted({r.refinements for r in reps}),
                     "inner_iterations": {"min": min(r.iterations for r in reps), "max": max(r.iterations for r in reps)},
                     "max_relative_residual": max(r.relative_residual for r in reps),
                     "max_closure": max(r.closure for r in reps), "status_ok": all(r.status == 0 for r in reps),
                     "roofline_fine_sweeps": {"bound": "hbm", "achieved": achieved, "peak": peak, "peak_kind": peak_kind,
                                              "unit": "GB/s", "frac": achieved / peak if achieved else None,
                                              "launches": int(nl.value), "bytes_per_launch": nbytes.value / max(1, nl.value),
                                              "bytes": "matrix and indices once per row, the 32 right-hand sides' vectors"}}
    # the same 32 sub-steps one per call through the plain FP64 drop-in, with the FP64 tuning
    # (the comparator) and with the options' untuned sweeps
    for key, tuning in (("one_at_a_time_fp64", tunings.get("fp64")), ("one_at_a_time_fp64_untuned", None)):
        if key == "one_at_a_time_fp64_untuned" and tuning is None and not tunings:
            continue
        m.set_tuning(tuning)
        for _ in range(2):
            pg.transport_step(m, t0, src[0], inp.heat_capacity, inp.dt, inp.conductance, precision="fp64", **SOLVER)
        torch.cuda.synchronize()
        t = time.perf_counter()
        for j in range(rhs):
            pg.transport_step(m, t0, src[j], inp.heat_capacity, inp.dt, inp.conductance, precision="fp64", **SOLVER)
        torch.cuda.synchronize()
        out[key] = {"value": rhs / (time.perf_counter() - t), "unit": "sub-steps/s",
                    "settings": "autotuned (the block's FP64 tuning)" if tuning is not None else "untuned"}
    m.set_tuning(None)
    for name in ("A_fp64", "B_mixed"):
        if name in out:
            out["value"] = out[name]["value"]
            out[f"speedup_block_{name.split('_')[1]}_vs_one_at_a_time"] = (out[name]["value"] /
                                                                         out["one_at_a_time_fp64"]["value"])
    if not args.skip_cpu:
        t = time.perf_counter()
        refs = O.transport_steps(m.arrays(), inp.conductance, inp.heat_capacity, inp.dt, [inp.t0] * rhs,
                                 [np.ascontiguousarray(x) for x in sources], tol=1e-13)
        cpu_s = time.perf_counter() - t
        for name in results:
            errs = [float(np.max(np.abs(results[name][j] - refs[j][0]))) for j in range(rhs)]
            out[name]["oracle_error"] = {"max_abs_T_K": max(errs), "per_rhs_max_abs_T_K": errs}
        out["cpu_baseline"] = {"value": rhs / cpu_s, "unit": "sub-steps/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": "the 32 sub-steps by the oracle (FP64 PCG + SGS V-cycle) to 1e-13, one "
                                         "process per core", "pcg_iterations": [r[2] for r in refs]}
    print(json.dumps(out))


# ---- CPU baseline and the reference arm ------------------------------------------------------

def inp_dict(inp) -> dict:
    return {"conductance": inp.conductance, "heat_capacity": inp.heat_capacity, "dt": inp.dt, "t0": inp.t0,
            "source": inp.source}


def _oracle_run(payload):
    arrays, inp, edge_g, tol = payload
    from oracle import oracle as O

    om = O.OracleMesh(arrays)
    h = O.OracleHierarchy(om)
    t = time.perf_counter()
    out = h.transport_step(inp["conductance"], inp["heat_capacity"], inp["dt"], inp["t0"], inp["source"], tol=tol,
                           edge_g=None if edge_g is None else om.directed_conductance(edge_g))
    return time.perf_counter() - t, out


def _oracle_solve(payload):
    """One planet's sub-step by the oracle's port of the reference (FP64 PCG + SGS V-cycle):
    its time and PCG iterations."""
    dt, out = _oracle_run(payload)
    return dt, out["iterations"]


def _oracle_solve_full(payload):
    """The same, returning the new temperature and the transport H."""
    _, out = _oracle_run(payload)
    return out["t_new"], out["transport"]


def cpu_baseline(planets, args):
    """A bounded sample on one host core: every planet of the mix once (about 10-30 s)."""
    total, iters = 0.0, 0
    for m, inp in planets:
        dt, it = _oracle_solve((m.arrays(), inp_dict(inp), inp.edge_conductance, 1e-10))
        total += dt
        iters += it
    return {"value": len(planets) / total, "unit": "sub-steps/s", "cores": 1, "kind": "port",
            "sample": f"all {len(planets)} planets of the workload once, one core, FP64 PCG + SGS V-cycle to 1e-10 "
                      "(the oracle's restatement of the reference's solve: bit-identical solutions, within 1% of the "
                      "reference's own speed where both compile)",
            "pcg_iterations": iters}


def run_reference(args, rank, world):
    """The reference's algorithm (the oracle's port) on all host cores, one process per core,
    every planet of the workload per step. Inputs are built by the oracle itself (its
    restatement of the mesh builder and insolation): this arm loads no product library."""
    if rank != 0:
        return
    import multiprocessing as mp

    if args.workload not in WORKLOAD_NAMES:
        print(json.dumps({"impl": "reference", "unavailable": f"no CPU reference arm for workload {args.workload}"}))
        return
    planets = oracle_workload(args.workload, args.seed)
    payloads = [(a, inp_dict(inp), inp.edge_conductance, 1e-10) for a, inp in planets]
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
    cells = sum(len(a["area_m2"]) for a, _ in planets)
    config = static_config(args.workload, len(planets), cells)
    config["pcg_iterations"] = sum(r[1] for r in results)
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
        "config": config,
        "cpu_baseline": {"value": value, "unit": "sub-steps/s", "cores": cores, "kind": "port",
                         "sample": "every planet of the workload per step, one process per core (the oracle's "
                                   "restatement of the reference's FP64 PCG + SGS solve: bit-identical solutions, "
                                   "within 1% of the reference's own speed where both compile); planets built by "
                                   "the oracle's restatement of the reference's mesh builder"},
        "e2e": {"value": value, "unit": "sub-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=["batch", "l8", "l8rhs", "ops", "serve", "next"], default="batch")
    ap.add_argument("--serve-requests", type=int, default=2000, help="requests per offered rate (fewer at 50/s)")
    ap.add_argument("--ops-levels", type=int, nargs="+", default=[6, 8],
                    help="ops workload: mesh levels of the operator and column timings (the L6 solve runs with 6)")
    ap.add_argument("--ops-reps", type=int, default=7, help="ops workload: timed launches per kernel (median)")
    ap.add_argument("--l8rhs-variants", nargs="+", choices=["fp64", "mixed"], default=["fp64", "mixed"],
                    help="l8rhs workload: the block solve's precisions (A: fp64, B: mixed)")
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
    if args.workload == "ops":
        global OPS_REPS
        OPS_REPS = args.ops_reps
        run_ops(args, rank, local_rank)
        return
    if args.workload == "l8rhs":
        run_l8rhs(args, rank, local_rank)
        return
    run_gb300(args, rank, world, local_rank)


if __name__ == "__main__":
    main()

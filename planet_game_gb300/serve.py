"""Continuous-batching request loop for implicit heat-transport sub-steps.

Requests ask for one sub-step of one planet: the planet's temperature advances from its
resident state by the implicit step with the request's source term. The server keeps a
population of planets of mesh levels L4-L8; every planet's mesh, multigrid hierarchy,
matrix values and state stay resident in HBM.

Lanes: one per mesh level, each a resident batch of that level's planets with its own
CUDA stream and host thread. A lane works in rounds: it takes, for every planet with
pending requests, the oldest one, and solves them together (the other planets of the
batch are masked out); requests that arrive while a round runs are admitted at the next
round of their lane, while the other lanes keep the device busy - their work overlaps on
the GPU. Lanes are admitted by an HBM budget: a lane is built when its first request
arrives if its bytes fit; otherwise the least recently used idle lane is evicted first,
or the request waits until memory frees up.

The comparator (`OneAtATime`) serves the same trace with the plain drop-in: one request
at a time, each planet solved alone in plain FP64.

`NativeServer` is the library's own loop (psgb_server_*): the same policy with the lanes and
their worker threads in C++, host arrays in and out.
"""
from __future__ import annotations

import collections
import threading
import time
from dataclasses import dataclass

import numpy as np

from . import api, capi
from . import workloads as W


@dataclass
class PlanetState:
    level: int
    radius: float
    mesh: api.PlanetMesh
    state: object                       # device tensor: the resident temperature (K)
    edge_conductance: np.ndarray | None
    heat_capacity: float
    dt: float
    conductance: float


@dataclass
class ServedRequest:
    arrival_s: float                    # offered arrival time (relative to the trace start)
    level: int
    planet: int                         # index within its level's population
    source: np.ndarray                  # W/m^2, host
    done_s: float = -1.0
    result: np.ndarray | None = None    # the new temperature (host)
    status: int = -1
    iterations: int = 0
    t_in: np.ndarray | None = None      # the state the step started from (for checks)


def build_population(per_level: int, levels=(4, 5, 6, 7, 8), seed: int = 7, device=None):
    """Planets of each level with seeded radii, per-edge diffusivities and initial states."""
    import torch

    rng = np.random.default_rng(seed)
    population: dict[int, list[PlanetState]] = {}
    for level in levels:
        planets = []
        for k in range(per_level):
            radius = float(rng.uniform(3e6, 9e6))
            pseed = int(rng.integers(0, 2**31))
            m = api.make_icosphere(level, radius)
            kappa = W.lognormal_edge_diffusivity(m.edge_count, pseed)
            inp = W.step_inputs(m, pseed, edge_diffusivity=kappa)
            planets.append(PlanetState(level, radius, m, torch.from_numpy(inp.t0).to(device), inp.edge_conductance,
                                       inp.heat_capacity, inp.dt, inp.conductance))
        population[level] = planets
    return population


def request_source(p: PlanetState, rng) -> np.ndarray:
    """A request's source term for planet `p` (W/m^2): absorbed sub-step-mean insolation
    less a linearised outgoing flux of a latitude-dependent temperature, plus noise."""
    if not hasattr(p, "_q"):
        p._lat = W.latitude(p.mesh.arrays()["center"])
        p._q = p.mesh.substep_mean_insolation(0).astype(np.float64)
    base_t = 288.0 - 40.0 * np.sin(p._lat) ** 2
    return 0.7 * p._q - (203.3 + 2.09 * (base_t - 273.15)) + rng.normal(0.0, 5.0, len(p._lat))


def make_requests(trace, population, seed: int = 11):
    """Requests of a trace: each carries a source term for its planet (seeded)."""
    rng = np.random.default_rng(seed)
    out = []
    for r in trace:
        k = r.planet % len(population[r.level])
        out.append(ServedRequest(r.arrival_s, r.level, k, request_source(population[r.level][k], rng)))
    return out


def typical_sources(population, seed: int = 13) -> dict:
    """One source per planet, drawn as requests draw theirs: what lanes (and the
    comparator's one-planet batches) are tuned on ahead of traffic."""
    rng = np.random.default_rng(seed)
    return {level: [request_source(p, rng) for p in planets] for level, planets in sorted(population.items())}


class _Lane:
    def __init__(self, server, level):
        import torch

        self.server = server
        self.level = level
        self.planets = server.population[level]
        self.batch = None
        self.edge_conductance = None        # "stored" once the lane's batch holds the planets' arrays
        self.bytes = 0
        self.pending: dict[int, collections.deque] = collections.defaultdict(collections.deque)
        self.cv = threading.Condition(server.lock)
        self.stream = torch.cuda.Stream()
        self.last_used = 0.0
        self.busy = False
        self.thread = threading.Thread(target=self._run, daemon=True)
        self.rounds = 0
        self._staging = None                # per planet: pinned source, device source, pinned result

    def _stage(self):
        """Page-locked host buffers and device buffers for every planet of the lane (made
        once): sources go up and results come down asynchronously on the lane's stream, with
        one synchronisation a round instead of two blocking copies a planet."""
        import torch

        if self._staging is None:
            self._staging = []
            for p in self.planets:
                n = p.mesh.cell_count
                self._staging.append((torch.empty(n, dtype=torch.float64, pin_memory=True),
                                      torch.empty(n, dtype=torch.float64, device=self.server.device),
                                      torch.empty(n, dtype=torch.float64, pin_memory=True)))
        return self._staging

    def _round(self, reqs: dict[int, ServedRequest]):
        import torch

        n = len(self.planets)
        active = [i in reqs for i in range(n)]
        staging = self._stage()
        with torch.cuda.stream(self.stream):
            t0 = [p.state if active[i] else None for i, p in enumerate(self.planets)]
            src = [None] * n
            for i in reqs:
                host, dev, _ = staging[i]
                np.copyto(host.numpy(), reqs[i].source)
                dev.copy_(host, non_blocking=True)
                src[i] = dev
            outs, reps = self.batch.transport_step(
                t0, src, [p.heat_capacity for p in self.planets], [p.dt for p in self.planets],
                conductance=[p.conductance for p in self.planets],
                edge_conductance=self.edge_conductance, active=active, **self.server.options)
            for i in reqs:
                if self.server.keep_inputs:
                    reqs[i].t_in = self.planets[i].state.cpu().numpy()
                staging[i][2].copy_(outs[i], non_blocking=True)
            self.stream.synchronize()
            for i, r in reqs.items():
                self.planets[i].state = outs[i]
                r.result = staging[i][2].numpy().copy()
                r.status = reps[i].status
                r.iterations = reps[i].iterations
        done = time.perf_counter() - self.server.t_start
        for r in reqs.values():
            r.done_s = done

    def _run(self):
        srv = self.server
        while True:
            with self.cv:
                while not srv.stopping and not any(self.pending.values()):
                    self.cv.wait()
                if srv.stopping and not any(self.pending.values()):
                    return
                reqs = {i: q.popleft() for i, q in self.pending.items() if q}
                self.busy = True
            try:
                self._round(reqs)
                self.rounds += 1
            except Exception as exc:  # report, then let the server surface it
                srv.errors.append(exc)
                for r in reqs.values():
                    r.done_s = time.perf_counter() - srv.t_start
                    r.status = -2
            with self.cv:
                self.busy = False
                self.last_used = time.perf_counter()
                srv.completed += len(reqs)
                srv.done_cv.notify_all()


class Server:
    """The continuous-batching request loop (see the module docstring)."""

    def __init__(self, population, budget_bytes: float = 150e9, precision: str = "mixed", method: str = "bicgstab",
                 device=None, keep_inputs: bool = False, autotune: bool = True, **solver):
        import torch

        self.population = population
        self.device = device or torch.device("cuda", 0)
        self.budget = float(budget_bytes)
        self.options = dict(precision=precision, method=method, **solver)
        self.lock = threading.Lock()
        self.done_cv = threading.Condition(self.lock)
        self.lanes: dict[int, _Lane] = {}
        self.resident_bytes = 0
        self.stopping = False
        self.completed = 0
        self.errors: list[Exception] = []
        self.keep_inputs = keep_inputs
        self.evictions = 0
        self.autotune = autotune
        self.tunings: dict[int, dict] = {}     # per level, from the lane's first admission
        self.t_start = time.perf_counter()

    # -- admission ------------------------------------------------------------------------
    def _lane_bytes(self, level) -> int:
        # resident: the batch's workspace plus every planet's state
        cells = sum(p.mesh.cell_count for p in self.population[level])
        return int(cells * 700)   # measured layout cost per cell of a mixed-precision batch, with margin

    def _admit(self, level, sources=None) -> _Lane | None:
        """Lane of `level`, built if the budget allows (evicting idle lanes); None: wait.
        `sources` ({planet index: host source}): the work the lane is admitted for, which a
        lane tuned at admission is tuned on (zero sources elsewhere)."""
        lane = self.lanes.get(level)
        if lane is not None and lane.batch is not None:
            return lane
        need = self._lane_bytes(level)
        while self.resident_bytes + need > self.budget:
            idle = [l for l in self.lanes.values() if l.batch is not None and not l.busy and not any(l.pending.values())]
            if not idle:
                return None
            victim = min(idle, key=lambda l: l.last_used)
            victim.batch = None
            self.resident_bytes -= victim.bytes
            victim.bytes = 0
            self.evictions += 1
        if lane is None:
            lane = _Lane(self, level)
            self.lanes[level] = lane
            lane.thread.start()
        lane.batch = api.Batch([p.mesh for p in self.population[level]])
        edges = [p.edge_conductance for p in self.population[level]]
        lane.edge_conductance = None
        if any(e is not None for e in edges):
            lane.batch.set_edge_conductance(edges)
            lane.edge_conductance = "stored"
        if self.autotune:
            if level not in self.tunings:
                self.tunings[level] = self._tune(lane.batch, level, sources)
            else:
                lane.batch.set_tuning(self.tunings[level])
        lane.bytes = need
        self.resident_bytes += need
        return lane

    def _tune(self, batch, level, sources=None) -> dict:
        """Per-level settings for a lane, from trial solves of a step of its planets with
        `sources` ({planet index: host source}; zero for the others: they converge at once
        and do not set the pace)."""
        import torch

        planets = self.population[level]
        sources = sources or {}
        src = [torch.from_numpy(np.ascontiguousarray(sources[i], np.float64)).to(p.state.device) if i in sources
               else torch.zeros_like(p.state) for i, p in enumerate(planets)]
        return batch.autotune([p.state for p in planets], src, [p.heat_capacity for p in planets],
                              [p.dt for p in planets], conductance=[p.conductance for p in planets],
                              edge_conductance=self.lanes[level].edge_conductance, **self.options)

    def prepare(self, levels=None, sources=None):
        """Admit (and tune) the lanes of `levels` ahead of traffic, as far as the budget
        allows; `sources` ({level: [host source per planet]}, e.g. typical_sources) is what
        they are tuned on."""
        with self.lock:
            for level in (levels if levels is not None else sorted(self.population)):
                per = dict(enumerate(sources[level])) if sources is not None and level in sources else None
                if self._admit(level, per) is None:
                    break

    def submit(self, req: ServedRequest) -> bool:
        """Queue a request; False if its lane cannot be admitted yet (memory)."""
        with self.lock:
            lane = self._admit(req.level, {req.planet: req.source})
            if lane is None:
                return False
            lane.pending[req.planet].append(req)
            lane.cv.notify()
            return True

    def run_trace(self, requests: list[ServedRequest], realtime: bool = True):
        """Replay arrivals (at their offered times when `realtime`), wait for completion of
        every request of this trace (the server's completion count is cumulative: only the
        completions after this call's start count)."""
        with self.done_cv:
            base = self.completed
        self.t_start = time.perf_counter()
        waiting = collections.deque()
        for r in requests:
            if realtime:
                delay = r.arrival_s - (time.perf_counter() - self.t_start)
                if delay > 0:
                    time.sleep(delay)
            waiting.append(r)
            while waiting and self.submit(waiting[0]):
                waiting.popleft()
        while waiting:
            time.sleep(0.001)
            while waiting and self.submit(waiting[0]):
                waiting.popleft()
        with self.done_cv:
            while self.completed - base < len(requests) and not self.errors:
                self.done_cv.wait(timeout=1.0)
        if self.errors:
            raise self.errors[0]

    def close(self):
        with self.lock:
            self.stopping = True
            for lane in self.lanes.values():
                lane.cv.notify_all()
        for lane in self.lanes.values():
            lane.thread.join(timeout=30)


class NativeServer:
    """The library's serving loop (psgb_server_*): register planets, submit sub-steps,
    wait for their new temperatures. Lanes per mesh level, resident under `budget_bytes`
    of device memory; `solver` as for `api.solve_options`."""

    def __init__(self, budget_bytes: float = 150e9, precision: str = "mixed", method: str = "bicgstab",
                 autotune: bool = True, device: int = 0, bytes_per_cell: float = 700.0, yield_after_s: float = 0.25,
                 **solver):
        import ctypes as C

        self._C = C
        self._lib = capi.load()
        cfg = capi.ServerConfig()
        cfg.budget_bytes, cfg.bytes_per_cell = float(budget_bytes), float(bytes_per_cell)
        cfg.options = api.solve_options(precision=precision, method=method, **solver)
        cfg.autotune, cfg.device, cfg.yield_after_s = int(bool(autotune)), int(device), float(yield_after_s)
        handle = C.c_void_p()
        capi.check(self._lib.psgb_server_create(C.byref(cfg), C.byref(handle)))
        self._h = handle
        self._cells: dict[int, int] = {}

    def add_planet(self, level: int, radius_m: float, heat_capacity: float, dt: float, conductance: float, t0_K,
                   edge_conductance=None) -> int:
        """Registers a planet (before its level's first request); returns its id."""
        C = self._C
        t0 = np.ascontiguousarray(t0_K, dtype=np.float64)
        edges = None if edge_conductance is None else np.ascontiguousarray(edge_conductance, dtype=np.float64)
        cells = 10 * 4 ** int(level) + 2   # the icosphere's cells at this level
        if t0.size != cells:
            raise ValueError("the initial temperature does not match the level's cells")
        params = capi.StepParams(heat_capacity, dt, conductance, None if edges is None else edges.ctypes.data, 0)
        pid = C.c_uint32()
        capi.check(self._lib.psgb_server_add_planet(self._h, level, radius_m, C.byref(params),
                                                    t0.ctypes.data_as(C.c_void_p), C.byref(pid)))
        self._cells[pid.value] = cells
        return pid.value

    def submit(self, planet: int, source_W_m2) -> int:
        C = self._C
        src = np.ascontiguousarray(source_W_m2, dtype=np.float64)
        if src.size != self._cells.get(planet, -1):
            raise ValueError("unknown planet or a source of the wrong size")
        rid = C.c_uint64()
        capi.check(self._lib.psgb_server_submit(self._h, planet, src.ctypes.data_as(C.c_void_p), C.byref(rid)))
        return rid.value

    def wait(self, request: int, planet: int, timeout_s: float = -1.0):
        """(new temperature, report) of a request of `planet`; raises GB300Error on failure."""
        C = self._C
        out = np.empty(self._cells[planet])
        rep = capi.StepReport()
        capi.check(self._lib.psgb_server_wait(self._h, request, timeout_s, out.ctypes.data_as(C.c_void_p),
                                              C.byref(rep)))
        return out, rep

    def state(self, planet: int) -> np.ndarray:
        out = np.empty(self._cells[planet])
        capi.check(self._lib.psgb_server_state(self._h, planet, out.ctypes.data_as(self._C.c_void_p)))
        return out

    def stats(self) -> dict:
        st = capi.ServerStats()
        capi.check(self._lib.psgb_server_stats_get(self._h, self._C.byref(st)))
        return {name: getattr(st, name) for name, _ in capi.ServerStats._fields_}

    def reset_stats(self) -> None:
        """Forget the counts and latencies so far; call it while no request is in flight."""
        capi.check(self._lib.psgb_server_stats_reset(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            self._lib.psgb_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()


class OneAtATime:
    """The comparator: requests in arrival order, one at a time, plain FP64, each planet
    solved alone. `tuned` (default): each planet in a one-planet batch with the launch
    shapes and sweeps autotuned once per mesh level (api.TunedSolo), as the batched lanes
    are tuned; otherwise the single-planet entry point with the untuned defaults."""

    def __init__(self, population, device=None, tuned: bool = True, **solver):
        import torch

        self.population = population
        self.device = device or torch.device("cuda", 0)
        self.options = {"method": "bicgstab", **solver, "precision": "fp64"}
        self.solo = api.TunedSolo(**self.options) if tuned else None

    def run_trace(self, requests: list[ServedRequest], realtime: bool = True):
        import torch

        t_start = time.perf_counter()
        for r in requests:
            if realtime:
                delay = r.arrival_s - (time.perf_counter() - t_start)
                if delay > 0:
                    time.sleep(delay)
            p = self.population[r.level][r.planet]
            src = torch.from_numpy(r.source).to(self.device)
            if self.solo is not None:
                out, rep = self.solo.step(p.mesh, p.state, src, p.heat_capacity, p.dt, p.conductance,
                                          edge_conductance=p.edge_conductance)
            else:
                out, _, rep = api.transport_step(p.mesh, p.state, src, p.heat_capacity, p.dt, p.conductance,
                                                 edge_conductance=p.edge_conductance, **self.options)
            p.state = out
            r.result = out.cpu().numpy()
            r.status = rep.status
            r.iterations = rep.iterations
            r.done_s = time.perf_counter() - t_start


def summarize(requests: list[ServedRequest]) -> dict:
    lat = np.array([r.done_s - r.arrival_s for r in requests])
    span = max(r.done_s for r in requests) - min(r.arrival_s for r in requests)
    return {"requests": len(requests), "sub_steps_per_s": len(requests) / span if span > 0 else None,
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "ok": int(sum(r.status == 0 for r in requests))}

"""Serving many independent hydro simulations on one GPU, with continuous batching.

A request asks for one 3D hydro job: a box of n^3 real cells (4 ghost layers, periodic, side 1)
with a Sedov-like blast (energy 1 within 3 cells of a random centre, ambient rho = 1,
p = 1e-5) or a Sod tube (rho, p = 1, 1 | 0.125, 0.1) along a random direction, advanced for a
fixed number of steps at CFL 0.3.  Requests arrive over time (a seeded Poisson stream).

`BatchedServer` keeps one cgb_batch: requests that have arrived are admitted whenever the
device memory budget and the job table have room, their state stays resident, and every
iteration advances the running jobs by one batch step; a job that has done its steps leaves
the batch and the next arrival takes its place (continuous batching).  Which admitted jobs run
is the scheduler's choice: "fcfs" (default) runs them in arrival order until the step holds
`saturation_cells` cells, enough to fill the GPU, and holds the rest (first come, first served
keeps the longest wait, and so the tail latency, lowest; the cap keeps the GPU full); "all"
steps every admitted job (processor sharing).  The batch's schedule (chains, solo threshold)
is picked by the autotuner (`tune.py`) on the workload's size mix when the server starts.

`PerRequestServer` is the baseline: the same admission, but every job is advanced by its own
launches of the single-box step (one box engine per job, each on its own stream), either
kernel by kernel every step ("per_request") or replayed from a CUDA graph of its own
("per_request_graph").

Latency of a request = time from its arrival to the completion on the GPU of its last step
(observed from the host by polling that step's event).  Throughput = cell updates of all
requests / (last completion - first arrival).
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from .batch import Batch, ic_blast, ic_shock_tube
from .engine import Box
from .integrator import Scheme

SIZES = (32, 48, 64, 96, 128)
N_GHOST = 4


@dataclass
class Request:
    rid: int
    arrival: float  # seconds after the start of the run
    n: int          # real cells per side
    kind: str       # "blast" or "tube"
    seed: int
    steps: int = 100
    # filled by the server
    admitted: float = math.nan
    done: float = math.nan

    @property
    def cells(self) -> int:
        return self.n ** 3

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def make_requests(rate: float, count: int, seed: int = 0, steps: int = 100, sizes=SIZES) -> list[Request]:
    """A seeded Poisson arrival stream: exponential gaps of mean 1/rate, sizes uniform over
    `sizes`, blast or tube with equal odds."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=count)
    t = np.cumsum(gaps) - gaps[0]
    out = []
    for i in range(count):
        out.append(Request(i, float(t[i]), int(rng.choice(sizes)), "blast" if rng.random() < 0.5 else "tube",
                           int(rng.integers(1 << 30)), steps))
    return out


def default_scheme() -> Scheme:
    """PPMC + HLLC + VL, dual energy, density and temperature floors, mixed precision."""
    return Scheme(reconstruction="PPMC", riemann_solver="HLLC", dual_energy=True, density_floor=True,
                  temperature_floor=True, gamma=5.0 / 3.0, precision="mixed")


def init_state(torch, req: Request, scheme: Scheme, stream):
    """Allocate the request's state on the device and write its initial condition (on `stream`)."""
    n, ng = req.n, N_GHOST
    N = n + 2 * ng
    nf = scheme.n_fields
    with torch.cuda.stream(stream):
        U = torch.empty((nf, N, N, N), dtype=torch.float64, device="cuda")
    dx = 1.0 / n
    rng = np.random.default_rng(req.seed)
    centre = tuple(float(c) for c in rng.uniform(0.25, 0.75, size=3))
    if req.kind == "blast":
        ic_blast(U, ng, dx, centre, radius=3.0 * dx, energy=1.0, rho=1.0, p=1e-5, gamma=scheme.gamma,
                 dual_energy=scheme.dual_energy, stream=stream)
    else:
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        ic_shock_tube(U, ng, dx, centre, tuple(float(c) for c in v), gamma=scheme.gamma,
                      dual_energy=scheme.dual_energy, stream=stream)
    return U, dx


def state_bytes(req: Request, scheme: Scheme) -> int:
    N = req.n + 2 * N_GHOST
    return scheme.n_fields * N ** 3 * 8


@dataclass
class Report:
    mode: str
    requests: list
    wall: float
    steps_launched: int = 0
    extra: dict = field(default_factory=dict)

    def summary(self) -> dict:
        lat = np.array([r.latency for r in self.requests])
        first = min(r.arrival for r in self.requests)
        last = max(r.done for r in self.requests)
        cells = sum(r.cells * r.steps for r in self.requests)
        return {"mode": self.mode, "requests": len(self.requests), "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
                "cell_updates_per_s": cells / (last - first), "makespan_s": last - first, **self.extra}


class _Base:
    """Shared admission: arrived requests in arrival order, while the memory budget allows."""

    def __init__(self, torch, scheme: Scheme | None = None, mem_budget: int | None = None, max_active: int = 256,
                 depth: int = 2):
        self.torch = torch
        self.scheme = scheme or default_scheme()
        if mem_budget is None:  # admission by free device memory, with a fifth kept in reserve
            free, _ = torch.cuda.mem_get_info()
            mem_budget = int(free * 0.8)
        self.budget = mem_budget
        self.max_active = max_active
        self.depth = depth

    def _cost(self, req: Request) -> int:
        raise NotImplementedError

    def _event(self):
        """An event recorded after the step just queued (completes when that step has run)."""
        ev = self.torch.cuda.Event()
        ev.record(self._event_stream())
        return ev

    def run(self, requests: list[Request]) -> Report:
        queue = deque(sorted(requests, key=lambda r: r.arrival))
        used = 0
        active = {}      # key -> [req, steps_left, state, cost]
        inflight = deque()  # (event, [finished (req, cost, state)])
        done = []
        t0 = time.perf_counter()
        launched = 0
        while queue or active or inflight:
            now = time.perf_counter() - t0
            # admission
            while queue and queue[0].arrival <= now and len(active) < self.max_active:
                cost = self._cost(queue[0])
                if used + cost > self.budget and active:
                    break
                req = queue.popleft()
                req.admitted = now
                key, state = self._admit(req)
                active[key] = [req, req.steps, state, cost]
                used += cost
            if active:
                finished = self._step(active)
                launched += 1
                ev = self._event()
                fin = []
                for key in finished:
                    req, _, state, cost = active.pop(key)
                    self._retire(key)
                    fin.append((req, cost, state))
                inflight.append((ev, fin))
            # completions, oldest first; never more than `depth` steps queued ahead of the GPU
            while inflight and (inflight[0][0].query() or len(inflight) > self.depth or not active):
                ev, fin = inflight.popleft()
                ev.synchronize()
                t = time.perf_counter() - t0
                for req, cost, state in fin:
                    req.done = t
                    used -= cost
                    done.append(req)
            if not active and not inflight and queue:
                wait = queue[0].arrival - (time.perf_counter() - t0)
                if wait > 0:
                    time.sleep(min(wait, 0.01))
        wall = time.perf_counter() - t0
        return Report(self.mode, done, wall, launched, dict(getattr(self, "extra", {})))


class BatchedServer(_Base):
    mode = "batched"

    def __init__(self, torch, chains: int | None = None, policy: str = "fcfs", saturation_cells: int = 3 << 20,
                 autotune: bool = True, **kw):
        super().__init__(torch, **kw)
        if policy not in ("fcfs", "all"):
            raise ValueError("policy must be 'fcfs' or 'all'")
        self.stream = torch.cuda.Stream()
        self.batch = Batch(self.scheme, self.stream, c_cfl=0.3)
        self.extra = {}
        if autotune and chains is None:  # schedule picked by measurement on the workload's size mix
            from .tune import tune_batch

            t = tune_batch(torch, self.scheme, [n for n in SIZES for _ in range(2)])
            self.batch.set_chains(t["chains"])
            self.batch.set_solo_cells(t["solo_cells"])
            self.batch.set_tiles(t.get("tiles", 0))
            self.extra["tuned"] = {"chains": t["chains"], "solo_cells": t["solo_cells"], "tiles": t.get("tiles", 0)}
        else:
            self.batch.set_chains(chains or 2)
        self.policy = policy
        self.saturation_cells = saturation_cells
        self.held = set()

    def _cost(self, req):
        N = req.n + 2 * N_GHOST
        return state_bytes(req, self.scheme) + self.batch.job_bytes(N, N, N)

    def _admit(self, req):
        U, dx = init_state(self.torch, req, self.scheme, self.stream)
        jid = self.batch.add(U, N_GHOST, dx, dx, dx)
        return jid, U

    def running(self, active) -> list:
        """Keys of the jobs to step now: all of them, or (fcfs) the earliest admitted ones up to
        the saturation cap (at least one)."""
        if self.policy == "all":
            return list(active)
        run, cells = [], 0
        for key, slot in active.items():  # admission order
            if run and cells >= self.saturation_cells:
                break
            run.append(key)
            cells += slot[0].cells
        return run

    def _step(self, active):
        run = set(self.running(active))
        for key in active:
            want = key not in run
            if want != (key in self.held):
                self.batch.hold(key, want)
                (self.held.add if want else self.held.discard)(key)
        self.batch.step(1)
        finished = []
        for key in run:
            slot = active[key]
            slot[1] -= 1
            if slot[1] == 0:
                finished.append(key)
        return finished

    def _retire(self, key):
        self.held.discard(key)
        self.batch.remove(key)

    def _event_stream(self):
        return self.stream

    def close(self):
        self.batch.close()


class PerRequestServer(_Base):
    """Baseline: every job advanced by its own launches of the single-box step (engine box on
    its own stream; plain kernel launches, or a CUDA graph per job when graph=True)."""

    mode = "per_request"

    def __init__(self, torch, graph: bool = False, **kw):
        super().__init__(torch, **kw)
        self.graph = graph
        self.mode = "per_request_graph" if graph else "per_request"
        self.main = torch.cuda.Stream()
        self.boxes = {}
        self.next = 0

    def _cost(self, req):
        N = req.n + 2 * N_GHOST
        nf = self.scheme.n_fields
        # engine box scratch: U½ nf + GEp + Epre + W 2 (nf + 1) fields of 8 bytes
        return state_bytes(req, self.scheme) + (nf + 2 + 2 * (nf + 1)) * N ** 3 * 8

    def _admit(self, req):
        stream = self.torch.cuda.Stream()
        U, dx = init_state(self.torch, req, self.scheme, stream)
        N = req.n + 2 * N_GHOST
        box = Box(N, N, N, N_GHOST, dx, dx, dx, self.scheme)
        box.use_graph(self.graph)
        key = self.next
        self.next += 1
        self.boxes[key] = (box, stream, U)
        return key, U

    def _step(self, active):
        finished = []
        for key, slot in active.items():
            box, stream, U = self.boxes[key]
            box.advance(U, 1, 0.3, stream)
            slot[1] -= 1
            if slot[1] == 0:
                finished.append(key)
        # the step of every job is queued; the event below waits on all of their streams
        for key in active:
            box, stream, U = self.boxes[key]
            self.main.wait_stream(stream)
        return finished

    def _retire(self, key):
        box, stream, U = self.boxes.pop(key)
        self._closing = getattr(self, "_closing", [])
        self._closing.append((box, stream))

    def _event_stream(self):
        return self.main

    def close(self):
        for box, stream, U in self.boxes.values():
            box.close()
        for box, stream in getattr(self, "_closing", []):
            stream.synchronize()
            box.close()


MODES = ("batched", "per_request", "per_request_graph")


def serve(torch, requests: list[Request], mode: str = "batched", **kw) -> dict:
    """Run `requests` through one server (a mode of MODES); returns the summary."""
    if mode not in MODES:
        raise ValueError(f"mode must be one of {MODES}")
    if mode == "batched":
        srv = BatchedServer(torch, **kw)
    else:
        srv = PerRequestServer(torch, graph=(mode == "per_request_graph"), **kw)
    try:
        rep = srv.run(requests)
    finally:
        torch.cuda.synchronize()
        srv.close()
    return rep.summary()


def sweep(torch, rates, counts, seeds, modes=MODES, steps: int = 100, **kw) -> dict:
    """Every mode on the same seeded request streams: for each rate (with its request count) and
    each seed, one run per mode; per rate the mean over seeds of throughput, p50 and p99 (and each
    seed's [throughput, p50, p99]), and the batched server's ratios against each per-request mode
    seed by seed as [min, mean, max] (throughput: batched / per-request; p99: per-request /
    batched, so above 1 means the batched server is ahead on both)."""
    out = {}
    for mode in modes:  # module loading, first captures and allocator growth outside the runs
        serve(torch, make_requests(rate=2000.0, count=6, seed=99, steps=5), mode=mode, **kw)
    for rate, count in zip(rates, counts):
        runs = {m: [] for m in modes}
        for seed in seeds:
            for mode in modes:
                runs[mode].append(serve(torch, make_requests(rate=rate, count=count, seed=seed, steps=steps), mode=mode,
                                        **kw))
        row = {"requests": count, "seeds": list(seeds)}
        for mode in modes:
            rs = runs[mode]
            row[mode] = {k: float(np.mean([r[k] for r in rs])) for k in ("cell_updates_per_s", "p50_ms", "p99_ms")}
            row[mode]["per_seed"] = [[r["cell_updates_per_s"], r["p50_ms"], r["p99_ms"]] for r in rs]
            if "tuned" in rs[0]:
                row[mode]["tuned"] = rs[0]["tuned"]
        for base in modes:
            if base == "batched":
                continue
            tr = [b["cell_updates_per_s"] / p["cell_updates_per_s"] for b, p in zip(runs["batched"], runs[base])]
            pr = [p["p99_ms"] / b["p99_ms"] for b, p in zip(runs["batched"], runs[base])]
            row[f"vs_{base}"] = {"throughput_ratio": [min(tr), float(np.mean(tr)), max(tr)],
                                 "p99_ratio": [min(pr), float(np.mean(pr)), max(pr)]}
        out[f"{rate:g}"] = row
    return out


def main():
    import argparse
    import json

    import torch

    ap = argparse.ArgumentParser(description="serving sweep: batched server against per-request launches")
    ap.add_argument("--rates", default="100,2000")
    ap.add_argument("--counts", default="200", help="requests per rate (one per rate, or one for all)")
    ap.add_argument("--seeds", default="17,18,19")
    a = ap.parse_args()
    rates = [float(r) for r in a.rates.split(",")]
    counts = [int(c) for c in a.counts.split(",")]
    counts = (counts * len(rates))[:len(rates)] if len(counts) < len(rates) else counts
    seeds = [int(s) for s in a.seeds.split(",")]
    print(json.dumps(sweep(torch, rates, counts, seeds)), flush=True)


if __name__ == "__main__":
    main()

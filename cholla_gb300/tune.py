"""Autotuner of the batch schedule.

A batch step has three run-time schedule choices (`cgb_batch_set_chains`,
`cgb_batch_set_solo_cells`, `cgb_batch_set_tiles`): how many parallel chains of launches the
shared jobs are spread over, from what size a job runs the single-box kernels in a chain of its
own, and which of the two compiled tile shapes the shared corrector sweeps use (x sweep / y and
z sweeps: 30 x 2 x 4 / 30 x 8 x 1 cells, or 64 x 2 x 2 / 32 x 8 x 1).  Chains and the solo
threshold give the same results bit for bit; the two tile shapes are two compiled instantiations
of the same sweep, in which the compiler contracts a few products differently, so they agree to
rounding.  Which is fastest depends on the mix of job sizes and on the GPU.  `tune_batch` builds a representative batch of the given sizes (seeded blast and shock
tube states), times a few steps of every candidate with CUDA events on the batch stream, and
returns the fastest.  Results are cached per (sizes, scheme) in memory and, when a path is
given, in a JSON file, so a server tunes once per size mix.

    python -m cholla_gb300.tune --sizes 32,48,64,96,128 --repeat 2 [--precision mixed] [--cache f.json]
"""
from __future__ import annotations

import json
from pathlib import Path

CHAINS = (1, 2, 4)
SOLO_CELLS = (1 << 20, 2 << 20, 4 << 20, 1 << 62)  # padded cells; the last: never solo
TILES = (0, 1)

_cache: dict = {}


def _key(sizes, scheme) -> str:
    return json.dumps({"sizes": sorted(int(n) for n in sizes), "recon": scheme.reconstruction,
                       "solver": scheme.riemann_solver, "precision": scheme.precision, "de": bool(scheme.dual_energy)})


def tune_batch(torch, scheme, sizes, steps: int = 6, warmup: int = 2, cache_path: str | Path | None = None) -> dict:
    """Fastest (chains, solo_cells, tiles) for a batch holding one job per entry of `sizes` (real
    cells per side).  Returns {"chains", "solo_cells", "tiles", "ms_per_step", "table"}."""
    key = _key(sizes, scheme)
    if key in _cache:
        return _cache[key]
    path = Path(cache_path) if cache_path else None
    if path and path.exists():
        stored = json.loads(path.read_text())
        if key in stored:
            _cache[key] = stored[key]
            return stored[key]
    from .batch import Batch
    from .serve import N_GHOST, Request, init_state

    stream = torch.cuda.Stream()
    states = [init_state(torch, Request(i, 0.0, int(n), "blast" if i % 2 == 0 else "tube", 1000 + i), scheme, stream)
              for i, n in enumerate(sizes)]
    torch.cuda.synchronize()
    table = []
    for tiles in TILES:
        for chains in CHAINS:
            for solo in SOLO_CELLS:
                bt = Batch(scheme, stream, c_cfl=0.3)
                bt.set_chains(chains)
                bt.set_solo_cells(solo)
                bt.set_tiles(tiles)
                work = [(U.clone(), dx) for U, dx in states]
                for U, dx in work:
                    bt.add(U, N_GHOST, dx, dx, dx)
                bt.step(warmup)  # the job set is stable from here: the timed steps replay one graph
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                bt.step(steps)
                b.record(stream)
                b.synchronize()
                table.append({"chains": chains, "solo_cells": solo, "tiles": tiles,
                              "ms_per_step": a.elapsed_time(b) / steps})
                bt.close()
                del work
    best = min(table, key=lambda r: r["ms_per_step"])
    out = {"chains": best["chains"], "solo_cells": best["solo_cells"], "tiles": best["tiles"],
           "ms_per_step": best["ms_per_step"], "table": table}
    _cache[key] = out
    if path:
        stored = json.loads(path.read_text()) if path.exists() else {}
        stored[key] = out
        path.write_text(json.dumps(stored, indent=1))
    return out


def main():
    import argparse

    import torch

    from .serve import default_scheme

    ap = argparse.ArgumentParser(description="time the batch schedules on a size mix and print the table")
    ap.add_argument("--sizes", default="32,48,64,96,128", help="real cells per side of the jobs")
    ap.add_argument("--repeat", type=int, default=2, help="jobs per size")
    ap.add_argument("--precision", choices=["mixed", "fp64_fast"], default="mixed")
    ap.add_argument("--cache", default=None, help="JSON file to read and extend")
    a = ap.parse_args()
    scheme = default_scheme()
    scheme.precision = a.precision
    sizes = [int(x) for x in a.sizes.split(",") if x] * a.repeat
    print(json.dumps(tune_batch(torch, scheme, sizes, cache_path=a.cache), indent=1))


if __name__ == "__main__":
    main()

"""Benchmark: cell updates/s of the VL hydro step on one GB300 (and N replicas under torchrun).

Workload (N=1 line): the 3D adiabatic hydro box -- 256^3 real cells (+4 ghosts), periodic,
gamma 5/3, PPMC + HLLC + VL, dual energy, density and temperature floors, CFL 0.3; seeded
lognormal density (sigma 0.5) and k^-2 velocities at rms Mach 2, uniform pressure.  A step
is one full VL step of the box through the library: ghost fill, dt from the device-side CFL
reduction, predictor, corrector, finalize (DE select/sync, temperature floor, CFL reduction).

    python bench.py [--steps K] [--warmup W] [--gpus N] [--n 256] [--impl ours|reference]

Besides the headline line's own numbers it reports, on the same GPU: the other arithmetic forms;
per-field accuracy against the exact FP64 form for the 256^3 box (20 steps) and every job of a
serving stream, and against the fast FP64 form for the 512^3 box in mixed precision (50 steps);
the 512^3 box's speed in every form and of the reference's own CUDA build; the 256^3 ideal-MHD
box; the serving sweep (100 and 2000 req/s, three seeds); the drop-in C ABI end to end with host
copies; and the CPU baseline (the FP64 host oracle on the same 256^3 box).

--impl reference times the reference's CPU path: the FP64 host restatement of the same scheme
(oracle/, OpenMP over every host core) on the same 256^3 box, W warm-up and K timed steps.
Multi-GPU (torchrun): every rank steps its own independent box (replicas; there is no
collective on this path); value = all cells updated / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

PEAKS = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0
L2_BYTES = 129 * 2 ** 20


def hbm_peak():
    try:
        return float(json.loads(PEAKS.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(world, value, device=None):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------------------------------
# CPU path (the oracle): cpu_baseline and --impl reference
# ------------------------------------------------------------------------------------------
def cpu_sample(n_sample: int, min_seconds: float, max_steps: int, threads: int):
    import oracle
    from cholla_gb300 import ics

    ng, gamma = 4, 5.0 / 3.0
    U = ics.turbulence_box(n_sample, ng, gamma, seed=0)
    nf, N = U.shape[0], U.shape[1]
    dx = 1.0 / n_sample
    oracle.set_threads(threads)
    cfg = oracle.config(N, N, N, ng, nf, de=True, recon=oracle.PPMC, solver=oracle.HLLC, gamma=gamma, dx=dx, dy=dx,
                        dz=dx)
    flat = U.reshape(-1)
    steps, t0 = 0, time.perf_counter()
    while True:
        oracle.set_boundaries(cfg, flat, (1,) * 6)
        dt = 0.3 / oracle.calc_dt(cfg, flat)
        oracle.vl_step_3d(cfg, flat, dt)
        oracle.temperature_floor(cfg, flat, 0.0)
        steps += 1
        el = time.perf_counter() - t0
        if steps >= max_steps or (min_seconds > 0 and el >= min_seconds):
            break
    return n_sample ** 3 * steps / el, steps, el


def run_reference(args, world, rank):
    """The reference's CPU implementation of the path: the FP64 host restatement (oracle), on the
    same n^3 box as our arm, every step a full step of it."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n = args.n
    cpu_sample(n, 0.0, args.warmup, threads)  # warm-up steps (untimed)
    cu_s, steps, el = cpu_sample(n, 0.0, args.steps, threads)
    sample = (f"{steps} full steps of the {n}^3 box of the same workload (seed 0), exact FP64 oracle, "
              f"{threads} OpenMP threads")
    line = {
        "metric": "cell updates/s", "value": cu_s, "unit": "cell-updates/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args),
        "cpu_baseline": {"value": cu_s, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": cu_s, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(args, n_override=None):
    n = n_override or args.n
    return {"workload": f"3D adiabatic hydro {n}^3 periodic turbulence-like box, PPMC+HLLC+VL, dual energy, "
                        f"density+temperature floors, CFL 0.3",
            "n": n, "n_ghost": 4, "fields": 6, "gamma": 5.0 / 3.0, "reconstruction": "PPMC",
            "riemann": "HLLC", "precision": getattr(args, "precision", "fp64_fast"),
            "l2": f"state {6 * (n + 8) ** 3 * 8 / 1e6:.0f} MB > L2 129 MB (inputs larger than L2)"}


# ------------------------------------------------------------------------------------------
# GPU path
# ------------------------------------------------------------------------------------------
def time_box(box, U, steps, stream, torch):
    """CUDA-event time of `steps` device-resident steps on `stream` (graph replay, dt on device)."""
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    box.advance(U, steps, 0.3, stream)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def kernel_breakdown(box, U, steps, stream):
    box.enable_timing(True)
    box.advance(U, steps, 0.3, stream)
    kt = box.kernel_times()
    box.enable_timing(False)
    k = max(kt["steps"], 1)
    return {name: kt[name] / k for name in ("predictor", "corrector", "finalize")}


def scheme_of(prec, gamma=5.0 / 3.0):
    from cholla_gb300 import integrator as I

    return I.Scheme(reconstruction="PPMC", riemann_solver="HLLC", dual_energy=True, density_floor=True,
                    temperature_floor=True, gamma=gamma, precision=prec)


# kernels one engine step launches: ghost fill, dt, [primitives], predictor, corrector (three
# sweeps), negative-density repair, finalize
LAUNCHES_PER_STEP = {"fp64": 8, "fp64_fast": 9, "mixed": 9}


def time_reference_build(R, U0, n, ng, gamma, dev, stream, torch, steps, sync_each=False):
    """ms per step of the reference's own CUDA build (its kernels, launched as VL_Algorithm_3D_CUDA
    launches them, plus its Calc_dt_GPU with the device-to-host copy of dt, its temperature floor and
    its ghost fill), on `stream`, after one warm-up step."""
    N, nf, dx = n + 2 * ng, U0.shape[0], 1.0 / n
    R.init("hydro_ppmc_hllc_de")
    R.set_stream(stream)
    R.set_sync_each(sync_each)
    Ur = torch.from_numpy(U0).to(dev)

    def ref_step():
        R.set_boundaries(Ur, N, N, N, ng, nf, (1,) * 6)
        dti = R.calc_dt(Ur, N, N, N, ng, nf, dx, dx, dx, gamma)
        R.vl_step_3d(Ur, N, N, N, ng, dx, dx, dx, 0.3 / dti, nf, gamma, 0.0)
        R.temperature_floor(Ur, N, N, N, ng, nf, 0.0)

    try:
        ref_step()
        stream.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(steps):
            ref_step()
        f1.record(stream)
        f1.synchronize()
        return f0.elapsed_time(f1) / steps
    finally:
        R.set_sync_each(False)
        del Ur


REF_BUILD_NOTE = ("reference hot-path .cu files compiled unchanged for sm_103a with its Makefile flags "
                  "(-O3 -fmad=false), launched kernel by kernel as VL_Algorithm_3D_CUDA does; 'no_sync' is its "
                  "-DDISABLE_GPU_ERROR_CHECKING build (no device synchronisation between kernels: the conservative "
                  "baseline the speedups divide by), 'sync_each' its default build (cudaDeviceSynchronize after "
                  "every kernel, src/utils/gpu.hpp:139-155)")


def run_ours(args, world, rank, local):
    import torch

    from cholla_gb300 import accuracy, ics
    from cholla_gb300 import integrator as I
    from cholla_gb300.engine import Box

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n, ng, gamma = args.n, 4, 5.0 / 3.0
    N = n + 2 * ng
    dx = 1.0 / n
    scheme = scheme_of

    U0 = ics.turbulence_box(n, ng, gamma, seed=rank)
    nf = U0.shape[0]
    state_bytes = U0.nbytes
    stream = torch.cuda.Stream(device=dev)
    U = torch.from_numpy(U0).to(dev)
    box = Box(N, N, N, ng, dx, dx, dx, scheme(args.precision))
    box.use_graph(True)
    box.advance(U, args.warmup, 0.3, stream)
    stream.synchronize()

    # ---- timed region: the headline arithmetic, device-resident, graph replay, dt on device ----
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = time_box(box, U, args.steps, stream, torch)
    torch.cuda.synchronize()
    barrier(world)
    ms_max = max_over_ranks(world, ms, dev)
    value = n ** 3 * args.steps * world / (ms_max / 1e3)

    # ---- per-kernel times over a second timed region (events on the launching stream) ----
    kt = kernel_breakdown(box, U, args.steps, stream)
    box.close()
    del U
    corr_ms = kt["corrector"]
    # algorithmic bytes of the corrector stage per step (its sweep launches): half-step primitives
    # in (6 fields, compute type), U^n in and U^{n+1} out (6 fields FP64), GasEnergy partial update
    # in, pre-sync energy out
    wbytes = 4 if args.precision == "mixed" else 8
    corr_bytes = n ** 3 * (nf * wbytes + 2 * nf * 8 + 2 * 8)
    peak, peak_kind = hbm_peak()
    achieved = corr_bytes / (corr_ms / 1e3) / 1e9

    # ---- the other arithmetic forms of the same step, for comparison (rank 0) ----
    others = {}
    if rank == 0 and not args.no_variants:
        for prec, k in (("fp64", 2), ("mixed", 20), ("fp64_fast", 5)):
            if prec == args.precision:
                continue
            Uv = torch.from_numpy(U0).to(dev)
            bv = Box(N, N, N, ng, dx, dx, dx, scheme(prec))
            bv.use_graph(True)
            bv.advance(Uv, 1, 0.3, stream)
            stream.synchronize()
            vms = time_box(bv, Uv, k, stream, torch) / k
            others[prec] = {"value": n ** 3 / (vms / 1e3), "ms_per_step": vms, "steps": k,
                            "kernels_ms": kernel_breakdown(bv, Uv, 2, stream)}
            bv.close()
            del Uv

    # ---- accuracy of the throughput forms against the exact FP64 form at n^3, 20 steps ----
    acc = None
    if rank == 0 and not args.no_accuracy:
        acc = accuracy.run(torch, n=n, steps=20, seed=rank, forms=("fp64_fast", "mixed"), U0=U0)

    # ---- the reference's own CUDA build on the same GPU (cubins compiled from its source) ----
    ref_gpu = None
    if rank == 0 and not args.no_reference_gpu:
        try:
            from oracle import reference_gpu as R

            if R.available():
                rms = time_reference_build(R, U0, n, ng, gamma, dev, stream, torch, 3)
                rms_sync = time_reference_build(R, U0, n, ng, gamma, dev, stream, torch, 2, sync_each=True)
                rv = n ** 3 / (rms / 1e3)
                ref_gpu = {"value": rv, "unit": "cell-updates/s", "ms_per_step": rms, "steps": 3,
                           "variant": "no_sync",
                           "sync_each": {"ms_per_step": rms_sync, "value": n ** 3 / (rms_sync / 1e3), "steps": 2},
                           "speedup_vs_reference_build": {"headline": (value / world) / rv,
                                                          **{p: o["value"] / rv for p, o in others.items()}},
                           "build": REF_BUILD_NOTE}
        except Exception as ex:  # the reference build is a comparison, not part of the product
            ref_gpu = {"unavailable": str(ex)[:200]}

    # ---- the 512^3 box: every form, the reference build, and mixed-precision accuracy (50 steps) ----
    big = None
    if rank == 0 and not args.no_512:
        big = run_512(args, dev, stream, torch)

    # ---- ideal MHD (PLMC + HLLD + CT) on the same GPU: ours and the reference build ----
    mhd = None
    if rank == 0 and not args.no_variants:
        mhd = run_mhd(args, dev, stream, torch)

    # ---- continuous-batching serving against per-request launches (rank 0) ----
    serving = None
    if rank == 0 and not args.no_serving:
        serving = run_serving(args, torch)

    # ---- end to end through the drop-in C ABI with host buffers ----
    e2e = None
    if rank == 0 and not args.no_e2e:
        # Double-buffered: step j's input is uploaded (copy stream `up`) while step j-1
        # computes, and step j's result is downloaded (stream `down`) while step j+1 computes;
        # every step still copies its whole state in from and out to pinned host memory.
        host = torch.from_numpy(ics.turbulence_box(n, ng, gamma, seed=rank)).pin_memory()
        outs = [torch.empty_like(host).pin_memory() for _ in range(2)]
        dbuf = [torch.empty_like(host, device=dev) for _ in range(2)]
        up, down = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)
        h2d, comp, d2h = ([torch.cuda.Event() for _ in range(2)] for _ in range(3))
        I.set_scheme(scheme(args.precision))
        I.set_stream(stream)
        k = max(4, min(args.steps, 8))  # enough steps to amortise the pipeline's fill and drain

        def upload(j):
            i = j % 2
            up.wait_event(d2h[i])  # step j-2's download has read this buffer
            with torch.cuda.stream(up):
                dbuf[i].copy_(host, non_blocking=True)
            h2d[i].record(up)

        def run(j):
            i, Ud = j % 2, dbuf[j % 2]
            stream.wait_event(h2d[i])
            I.Set_Boundaries(Ud, N, N, N, ng, nf, (1,) * 6)
            dti = I.Calc_dt_GPU(Ud, N, N, N, ng, nf, dx, dx, dx, gamma)
            I.VL_Algorithm_3D_CUDA(Ud, None, N, N, N, 0, 0, 0, ng, dx, dx, dx, 0, 0, 0, 0.3 / dti, nf, 0, 0.0)
            I.Apply_Temperature_Floor(Ud, N, N, N, ng, nf, 0.0)
            comp[i].record(stream)
            down.wait_event(comp[i])
            with torch.cuda.stream(down):
                outs[i].copy_(Ud, non_blocking=True)
            d2h[i].record(down)

        def run_steps(count):
            upload(0)
            for j in range(count):
                if j + 1 < count:
                    upload(j + 1)
                run(j)

        for ev in d2h:
            ev.record(stream)
        run_steps(2)  # warm-up
        for st_ in (stream, up, down):
            st_.synchronize()
        t0 = time.perf_counter()
        run_steps(k)
        for st_ in (stream, up, down):
            st_.synchronize()
        el = time.perf_counter() - t0
        I.set_stream(None)
        e2e = {"value": n ** 3 * k / el, "unit": "cell-updates/s", "h2d_bytes_per_step": state_bytes,
               "d2h_bytes_per_step": state_bytes, "steps": k,
               "path": "cgb_set_boundaries + cgb_calc_dt_gpu + cgb_vl_algorithm_3d + cgb_apply_temperature_floor, "
                       "pinned host state copied in and out every step, double-buffered (the next step's "
                       "upload and the previous step's download overlap the step on their own copy streams)"}
        del dbuf

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        cu_s, steps, el = cpu_sample(n, 10.0, 400, threads)
        cpu = {"value": cu_s, "unit": "cell-updates/s", "cores": threads, "kind": "port",
               "sample": f"{steps} full steps of the {n}^3 box of the same workload in {el:.1f} s (FP64 oracle, "
                         f"OpenMP on {threads} threads)"}

    if rank == 0:
        clocks = clk.summary()
        line = {
            "metric": "cell updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if args.precision == "mixed" else "f64",
            "data": "synthetic (seeded turbulence-like initial state, generated on the host)",
            "config": {**workload_config(args), "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": load_traffic(n, args.precision),
                         "kernel": "corrector (its sweep launches in one step)", "kernel_ms": corr_ms,
                         "kernels_ms": kt, "algorithmic_bytes_per_step": corr_bytes,
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json)",
                         "binding_ceiling": "FP64 pipe: GB300 FP64 FMA measured 1.19 TFLOP/s, divide 60 G/s"},
            "fp64_pipe": fp64_pipe(args.precision, value / world),
            "variants": others,
            "accuracy": acc,
            "at_512": big,
            "mhd": mhd,
            "serving": serving,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "reference_gpu": ref_gpu,
            "gpu_launches": LAUNCHES_PER_STEP[args.precision] * args.steps,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)


def run_512(args, dev, stream, torch):
    """The 512^3 box of the same workload: ms per step of every arithmetic form and of the
    reference's build on the same GPU, and the mixed form's per-field accuracy after 50 steps
    against the fast FP64 form on the same dt sequence (the fast form is within 1e-15 relative
    L1 per field of the exact one at this size; tests/test_config_scale_gpu.py checks the mixed
    form against the exact form itself, which takes 100 s here)."""
    from cholla_gb300 import accuracy, ics
    from cholla_gb300.engine import Box

    n, ng, gamma = 512, 4, 5.0 / 3.0
    N, dx = n + 2 * ng, 1.0 / n
    U0 = ics.turbulence_box(n, ng, gamma, seed=0)
    out = {"workload": "3D adiabatic hydro 512^3 periodic turbulence-like box (seed 0, rms Mach 2), PPMC+HLLC+VL, "
                       "dual energy, floors, CFL 0.3", "n": n}
    for prec, k in (("fp64_fast", 3), ("mixed", 10), ("fp64", 2)):
        U = torch.from_numpy(U0).to(dev)
        box = Box(N, N, N, ng, dx, dx, dx, scheme_of(prec))
        box.use_graph(True)
        box.advance(U, 1, 0.3, stream)
        stream.synchronize()
        ms = time_box(box, U, k, stream, torch) / k
        out[prec] = {"ms_per_step": ms, "value": n ** 3 / (ms / 1e3), "steps": k}
        box.close()
        del U
    try:
        from oracle import reference_gpu as R

        if R.available():
            rms = time_reference_build(R, U0, n, ng, gamma, dev, stream, torch, 2)
            out["reference_gpu"] = {"ms_per_step": rms, "value": n ** 3 / (rms / 1e3), "steps": 2,
                                    "variant": "no_sync", "build": REF_BUILD_NOTE}
            out["speedup_vs_reference_build"] = {p: rms / out[p]["ms_per_step"] for p in ("fp64_fast", "mixed", "fp64")}
    except Exception as ex:  # the reference build is a comparison, not part of the product
        out["reference_gpu"] = {"unavailable": str(ex)[:200]}
    if not args.no_accuracy:
        out["accuracy_mixed_vs_fp64_50_steps"] = accuracy.run(torch, n=n, steps=50, seed=0, forms=("mixed",), U0=U0,
                                                              baseline="fp64_fast")
    return out


def run_mhd(args, dev, stream, torch):
    """The 3D ideal-MHD workload at n^3 (PLMC + HLLD + constrained transport, beta = 1, random
    velocities and a divergence-free field from a random vector potential, CFL 0.3): our engine
    step and the reference's own kernels on the same GPU, 2 timed steps each."""
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I
    from cholla_gb300.engine import Box

    n, gamma = args.n, 5.0 / 3.0
    s = I.Scheme(reconstruction="PLMC", riemann_solver="HLLD", mhd=True, dual_energy=False, gamma=gamma)
    ng = s.n_ghost()
    U0 = ics.mhd_box(n, ng, gamma, seed=1)
    nf, N = U0.shape[0], U0.shape[1]
    dx = 1.0 / n
    out = {"workload": f"3D ideal MHD {n}^3 periodic, PLMC + HLLD + CT, beta 1, CFL 0.3; exact FP64 (bit-identical "
                       "to the reference build) and fast FP64 (the same arithmetic with multiply-adds contracted)"}
    k = 2
    for key, prec in (("ours", "fp64"), ("ours_fast", "fp64_fast")):
        sp = I.Scheme(reconstruction="PLMC", riemann_solver="HLLD", mhd=True, dual_energy=False, gamma=gamma,
                      precision=prec)
        U = torch.from_numpy(U0).to(dev)
        box = Box(N, N, N, ng, dx, dx, dx, sp)
        box.use_graph(True)
        box.advance(U, 1, 0.3, stream)
        stream.synchronize()
        ms = time_box(box, U, k, stream, torch) / k
        box.close()
        del U
        out[key] = {"ms_per_step": ms, "value": n ** 3 / (ms / 1e3), "unit": "cell-updates/s"}
    ms = out["ours"]["ms_per_step"]
    try:
        from oracle import reference_gpu as R

        if R.available("mhd_plmc_hlld"):
            R.init("mhd_plmc_hlld")
            R.set_stream(stream)
            Ur = torch.from_numpy(U0).to(dev)

            def ref_step():
                R.set_boundaries(Ur, N, N, N, ng, nf, (1,) * 6)
                dti = R.calc_dt(Ur, N, N, N, ng, nf, dx, dx, dx, gamma)
                R.vl_step_3d(Ur, N, N, N, ng, dx, dx, dx, 0.3 / dti, nf, gamma, 0.0)

            ref_step()
            stream.synchronize()
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f0.record(stream)
            for _ in range(k):
                ref_step()
            f1.record(stream)
            f1.synchronize()
            rms = f0.elapsed_time(f1) / k
            out["reference_gpu"] = {"ms_per_step": rms, "value": n ** 3 / (rms / 1e3)}
            out["speedup_vs_reference_build"] = {"exact": rms / ms, "fast": rms / out["ours_fast"]["ms_per_step"]}
            del Ur
    except Exception as ex:  # the reference build is a comparison, not part of the product
        out["reference_gpu"] = {"unavailable": str(ex)[:200]}
    return out


def run_serving(args, torch):
    """Batched serving workload: seeded Poisson streams of independent 3D hydro jobs (sizes
    uniform over 32^3 .. 128^3, Sedov-like blast or randomly oriented Sod tube, PPMC + HLLC mixed
    precision, 100 steps each, admitted by free device memory) served by the continuous-batching
    server and by per-request launches of the single-box step (kernel by kernel, and from a CUDA
    graph per request), each mode warmed up first, at every arrival rate: one seed below 100 req/s,
    every seed of --serve-seeds from 100 req/s up.  Latency = arrival to completion of the last step.
    Then every job of a further stream against its exact FP64 twin."""
    from cholla_gb300 import accuracy, serve

    rates = [float(r) for r in args.serve_rates.split(",") if r]
    counts = [int(c) for c in args.serve_count.split(",") if c]
    counts = (counts * len(rates))[:len(rates)] if len(counts) < len(rates) else counts
    seeds = [int(x) for x in args.serve_seeds.split(",") if x]
    out = {"workload": "Poisson streams of 3D hydro jobs, n in {32,48,64,96,128}, blast or Sod tube, "
                       "PPMC + HLLC mixed, 100 steps",
           "batched_server": "first come first served up to 3 Mi cells per step (rest held); batch schedule "
                             "(chains, solo threshold, sweep tile set) autotuned on the size mix at start-up",
           "ratios": "vs_<mode>: [min, mean, max] over seeds of batched/per-request throughput and of "
                     "per-request/batched p99 (above 1: the batched server is ahead)",
           "rates": {}}
    for rate, count in zip(rates, counts):
        row = serve.sweep(torch, [rate], [count], seeds if rate >= 100 else seeds[:1])
        out["rates"].update(row)
    if not args.no_accuracy and args.serve_twins > 0:
        reqs = serve.make_requests(rate=100.0, count=args.serve_twins, seed=23, steps=100)
        twins = accuracy.serving_twins(torch, reqs)
        worst = {f: max(t["rel_l1"][f] for t in twins) for f in twins[0]["rel_l1"]}
        out["accuracy_vs_fp64_twins"] = {
            "how": "every job of a seeded stream (seed 23) run as a batch job (the served arithmetic: the same "
                   "bits whatever shares the batch) against its exact FP64 twin on the job's own dt sequence; "
                   "relative L1 over the real cells",
            "jobs": twins, "max_rel_l1": worst}
    return out


def fp64_pipe(precision, cells_per_s):
    """The step against the FP64-pipe ceiling: FP64-pipe instructions per real cell of one step
    (ncu smsp__inst_executed_pipe_fp64 x 32 at 160^3, profiles/traffic.json) times the measured
    cell updates per second, against this GPU's FP64 FMA rate measured here (cgb_selftest_fp64_rate:
    every SM issuing independent FMA chains)."""
    import ctypes

    from cholla_gb300 import _lib as L

    try:
        per_cell = json.loads((ROOT / "profiles" / "traffic.json").read_text())["fp64_per_real_cell"][precision]
    except Exception:
        return None
    rate = ctypes.c_double()
    if L.lib().cgb_selftest_fp64_rate(12000, ctypes.byref(rate), None) != L.CGB_OK:
        return None
    achieved = per_cell * cells_per_s
    return {"achieved_instr_per_s": achieved, "peak_fma_per_s": rate.value, "frac": achieved / rate.value,
            "instructions_per_real_cell": per_cell,
            "source": "ncu smsp__inst_executed_pipe_fp64 x 32 per real cell of one step at 160^3 "
                      "(profiles/fast_kernels_160cube_ncu.txt) x cell updates/s; peak measured in this run "
                      "by cgb_selftest_fp64_rate"}


def load_traffic(n, precision):
    """DRAM bytes of the corrector stage (its three sweep launches) in one step, from the committed ncu
    summary (profiles/traffic.json, bytes per real cell at 160^3), scaled to n^3 real cells (traffic
    grows with the number of cells)."""
    f = ROOT / "profiles" / "traffic.json"
    try:
        d = json.loads(f.read_text())
        return d["corrector"][precision]["dram_bytes_per_real_cell"] * n ** 3
    except Exception:
        return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-512", action="store_true")
    ap.add_argument("--serve-rates", default="100,2000")
    ap.add_argument("--serve-count", default="200", help="requests per rate (one per rate, or one for all)")
    ap.add_argument("--serve-seeds", default="17,18,19", help="request-stream seeds of the rates from 100 req/s up")
    ap.add_argument("--serve-twins", type=int, default=12, help="served jobs checked against their FP64 twins")
    ap.add_argument("--precision", choices=["fp64_fast", "fp64", "mixed"], default="fp64_fast")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()

"""Accuracy of the throughput forms of the hydro step against the exact FP64 form.

The exact FP64 form reproduces the reference's own CUDA build bit for bit, so it is the FP64
baseline here.  One seeded turbulence-like box (lognormal density, k^-2 velocities at rms
Mach 2, uniform pressure 1, gamma 5/3, periodic, 4 ghost layers, PPMC + HLLC + VL with dual
energy and floors) is advanced `steps` steps by the exact form with its own CFL time steps
(CFL 0.3); the recorded dt sequence then drives the fast FP64 and the mixed-precision forms
from the same initial state, so every form ends at the same time.  Reported per field: the
relative L1 error over the real cells, sum |U_form - U_fp64| / sum |U_fp64|, and, per form,
the drift of the total mass (relative) and of the total momenta (relative to the summed
absolute momentum).  A periodic box conserves both to accumulation roundoff unless the density
floor or the averaging of non-positive densities fires (both add mass, in the reference too).

    python -m cholla_gb300.accuracy --n 512 --steps 50
"""
from __future__ import annotations

import argparse
import json
import time

FIELDS = ("density", "momentum_x", "momentum_y", "momentum_z", "Energy", "GasEnergy")


def _scheme(precision: str):
    from . import integrator as I

    return I.Scheme(reconstruction="PPMC", riemann_solver="HLLC", dual_energy=True, density_floor=True,
                    temperature_floor=True, gamma=5.0 / 3.0, precision=precision)


def _steps(torch, U, n, ng, precision, count, dts=None, cfl=0.3):
    """Advance U `count` steps in place through the drop-in calls, with the given time steps or
    (dts None) CFL time steps; returns the time steps taken."""
    from . import integrator as I

    s = _scheme(precision)
    I.set_scheme(s)
    N, nf = n + 2 * ng, U.shape[0]
    dx = 1.0 / n
    out = []
    for k in range(count):
        I.Set_Boundaries(U, N, N, N, ng, nf, (1,) * 6)
        dt = dts[k] if dts is not None else cfl / I.Calc_dt_GPU(U, N, N, N, ng, nf, dx, dx, dx, s.gamma)
        I.VL_Algorithm_3D_CUDA(U, None, N, N, N, 0, 0, 0, ng, dx, dx, dx, 0, 0, 0, dt, nf, 0, 0.0)
        I.Apply_Temperature_Floor(U, N, N, N, ng, nf, 0.0)
        out.append(dt)
    torch.cuda.synchronize()
    return out


def run(torch, n: int = 64, steps: int = 10, seed: int = 0, forms=("mixed", "fp64_fast"), mach: float = 2.0,
        U0=None, baseline: str = "fp64") -> dict:
    """U0: the initial state (host array of turbulence_box(n, 4, 5/3, seed, mach)) if already built.
    baseline: the FP64 form that sets the dt sequence and the reference state, "fp64" (exact, the
    reference build's bits) or "fp64_fast" (within 1e-15 of it per field after 50 steps at 512^3,
    and 2.6x faster: for large boxes whose exact run would take minutes)."""
    from . import ics

    if baseline not in ("fp64", "fp64_fast"):
        raise ValueError("baseline must be 'fp64' or 'fp64_fast'")
    ng = 4
    if U0 is None:
        U0 = ics.turbulence_box(n, ng, 5.0 / 3.0, seed=seed, mach=mach)
    real = (slice(None), slice(ng, ng + n), slice(ng, ng + n), slice(ng, ng + n))
    host = torch.from_numpy(U0)
    U = host.to("cuda")
    sums0 = U[real][:4].sum(dim=(1, 2, 3))
    t0 = time.perf_counter()
    dts = _steps(torch, U, n, ng, baseline, steps)
    t_base = time.perf_counter() - t0
    ref = U[real].clone()
    denom = ref.abs().sum(dim=(1, 2, 3))
    base_name = "exact" if baseline == "fp64" else "fast"
    res = {"workload": f"3D hydro {n}^3 periodic turbulence-like box (seed {seed}, rms Mach {mach:g}), PPMC + HLLC + "
                       f"VL, dual energy, {steps} steps at CFL 0.3 of the {base_name} FP64 form",
           "baseline": ("exact FP64 form (bit-identical to the reference build)" if baseline == "fp64" else
                        "fast FP64 form (within 1e-15 relative L1 per field of the exact form after 50 steps at "
                        "512^3)"),
           "t_end": float(sum(dts)), "steps": steps, "seconds": {baseline: t_base}, "rel_l1": {}, "conservation": {}}
    mom_scale = ref[1:4].abs().sum()  # momenta drift relative to the total absolute momentum
    drift_m = (U[real][1:4].sum(dim=(1, 2, 3)) - sums0[1:4]).abs().max() / mom_scale
    res["conservation"][baseline] = {"mass": float(((U[real][0].sum() - sums0[0]) / sums0[0]).abs()),
                                     "momentum": float(drift_m)}
    del U
    for form in forms:
        Uf = host.to("cuda")
        t0 = time.perf_counter()
        _steps(torch, Uf, n, ng, form, steps, dts)
        res["seconds"][form] = time.perf_counter() - t0
        cur = Uf[real]
        err = (cur - ref).abs().sum(dim=(1, 2, 3)) / denom
        res["rel_l1"][form] = {FIELDS[i]: float(err[i]) for i in range(cur.shape[0])}
        drift_m = (cur[1:4].sum(dim=(1, 2, 3)) - sums0[1:4]).abs().max() / mom_scale
        res["conservation"][form] = {"mass": float(((cur[0].sum() - sums0[0]) / sums0[0]).abs()),
                                     "momentum": float(drift_m)}
        del Uf, cur
    return res


def serving_twins(torch, requests, sensitivity: bool = True) -> list[dict]:
    """Accuracy of served jobs: each request of the serving workload (mixed precision, see serve.py)
    is run as the batched server runs it -- a cgb_batch job, whose result is the same bit for bit
    whatever else shares the batch -- one step at a time, recording the job's own dt sequence;
    then its exact FP64 twin (same initial state) takes the same dt sequence through the drop-in
    calls.  Per request: the relative L1 error per field of the served result against the twin.

    With `sensitivity`, a second exact FP64 run on the same dt sequence starts from the initial
    state with every density raised by one unit in the last place: its distance from the twin is
    how much this problem itself amplifies a rounding-sized perturbation in FP64, the scale against
    which the served result's error is read (a blast or tube that wraps around the periodic box
    amplifies rounding by orders of magnitude whatever the arithmetic)."""
    from .batch import Batch
    from .serve import N_GHOST, default_scheme, init_state

    scheme = default_scheme()
    stream = torch.cuda.Stream()
    ng = N_GHOST
    out = []
    for req in requests:
        U, dx = init_state(torch, req, scheme, stream)
        stream.synchronize()
        U0 = U.clone()
        b = Batch(scheme, stream)
        jid = b.add(U, ng, dx, dx, dx)
        dts = []
        for _ in range(req.steps):
            b.step(1)
            dts.append(b.job_time(jid)[1])
        b.close()
        twin = U0.clone()
        _steps(torch, twin, req.n, ng, "fp64", len(dts), dts)
        real = (slice(None), slice(ng, ng + req.n), slice(ng, ng + req.n), slice(ng, ng + req.n))
        ref = twin[real]
        den = ref.abs().sum(dim=(1, 2, 3)).clamp_min(1e-300)
        err = (U[real] - ref).abs().sum(dim=(1, 2, 3)) / den
        rec = {"rid": req.rid, "n": req.n, "kind": req.kind, "steps": len(dts),
               "rel_l1": {FIELDS[i]: float(err[i]) for i in range(err.shape[0])}}
        if sensitivity:
            pert = U0.clone()
            pert[0] = torch.nextafter(pert[0], torch.full_like(pert[0], float("inf")))
            _steps(torch, pert, req.n, ng, "fp64", len(dts), dts)
            sen = (pert[real] - ref).abs().sum(dim=(1, 2, 3)) / den
            rec["fp64_one_ulp_sensitivity"] = {FIELDS[i]: float(sen[i]) for i in range(sen.shape[0])}
            del pert
        out.append(rec)
        del U, U0, twin
    return out


def main():
    import torch

    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--mach", type=float, default=2.0)
    a = ap.parse_args()
    print(json.dumps(run(torch, a.n, a.steps, a.seed, mach=a.mach)), flush=True)


if __name__ == "__main__":
    main()

"""Batches and serving on the GPU.

Every job of a batch runs the same kernels on its own tiles and its own dt, so its
result must equal the job run alone in a batch of one bit for bit, whatever else shares the
batch and whenever it joined.  The single-box engine computes the same step with its own
(differently fused) kernels, so the compiler contracts a few products differently: after one
step the two agree to rounding (relative L1 per field 1e-7 mixed, 1e-15 fast FP64; measured
2.4e-8 and 4.5e-17).  Over more steps a strong blast amplifies such last-bit differences
through the PPM limiter's branches (the fast FP64 form and the exact one part the same way),
so the engine comparison is made after one step.  The serving loop is exercised end to end on
a short request stream in both modes.
"""
import numpy as np
import pytest

from helpers import real_slice

pytestmark = pytest.mark.gpu

NG = 4


def _scheme(precision, solver="HLLC", recon="PPMC"):
    from cholla_gb300 import integrator as I

    return I.Scheme(reconstruction=recon, riemann_solver=solver, dual_energy=True, density_floor=True,
                    temperature_floor=True, gamma=5 / 3, precision=precision)


def _job_state(cuda, n, kind, seed, scheme):
    from cholla_gb300 import serve

    req = serve.Request(0, 0.0, n, kind, seed)
    U, dx = serve.init_state(cuda, req, scheme, cuda.cuda.current_stream())
    cuda.cuda.synchronize()
    return U, dx


def _alone(cuda, U0, dx, scheme, steps):
    from cholla_gb300.engine import Box

    U = U0.clone()
    N = U.shape[1]
    box = Box(N, N, N, NG, dx, dx, dx, scheme)
    st = cuda.cuda.Stream()
    box.advance(U, steps, 0.3, st)
    st.synchronize()
    t, _ = box.time()
    box.close()
    return U.cpu().numpy(), t


def _in_batch(cuda, U0, dx, scheme, steps, solo_cells=None, tiles=0):
    from cholla_gb300.batch import Batch

    U = U0.clone()
    st = cuda.cuda.Stream()
    bt = Batch(scheme, st, c_cfl=0.3)
    bt.set_tiles(tiles)
    if solo_cells is not None:
        bt.set_solo_cells(solo_cells)
    jid = bt.add(U, NG, dx, dx, dx)
    bt.step(steps)
    st.synchronize()
    t, _ = bt.job_time(jid)
    bt.close()
    return U.cpu().numpy(), t


def _rel_l1(a, b):
    return np.abs(a - b).sum(axis=(1, 2, 3)) / np.maximum(np.abs(b).sum(axis=(1, 2, 3)), 1e-300)


TOL = {"mixed": 1e-7, "fp64_fast": 1e-15}
# The exact solver's Newton iteration stops when the relative pressure change falls to 1e-6; a
# last-bit difference can move that stop by one pass, which moves the star pressure by about the
# square of the change (1e-12 relative) on such faces.
TOL_EXACT = {"mixed": 1e-6, "fp64_fast": 1e-9}


def _same(a, b):
    return (a.view(np.int64) == b.view(np.int64)) | (np.isnan(a) & np.isnan(b))


MIX5 = [(16, "blast", 1), (24, "tube", 2), (20, "blast", 3), (12, "tube", 4), (32, "tube", 5)]
# 21 jobs: two chunks of launches (16 jobs per chunk) running side by side
MIX21 = [(8 + 2 * (i % 5), "blast" if i % 3 else "tube", 30 + i) for i in range(21)]


# 24^3 and 32^3 jobs (32^3 and 40^3 padded) run solo when the threshold is 30000 padded cells
SOLO = 30000


@pytest.mark.parametrize("precision,jobs,chains,solo", [("mixed", MIX5, 1, None), ("fp64_fast", MIX5, 1, None),
                                                        ("mixed", MIX5, 3, None), ("mixed", MIX21, 1, None),
                                                        ("mixed", MIX21, 4, None), ("mixed", MIX5, 1, SOLO),
                                                        ("fp64_fast", MIX5, 2, SOLO)],
                         ids=["mixed-5", "fp64_fast-5", "mixed-5-3chains", "mixed-21", "mixed-21-4chains",
                              "mixed-5-solo", "fp64_fast-5-solo"])
def test_each_job_same_alone_and_in_the_mix(cuda, precision, jobs, chains, solo):
    """A job's result does not depend on the other jobs, on how they are spread over chains of
    launches (up to 16 jobs per chain, chains side by side) or on its place in them."""
    from cholla_gb300.batch import Batch

    s = _scheme(precision)
    states = [_job_state(cuda, n, k, sd, s) for n, k, sd in jobs]
    steps = 12
    alone = [_in_batch(cuda, U, dx, s, steps, solo) for U, dx in states]
    st = cuda.cuda.Stream()
    bt = Batch(s, st, c_cfl=0.3)
    bt.set_chains(chains)
    if solo is not None:
        bt.set_solo_cells(solo)
    mix = []
    for U0, dx in states:
        U = U0.clone()
        mix.append((U, bt.add(U, NG, dx, dx, dx)))
    bt.step(steps)
    st.synchronize()
    for (U, jid), (a, t_alone), (n, kind, sd) in zip(mix, alone, jobs):
        b = U.cpu().numpy()
        rs = real_slice(NG)
        assert _same(a[rs], b[rs]).all(), f"job {n}^3 {kind}: {(~_same(a[rs], b[rs])).sum()} values differ"
        t, _ = bt.job_time(jid)
        assert t == t_alone
        assert np.isfinite(b[rs]).all()
    bt.close()


@pytest.mark.parametrize("solver,recon", [("HLLC", "PPMC"), ("HLL", "PPMC"), ("HLLC", "PPMP"), ("ROE", "PLMP"),
                                          ("EXACT", "PLMC")])
@pytest.mark.parametrize("precision", ["mixed", "fp64_fast"])
def test_batch_step_agrees_with_the_engine_to_rounding(cuda, precision, solver, recon):
    s = _scheme(precision, solver, recon)
    tol = (TOL_EXACT if solver == "EXACT" else TOL)[precision]
    jobs = [(16, "blast", 1), (24, "tube", 2), (20, "blast", 3), (12, "tube", 4), (48, "blast", 7)]
    for n, kind, sd in jobs:
        U, dx = _job_state(cuda, n, kind, sd, s)
        b, tb = _in_batch(cuda, U, dx, s, 1)
        e, te = _alone(cuda, U, dx, s, 1)
        rs = real_slice(NG)
        err = _rel_l1(b[rs], e[rs])
        assert np.all(err <= tol), f"job {n}^3 {kind}: {err}"
        assert tb == te


def test_jobs_joining_and_leaving_midway(cuda):
    """Job A runs 10 steps; B joins after A's 4th and runs 6; C joins with B and leaves after 3.
    Each equals its run alone in a batch."""
    from cholla_gb300.batch import Batch

    s = _scheme("mixed")
    (UA0, dxa), (UB0, dxb), (UC0, dxc) = (_job_state(cuda, 20, "blast", 11, s), _job_state(cuda, 16, "tube", 12, s),
                                           _job_state(cuda, 24, "tube", 13, s))
    st = cuda.cuda.Stream()
    bt = Batch(s, st, c_cfl=0.3)
    UA, UB, UC = UA0.clone(), UB0.clone(), UC0.clone()
    a = bt.add(UA, NG, dxa, dxa, dxa)
    bt.step(4)
    b = bt.add(UB, NG, dxb, dxb, dxb)
    c = bt.add(UC, NG, dxc, dxc, dxc)
    bt.step(3)
    bt.remove(c)
    bt.step(3)
    st.synchronize()
    assert len(bt) == 2
    rs = real_slice(NG)
    for U, U0, dx, steps in ((UA, UA0, dxa, 10), (UB, UB0, dxb, 6), (UC, UC0, dxc, 3)):
        ref, _ = _in_batch(cuda, U0, dx, s, steps)
        assert _same(ref[rs], U.cpu().numpy()[rs]).all()
    bt.close()


@pytest.mark.parametrize("precision", ["mixed", "fp64_fast"])
def test_solo_job_equals_the_box_engine_bitwise(cuda, precision):
    """A job at or above the solo threshold runs the box engine's own step inside the batch."""
    s = _scheme(precision)
    for n, kind, sd in ((24, "tube", 2), (32, "blast", 5)):
        U, dx = _job_state(cuda, n, kind, sd, s)
        b, tb = _in_batch(cuda, U, dx, s, 6, solo_cells=SOLO)
        e, te = _alone(cuda, U, dx, s, 6)
        rs = real_slice(NG)
        assert _same(b[rs], e[rs]).all(), f"{n}^3 {kind}"
        assert tb == te


def test_held_job_resumes_where_it_stopped(cuda):
    """B is held for 3 of A's 7 steps: B ends 4 steps on, equal to 4 steps of B alone."""
    from cholla_gb300.batch import Batch

    s = _scheme("mixed")
    (UA0, dxa), (UB0, dxb) = _job_state(cuda, 20, "blast", 21, s), _job_state(cuda, 16, "tube", 22, s)
    st = cuda.cuda.Stream()
    bt = Batch(s, st, c_cfl=0.3)
    UA, UB = UA0.clone(), UB0.clone()
    a = bt.add(UA, NG, dxa, dxa, dxa)
    b = bt.add(UB, NG, dxb, dxb, dxb)
    bt.step(2)
    bt.hold(b)
    bt.step(3)
    bt.hold(b, False)
    bt.step(2)
    bt.hold(a)
    bt.hold(b)
    bt.step(1)  # everything held: no work
    st.synchronize()
    rs = real_slice(NG)
    for U, U0, dx, steps, jid in ((UA, UA0, dxa, 7, a), (UB, UB0, dxb, 4, b)):
        ref, t_ref = _in_batch(cuda, U0, dx, s, steps)
        assert _same(ref[rs], U.cpu().numpy()[rs]).all()
        assert bt.job_time(jid)[0] == t_ref
    bt.close()


@pytest.mark.parametrize("mode", ["batched", "per_request", "per_request_graph"])
def test_serving_loop_completes_a_request_stream(cuda, mode):
    from cholla_gb300 import serve

    reqs = serve.make_requests(rate=500.0, count=12, seed=5, steps=8, sizes=(16, 24, 32))
    summ = serve.serve(cuda, reqs, mode=mode)
    assert summ["requests"] == 12
    assert 0 < summ["p50_ms"] <= summ["p99_ms"]
    assert summ["cell_updates_per_s"] > 0


def test_autotuner_picks_a_measured_candidate(cuda):
    from cholla_gb300 import tune

    s = _scheme("mixed")
    r = tune.tune_batch(cuda, s, [16, 24, 32, 40], steps=2, warmup=2)
    assert len(r["table"]) == len(tune.CHAINS) * len(tune.SOLO_CELLS) * len(tune.TILES)
    assert all(row["ms_per_step"] > 0 for row in r["table"])
    best = min(r["table"], key=lambda row: row["ms_per_step"])
    assert (r["chains"], r["solo_cells"], r["tiles"]) == (best["chains"], best["solo_cells"], best["tiles"])
    assert tune.tune_batch(cuda, s, [40, 32, 24, 16]) is r  # cached per size mix


@pytest.mark.parametrize("precision", ["mixed", "fp64_fast"])
def test_tile_sets_agree_to_rounding(cuda, precision):
    """The two compiled sweep tile shapes of the shared kernels (cgb_batch_set_tiles) compute the
    same step; as for the engine's kernels, the compiler contracts a few products differently in
    the two instantiations, so after one step a job agrees to rounding (relative L1 per field
    1e-7 mixed, 1e-15 fast FP64), and each tile set is deterministic on its own.  The sizes leave
    partial tiles in both shapes (20, 24, 36 real cells against 30- and 64-cell x pencils)."""
    s = _scheme(precision)
    rs = real_slice(NG)
    for n, kind, sd in [(20, "blast", 11), (24, "tube", 12), (36, "blast", 13)]:
        U, dx = _job_state(cuda, n, kind, sd, s)
        a, ta = _in_batch(cuda, U, dx, s, 1, tiles=0)
        b, tb = _in_batch(cuda, U, dx, s, 1, tiles=1)
        err = _rel_l1(b[rs], a[rs])
        assert np.all(err <= TOL[precision]), f"{n}^3 {kind}: {err}"
        assert ta == tb
        for tiles, ref in ((0, a), (1, b)):
            again, _ = _in_batch(cuda, U, dx, s, 1, tiles=tiles)
            assert _same(again[rs], ref[rs]).all()

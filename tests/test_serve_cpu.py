"""Host logic of the serving loop without a GPU: the arrival stream and the admission /
retirement bookkeeping, driven by a fake backend whose steps complete at once."""
import numpy as np

from cholla_gb300 import serve


def test_poisson_stream_is_seeded_and_well_formed():
    a = serve.make_requests(rate=100.0, count=500, seed=3)
    b = serve.make_requests(rate=100.0, count=500, seed=3)
    assert [(r.arrival, r.n, r.kind, r.seed) for r in a] == [(r.arrival, r.n, r.kind, r.seed) for r in b]
    t = np.array([r.arrival for r in a])
    assert t[0] == 0.0 and np.all(np.diff(t) >= 0)
    assert abs(np.mean(np.diff(t)) - 0.01) < 0.002  # mean gap 1/rate
    assert {r.n for r in a} <= set(serve.SIZES) and len({r.n for r in a}) == len(serve.SIZES)
    assert {r.kind for r in a} == {"blast", "tube"}


class _Done:
    def query(self):
        return True

    def synchronize(self):
        pass


class FakeServer(serve._Base):
    mode = "fake"

    def __init__(self, budget, cost, max_active=256):
        self.scheme = serve.default_scheme()
        self.budget, self.max_active, self.depth = budget, max_active, 2
        self.cost, self.live, self.peak_used, self.used_now, self.peak_active = cost, {}, 0, 0, 0

    def _cost(self, req):
        return self.cost

    def _event(self):
        return _Done()

    def _admit(self, req):
        self.used_now += self.cost
        self.peak_used = max(self.peak_used, self.used_now)
        self.live[req.rid] = req
        self.peak_active = max(self.peak_active, len(self.live))
        return req.rid, None

    def _step(self, active):
        out = []
        for key, slot in active.items():
            slot[1] -= 1
            if slot[1] == 0:
                out.append(key)
        return out

    def _retire(self, key):
        self.live.pop(key)
        self.used_now -= self.cost


def test_admission_respects_memory_budget_and_every_request_completes():
    reqs = serve.make_requests(rate=1e6, count=40, seed=1, steps=5)  # all arrive at once
    srv = FakeServer(budget=10 * 100, cost=100)
    rep = srv.run(reqs)
    assert len(rep.requests) == 40
    assert srv.peak_active <= 10 and srv.peak_used <= 1000
    assert all(r.done >= r.admitted >= r.arrival for r in rep.requests)
    s = rep.summary()
    assert s["requests"] == 40 and s["p99_ms"] >= s["p50_ms"] >= 0


def test_a_job_larger_than_the_budget_still_runs_alone():
    reqs = serve.make_requests(rate=1e6, count=3, seed=2, steps=2)
    srv = FakeServer(budget=50, cost=100)
    rep = srv.run(reqs)
    assert len(rep.requests) == 3 and srv.peak_active == 1


def _sched(policy, cap):
    srv = object.__new__(serve.BatchedServer)  # the scheduler alone, no batch behind it
    srv.policy, srv.saturation_cells = policy, cap
    return srv


def test_fcfs_runs_the_earliest_jobs_up_to_the_saturation_cap():
    reqs = [serve.Request(i, 0.0, n, "tube", i) for i, n in enumerate((128, 32, 96, 64, 128))]
    active = {r.rid: [r, r.steps, None, 0] for r in reqs}  # admission order
    cap = 128 ** 3 + 32 ** 3 + 1
    assert _sched("fcfs", cap).running(active) == [0, 1, 2]  # stops once the cap is reached
    assert _sched("fcfs", 1).running(active) == [0]  # at least one job
    assert _sched("fcfs", 10 ** 12).running(active) == [0, 1, 2, 3, 4]
    assert _sched("all", 1).running(active) == [0, 1, 2, 3, 4]


def test_sweep_aggregates_every_seed_and_ratio(monkeypatch):
    """serve.sweep runs every mode on the same seeded streams and reports, per rate, the mean over
    seeds and the batched server's per-seed ratios as [min, mean, max] (throughput batched /
    per-request, p99 per-request / batched): checked with a fake `serve` whose numbers are known."""
    table = {  # (mode, seed) -> (throughput, p50, p99)
        ("batched", 1): (2.0, 10.0, 20.0), ("batched", 2): (3.0, 12.0, 30.0),
        ("per_request", 1): (1.0, 20.0, 40.0), ("per_request", 2): (2.0, 30.0, 60.0),
        ("per_request_graph", 1): (2.0, 15.0, 20.0), ("per_request_graph", 2): (1.5, 18.0, 45.0),
    }
    calls = []

    def fake_serve(torch, reqs, mode="batched", **kw):
        calls.append((mode, len(reqs)))
        if len(reqs) == 6:  # the warm-up stream
            return {"cell_updates_per_s": 1.0, "p50_ms": 1.0, "p99_ms": 1.0}
        key = (mode, 1 if reqs[0].seed == serve.make_requests(5.0, 3, seed=1)[0].seed else 2)
        t, p50, p99 = table[key]
        return {"cell_updates_per_s": t, "p50_ms": p50, "p99_ms": p99, **({"tuned": {"chains": 1}} if mode == "batched" else {})}

    monkeypatch.setattr(serve, "serve", fake_serve)
    out = serve.sweep(None, [5.0], [3], [1, 2])
    row = out["5"]
    assert row["requests"] == 3 and row["seeds"] == [1, 2]
    assert row["batched"]["cell_updates_per_s"] == 2.5 and row["per_request"]["p99_ms"] == 50.0
    assert row["batched"]["per_seed"] == [[2.0, 10.0, 20.0], [3.0, 12.0, 30.0]]
    assert row["batched"]["tuned"] == {"chains": 1}
    assert row["vs_per_request"]["throughput_ratio"] == [1.5, 1.75, 2.0]
    assert row["vs_per_request"]["p99_ratio"] == [2.0, 2.0, 2.0]
    assert row["vs_per_request_graph"]["throughput_ratio"] == [1.0, 1.5, 2.0]
    assert row["vs_per_request_graph"]["p99_ratio"] == [1.0, 1.25, 1.5]
    assert sum(1 for m, n in calls if n == 3) == 6  # three modes x two seeds

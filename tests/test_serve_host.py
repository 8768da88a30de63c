"""The serving scheduler's host logic (serve.Server.run) on fake instances: admission under the
slot and HBM limits, every request stepped exactly its step count, zero-step requests, and every
instance and batch closed when a batch step fails.  No GPU: BatchSim and the results are faked."""
import pytest

serve = pytest.importorskip("nebulaviewer_gb300.serve")


class FakeSim:
    def __init__(self, cells):
        self._n = cells
        self.steps = 0
        self.closed = False

    def close(self):
        self.closed = True


class FakeSnap:
    def __init__(self, cells):
        self.cells = cells
        self.made = []

    def branch(self, mod):
        s = FakeSim(self.cells)
        self.made.append(s)
        return s


def install(monkeypatch, max_slots=None, budget_cells=None, fail_on_tick=None):
    log = {"batches": [], "ticks": 0}

    class FakeBatch:
        def __init__(self, sims):
            assert all(not s.closed for s in sims)
            if max_slots is not None:
                assert len(sims) <= max_slots
            if budget_cells is not None:
                assert sum(s._n for s in sims) <= budget_cells
            self.sims = sims
            self.closed = False
            log["batches"].append(self)

        def step(self, k):
            log["ticks"] += 1
            if fail_on_tick is not None and log["ticks"] == fail_on_tick:
                raise RuntimeError("injected batch-step failure")
            for s in self.sims:
                s.steps += k

        def close(self):
            self.closed = True

    monkeypatch.setattr(serve, "BatchSim", FakeBatch)
    monkeypatch.setattr(serve, "result_of", lambda sim: dict(t=0.0, it=sim.steps, totals=None, xi_mean=0.0, state=[]))
    return log


def requests(snaps, steps):
    return [serve.Request(i, 0.001 * i, i % len(snaps), None, n) for i, n in enumerate(steps)]


def test_every_request_runs_its_steps_within_slots_and_budget(monkeypatch):
    snaps = [FakeSnap(1000), FakeSnap(3000)]
    log = install(monkeypatch, max_slots=3, budget_cells=5000)
    reqs = requests(snaps, [5, 2, 7, 1, 4, 3, 6, 2])
    srv = serve.Server(snaps, budget_bytes=5000 * 48.0, bytes_per_cell=48, max_slots=3)
    stats, done = srv.run(reqs, realtime=False)
    assert stats["requests"] == len(reqs) and len(done) == len(reqs)
    assert sorted(r.rid for r in done) == list(range(len(reqs)))
    for r in done:
        assert r.result["it"] == r.nsteps and r.sim is None and r.t_done >= r.t_admit
    assert all(s.closed for sn in snaps for s in sn.made)
    assert all(b.closed for b in log["batches"])
    assert stats["cell_steps"] == sum(r.nsteps * snaps[r.snap].cells for r in reqs)
    assert stats["p50_ms"] is not None and stats["p99_ms"] >= stats["p50_ms"]


def test_zero_step_requests_finish_at_admission(monkeypatch):
    snaps = [FakeSnap(100)]
    log = install(monkeypatch)
    stats, done = serve.Server(snaps).run(requests(snaps, [0, 3, 0]), realtime=False)
    assert stats["requests"] == 3
    assert {r.rid: r.result["it"] for r in done} == {0: 0, 1: 3, 2: 0}
    assert log["ticks"] == 3 and all(s.closed for s in snaps[0].made)


def test_no_requests_and_negative_step_counts():
    stats, done = serve.Server([]).run([], realtime=False)
    assert stats["requests"] == 0 and done == [] and stats["p50_ms"] is None
    with pytest.raises(ValueError):
        serve.Request(0, 0.0, 0, None, -1)


def test_a_failing_batch_step_closes_every_instance(monkeypatch):
    snaps = [FakeSnap(100), FakeSnap(200)]
    log = install(monkeypatch, fail_on_tick=3)
    with pytest.raises(RuntimeError, match="injected"):
        serve.Server(snaps, max_slots=2).run(requests(snaps, [4, 4, 4, 4]), realtime=False)
    assert all(s.closed for sn in snaps for s in sn.made)
    assert all(b.closed for b in log["batches"])


def test_a_request_beyond_the_budget_is_refused(monkeypatch):
    snaps = [FakeSnap(100), FakeSnap(10 ** 6)]
    install(monkeypatch)
    with pytest.raises(RuntimeError, match="budget"):
        serve.Server(snaps, budget_bytes=48.0 * 1000).run(requests(snaps, [2, 2]), realtime=False)
    assert all(s.closed for sn in snaps for s in sn.made)

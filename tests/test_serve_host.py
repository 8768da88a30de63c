"""The serving scheduler's host logic (serve.Server.run) on fake instances: admission under the
slot limit and under the HBM budget counted with every pooled instance's true footprint (busy or
idle), instances reused for later requests of the same snapshot, a warm pool built before traffic within
the budget, idle instances of other snapshots closed (least recently used first) to make room, every request stepped exactly its step
count, zero-step requests, and every instance and batch closed when a batch step fails.  No GPU:
BatchSim and the results are faked."""
import pytest

serve = pytest.importorskip("nebulaviewer_gb300.serve")


class FakeSim:
    def __init__(self, cells, nbytes):
        self._n = cells
        self.nbytes = nbytes
        self.steps = 0
        self.closed = False

    def footprint(self):
        return self.nbytes

    def step(self, k, sync=True):                # stepped alone (an instance of solo_cells or more)
        assert not self.closed
        self.steps += k
        self.alone = getattr(self, "alone", 0) + k

    def close(self):
        self.closed = True


class FakeSnap:
    def __init__(self, cells, nbytes=None, device=None):
        self.cells = cells
        self.footprint = nbytes if nbytes is not None else 40 * cells + 1000     # fields + some scratch
        self.made = []
        self.branched_into = 0
        if device is not None:
            self.device = device

    def branch(self, mod, stream=None):
        s = FakeSim(self.cells, self.footprint)
        s.stream = stream
        self.made.append(s)
        return s

    def branch_into(self, sim, mod):
        assert sim in self.made and not sim.closed
        sim.steps = 0                      # the snapshot's state again
        self.branched_into += 1
        return sim


def install(monkeypatch, max_slots=None, budget=None, fail_on_tick=None):
    log = {"batches": [], "ticks": 0, "calls": 0, "peak": 0}

    class FakeBatch:
        def __init__(self, sims):
            assert all(not s.closed for s in sims)
            if budget is not None:
                assert sum(s.footprint() for s in sims) <= budget          # the whole pool, idle ones too
            self.sims = sims
            self.active = [True] * len(sims)
            self.closed = False
            log["batches"].append(self)

        def set_active(self, flags):
            assert len(flags) == len(self.sims)
            self.active = list(flags)

        def step(self, k, sync=True):
            log["calls"] += 1
            log["ticks"] += k
            if fail_on_tick is not None and log["ticks"] >= fail_on_tick:
                raise RuntimeError("injected batch-step failure")
            live = [s for s, a in zip(self.sims, self.active) if a]
            assert live and all(not s.closed for s in live)
            if max_slots is not None:
                assert len(live) <= max_slots
            log["peak"] = max(log["peak"], sum(s.footprint() for s in self.sims))
            for s in live:
                s.steps += k

        def check_status(self):
            assert not self.closed

        def sync(self):
            self.check_status()

        def close(self):
            self.closed = True

    monkeypatch.setattr(serve, "BatchSim", FakeBatch)
    monkeypatch.setattr(serve, "result_of", lambda sim, keep_state=True: dict(t=0.0, it=sim.steps, totals=None,
                                                                              xi_mean=0.0, state=[]))
    return log


def requests(snaps, steps, pick=None):
    pick = pick or (lambda i: i % len(snaps))
    return [serve.Request(i, 0.001 * i, pick(i), None, n) for i, n in enumerate(steps)]


def test_every_request_runs_its_steps_within_slots_and_budget(monkeypatch):
    snaps = [FakeSnap(1000), FakeSnap(3000)]
    budget = snaps[0].footprint + 2 * snaps[1].footprint
    log = install(monkeypatch, max_slots=3, budget=budget)
    reqs = requests(snaps, [5, 2, 7, 1, 4, 3, 6, 2, 5, 3])
    srv = serve.Server(snaps, budget_bytes=budget, max_slots=3)
    stats, done = srv.run(reqs, realtime=False)
    assert stats["requests"] == len(reqs) and len(done) == len(reqs)
    assert sorted(r.rid for r in done) == list(range(len(reqs)))
    for r in done:
        assert r.result["it"] == r.nsteps and r.sim is None and r.t_done >= r.t_admit
    assert all(s.closed for sn in snaps for s in sn.made)
    assert all(b.closed for b in log["batches"])
    assert stats["cell_steps"] == sum(r.nsteps * snaps[r.snap].cells for r in reqs)
    assert stats["p50_ms"] is not None and stats["p99_ms"] >= stats["p50_ms"]
    assert stats["peak_pool_bytes"] <= budget and log["peak"] <= budget


def test_instances_are_reused_and_the_batch_is_not_rebuilt_per_admission(monkeypatch):
    snaps = [FakeSnap(500)]
    log = install(monkeypatch, max_slots=2)
    reqs = requests(snaps, [3, 3, 4, 2, 5, 1, 3, 2])
    stats, done = serve.Server(snaps, max_slots=2).run(reqs, realtime=False)
    assert stats["requests"] == 8 and stats["instances_built"] == 2 == len(snaps[0].made)
    assert stats["branches_in_place"] == 6 == snaps[0].branched_into
    assert stats["batch_rebuilds"] == len(log["batches"]) <= 2          # only when the pool grew
    assert {r.rid: r.result["it"] for r in done} == {r.rid: r.nsteps for r in reqs}
    # a round trip runs as many ticks as no busy request finishes within
    assert stats["ticks"] == log["ticks"] and stats["round_trips"] == log["calls"] < log["ticks"]


def test_a_warm_pool_serves_every_request_by_device_copies(monkeypatch):
    snaps = [FakeSnap(500), FakeSnap(800)]
    log = install(monkeypatch, max_slots=6)
    reqs = requests(snaps, [3, 3, 4, 2, 5, 1])       # snapshots 0, 1, 0, 1, 0, 1
    srv = serve.Server(snaps, max_slots=6)
    stats, done = srv.run(reqs, realtime=False, warm={0: 3, 1: 3})
    assert stats["instances_prewarmed"] == 6 and stats["instances_built"] == 0
    assert stats["branches_in_place"] == 6 == snaps[0].branched_into + snaps[1].branched_into
    assert stats["batch_rebuilds"] == 1 == len(log["batches"])     # the warm pool never changes
    assert {r.rid: r.result["it"] for r in done} == {r.rid: r.nsteps for r in reqs}
    assert all(s.closed for sn in snaps for s in sn.made)
    # a warm pool stops at the budget
    snaps = [FakeSnap(1000)]
    budget = 2 * snaps[0].footprint + 10
    install(monkeypatch, budget=budget)
    stats, _ = serve.Server(snaps, budget_bytes=budget).run(requests(snaps, [2, 2, 2]), realtime=False, warm={0: 5})
    assert stats["instances_prewarmed"] == 2 and stats["instances_built"] == 0 and stats["peak_pool_bytes"] <= budget


def test_idle_instances_of_other_snapshots_make_room(monkeypatch):
    snaps = [FakeSnap(1000), FakeSnap(2000)]
    budget = snaps[1].footprint + 10                 # one instance at a time
    log = install(monkeypatch, budget=budget)
    reqs = requests(snaps, [3, 2, 4, 1, 2])          # snapshots 0, 1, 0, 1, 0
    stats, done = serve.Server(snaps, budget_bytes=budget).run(reqs, realtime=False)
    assert stats["requests"] == 5 and stats["evicted"] == 4 and stats["instances_built"] == 5
    assert stats["peak_pool_bytes"] <= budget and log["peak"] <= budget
    assert all(s.closed for sn in snaps for s in sn.made)


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
        serve.Server(snaps, budget_bytes=snaps[0].footprint * 2).run(requests(snaps, [2, 2]), realtime=False)
    assert all(s.closed for sn in snaps for s in sn.made)


def test_instances_of_solo_cells_or_more_step_alone(monkeypatch):
    """instances that fill the GPU on their own are stepped through their own Sim.step in the same
    ticks and never enter a batch; the smaller ones are batched; every request runs its steps"""
    snaps = [FakeSnap(1000), FakeSnap(5000)]
    log = install(monkeypatch, max_slots=4)
    reqs = requests(snaps, [5, 2, 7, 1, 4, 3, 6, 2])          # snapshots 0, 1, 0, 1, ...
    stats, done = serve.Server(snaps, max_slots=4, solo_cells=4000).run(reqs, realtime=False)
    assert {r.rid: r.result["it"] for r in done} == {r.rid: r.nsteps for r in reqs}
    big, small = snaps[1].made, snaps[0].made
    assert big and small and all(s not in b.sims for b in log["batches"] for s in big)
    assert all(any(s in b.sims for b in log["batches"]) for s in small)
    assert sum(getattr(s, "alone", 0) for s in big) == stats["solo_ticks"] == sum(r.nsteps for r in reqs if r.snap == 1)
    assert sum(getattr(s, "alone", 0) for s in small) == 0
    assert stats["cell_steps"] == sum(r.nsteps * snaps[r.snap].cells for r in reqs)
    # large instances joining the pool rebuilt no batch: every rebuild changed the batched set
    sets = [tuple(id(s) for s in b.sims) for b in log["batches"]]
    assert stats["batch_rebuilds"] == len(sets) == len(set(sets)) <= len(small)
    assert all(s.closed for sn in snaps for s in sn.made) and all(b.closed for b in log["batches"])
    # large instances built (arrivals 1 ms apart) while a small one keeps stepping in its batch:
    # the batch is built once
    snaps = [FakeSnap(1000), FakeSnap(5000)]
    log = install(monkeypatch, max_slots=3)
    reqs = requests(snaps, [400, 2, 2, 2, 2, 2], pick=lambda i: 0 if i == 0 else 1)
    stats, done = serve.Server(snaps, max_slots=3, solo_cells=4000).run(reqs, realtime=True)
    assert {r.rid: r.result["it"] for r in done} == {r.rid: r.nsteps for r in reqs}
    assert stats["batch_rebuilds"] == 1 == len(log["batches"]) and len(snaps[1].made) >= 1
    # a pool of large instances only builds no batch at all
    snaps = [FakeSnap(5000)]
    log = install(monkeypatch)
    stats, done = serve.Server(snaps, solo_cells=4000).run(requests(snaps, [3, 4, 2]), realtime=False)
    assert log["batches"] == [] and stats["batch_rebuilds"] == 0 and log["calls"] == 0
    assert {r.rid: r.result["it"] for r in done} == {0: 3, 1: 4, 2: 2}
    # solo_cells=None batches every instance
    snaps = [FakeSnap(5000)]
    log = install(monkeypatch)
    stats, _ = serve.Server(snaps, solo_cells=None).run(requests(snaps, [3, 4]), realtime=False)
    assert stats["solo_ticks"] == 0 and log["ticks"] >= 4


def test_instances_stepped_alone_share_one_stream_apart_from_the_batch(monkeypatch):
    """on a CUDA device every instance of solo_cells or more is built on one stream of the server's
    (the same for all of them, so two never run side by side), the batched ones on the current
    stream; solo_streams=False keeps every instance on the current stream"""
    made = []

    class FakeStream:
        def __init__(self, device=None):
            made.append(self)

    monkeypatch.setattr(serve.torch.cuda, "Stream", FakeStream)
    snaps = [FakeSnap(1000, device="cuda:0"), FakeSnap(5000, device="cuda:0")]
    install(monkeypatch, max_slots=6)
    reqs = requests(snaps, [3, 4, 2, 5, 1, 3])
    stats, done = serve.Server(snaps, max_slots=6, solo_cells=4000).run(reqs, realtime=False)
    assert {r.rid: r.result["it"] for r in done} == {r.rid: r.nsteps for r in reqs}
    assert len(made) == 1 and len(snaps[1].made) >= 2
    assert all(s.stream is made[0] for s in snaps[1].made)
    assert all(s.stream is None for s in snaps[0].made)
    snaps = [FakeSnap(1000, device="cuda:0"), FakeSnap(5000, device="cuda:0")]
    install(monkeypatch, max_slots=6)
    serve.Server(snaps, max_slots=6, solo_cells=4000, solo_streams=False).run(requests(snaps, [3, 4]), realtime=False)
    assert len(made) == 1 and all(s.stream is None for sn in snaps for s in sn.made)

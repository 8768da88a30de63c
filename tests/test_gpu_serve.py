"""Serving with continuous batching: requests branch from device snapshots, are admitted as
slots / HBM budget free up, overlap on the device in one batch, and each result is the same as
running the request alone: bit-identical with the exact build; within the path's tolerance
(rel-L_inf 1e-5) with the fast build, whose batched and single-instance kernels may contract
multiply-adds differently."""
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=("exact", "fast"))
def env(request):
    from nebulaviewer_gb300 import build
    build.build(verbose=False)
    from nebulaviewer_gb300 import ics, serve, sim
    bases = [ics.torus(seed=3, device="cuda", shape=(32, 32, 32), nstars=2),
             ics.sheet(res=24, seed=4, nstars=3, device="cuda", shape=(32, 40, 24))]
    snaps = []
    for ic in bases:
        s = sim.Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                               ic["P"], mom=ic["mom"], rays=(64, 128), fuv_grid=(16, 16, 32), arith=request.param)
        s.step(4)
        snaps.append(serve.Snapshot(s))
        s.close()
    return serve, snaps


def _close(a, b, exact):
    if exact:
        return torch.equal(a, b)
    a, b = a.double(), b.double()
    return float((a - b).abs().max()) <= 1e-5 * max(float(b.abs().max()), 1e-30)


@pytest.mark.parametrize("slots,tight,solo", ((3, False, None), (8, True, None), (4, False, 31000)))
def test_served_results_equal_alone(env, slots, tight, solo):
    """8 requests over two snapshots: with 3 slots the pool's instances are branched into again by
    later requests; with a budget of one and a half instances (the two snapshots' instances are of
    about the same size), an idle instance is closed whenever the other snapshot needs room; with
    solo_cells between the two sizes, the torus instances (32^3 cells) step alone through Sim.step
    in the same ticks as the batched sheet instances (32 x 40 x 24)"""
    serve, snaps = env
    exact = snaps[0].arith == "exact"
    reqs = serve.poisson_requests(snaps, 8, rate=1000.0, seed=slots, steps=(3, 9))
    budget = max(s.footprint for s in snaps) * 1.5 if tight else 1e12
    srv = serve.Server(snaps, budget_bytes=budget, max_slots=slots, keep_state=True, solo_cells=solo)
    stats, done = srv.run(reqs, realtime=False)
    assert (stats["solo_ticks"] > 0) == (solo is not None)
    assert stats["requests"] == 8 and stats["ticks"] >= max(r.nsteps for r in done)
    assert stats["peak_pool_bytes"] <= budget
    assert stats["branches_in_place"] > 0 if not tight else stats["evicted"] > 0
    assert snaps[0].cells > 31000 > snaps[1].cells
    for r in done:
        ref = serve.run_alone(snaps[r.snap], r)
        assert r.result["it"] == ref["it"]
        assert r.result["t"] == ref["t"] if exact else abs(r.result["t"] - ref["t"]) <= 1e-6 * ref["t"]
        for a, b in zip(r.result["state"], ref["state"]):
            assert _close(a, b, exact)
        if exact:
            assert r.result["totals"] == ref["totals"]
        else:
            assert all(abs(x - y) <= 1e-6 * max(abs(y), 1e-30) + 1e-9 for x, y in zip(r.result["totals"], ref["totals"]))


def test_snapshot_branch_resumes_the_state(env):
    serve, snaps = env
    s = snaps[0].branch()
    assert torch.equal(s._rho, snaps[0].fields["rho"]) and torch.equal(s._xi, snaps[0].fields["xi"])
    assert s.it == snaps[0].meta["it"] and s.t == snaps[0].meta["t"]
    assert s.footprint() == snaps[0].footprint
    # a used instance branched into again starts from the same state as a fresh branch
    mod = ("q", 1, 1.5)
    s.step(5)
    snaps[0].branch_into(s, mod)
    f = snaps[0].branch(mod)
    for k in ("rho", "mx", "xi", "dfront", "g0"):
        assert torch.equal(getattr(s, "_" + k), getattr(f, "_" + k))
    assert s.it == f.it and s.t == f.t and s.stars == f.stars
    s.step(4)
    f.step(4)
    assert torch.equal(s._rho, f._rho) and torch.equal(s._xi, f._xi)
    s.close()
    f.close()

"""The timeline cache's bookkeeping on the host, with a stand-in simulation whose snapshot pack
writes its clock into the slot: lattice-aligned captures, coarsening under the slot budget
(survivors on a regular time grid, the newest always kept), no new slot once the budget is
reached, truncation for a branch, restore, budget changes and a run crossing tau = 0."""
import pytest
import torch

from nebulaviewer_gb300.timeline import LATTICE_POINTS, Timeline


class FakeSim:
    def __init__(self, n=8, t_end=1.0, tau0=0.0):
        self.shape = (n, 1, 1)
        self._n = n
        self.device = torch.device("cpu")
        self.P = {"t_end": t_end}
        self.now = tau0
        self.restored = None
        self.packs = 0

    def tau(self):
        return self.now

    def update_render_fields(self, force=False):
        return True

    def snapshot_pack(self, buf):
        self.packs += 1
        buf.view(torch.float64)[0] = self.now

    def snapshot_unpack(self, buf):
        self.restored = float(buf.view(torch.float64)[0])

    def get_state_meta(self):
        return {"tau": self.now}

    def set_state_meta(self, m):
        self.now = m["tau"]


def run(tl, sim, dt, n):
    for _ in range(n):
        sim.now += dt
        tl.maybe_capture(sim)


def test_captures_follow_the_lattice_and_coarsen_on_a_regular_grid():
    sim = FakeSim(n=8, t_end=1.0)
    tl = Timeline(budget_gb=8 * 13 * 10 / 1e9)                    # 10 slots
    tl.clear(sim)
    base = 1.0 / LATTICE_POINTS
    assert tl.capacity() == 10 and tl.base == pytest.approx(base)
    run(tl, sim, base / 3, 600)                                    # 200 bins: forces several coarsenings
    assert len(tl.snaps) <= 10 and tl.level >= 4
    taus = tl.taus()
    assert taus == sorted(taus) and sim.now - tl.stride <= taus[-1] <= sim.now
    # the survivors sit in consecutive groups of 2^level bins, starting with the first capture (a
    # group may hold a second one: a former newest, dropped at the next coarsening)
    groups = [tl._group(tl._bin(t)) for t in taus]
    assert groups == sorted(groups) and groups[0] == 0
    assert sorted(set(groups)) == list(range(groups[0], groups[-1] + 1))
    assert len(tl.snaps) - len(set(groups)) <= 1
    # no more slots than the budget allows, whatever happened
    assert len(tl._slots) <= 10
    # the buffers hold what was packed at those times
    for s in tl.snaps:
        assert float(s["buf"].view(torch.float64)[0]) == s["tau"]


def test_no_new_slot_once_full():
    sim = FakeSim(n=8, t_end=1.0)
    tl = Timeline(budget_gb=8 * 13 * 6 / 1e9)
    tl.clear(sim)
    run(tl, sim, 1.0 / LATTICE_POINTS, 40)
    slots = list(tl._slots)
    assert len(slots) == 6
    run(tl, sim, 1.0 / LATTICE_POINTS, 400)
    assert len(tl._slots) == 6 and all(a is b for a, b in zip(slots, tl._slots))


def test_truncate_restore_and_branch():
    sim = FakeSim(n=8, t_end=0.5)
    tl = Timeline(budget_gb=8 * 13 * 32 / 1e9)
    tl.clear(sim)
    run(tl, sim, 0.5 / LATTICE_POINTS, 20)
    i = tl.nearest(sim.now / 2)
    tau = tl.snaps[i]["tau"]
    assert tl.index_at_or_before(tau) == i and tl.index_at_or_before(-1.0) is None
    assert tl.restore(sim, i) and sim.restored == tau and sim.now == tau
    free0 = len(tl._free)
    tl.truncate_after(tau)
    assert tl.taus()[-1] == tau and len(tl._free) > free0
    run(tl, sim, 0.5 / LATTICE_POINTS, 5)                          # the branch is captured anew
    assert tl.taus() == sorted(tl.taus()) and tl.taus()[-1] > tau
    other = FakeSim(n=16)
    assert not tl.restore(other, 0)                                # another grid: refused


def test_budget_changes_and_a_run_across_zero():
    sim = FakeSim(n=8, t_end=1.0, tau0=-0.3)                       # stirring phase: tau < 0
    tl = Timeline(budget_gb=8 * 13 * 12 / 1e9)
    tl.clear(sim)
    run(tl, sim, 1.0 / LATTICE_POINTS, 200)                        # -0.3 .. +0.48
    assert min(tl.taus()) < 0.0 < max(tl.taus()) and len(tl.snaps) <= 12
    tl.set_budget(8 * 13 * 2 / 1e9)                                # two slots: the first and the newest
    assert len(tl.snaps) == 2 and len(tl._slots) == 2 and tl.taus()[0] < 0.0 < tl.taus()[1]
    for s in tl.snaps:
        assert float(s["buf"].view(torch.float64)[0]) == s["tau"]
    tl.set_budget(8 * 13 * 1 / 1e9)
    assert len(tl.snaps) == 1
    last = tl.taus()[0]
    run(tl, sim, 1.0 / LATTICE_POINTS, 50)
    assert len(tl.snaps) == 1 and tl.taus()[0] > last                # still capturing, one slot
    assert "snapshots" in tl.status()
    tl.clear(sim)
    assert tl.status() == "timeline empty" and tl.snaps == []

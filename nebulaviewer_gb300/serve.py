"""Serving branch requests from device snapshots with continuous batching.

A request branches from a device snapshot of an instance (the state the reference keeps in
its timeline, timeline.py:95-203, restored through Sim.set_state_meta, sim.py:1185-1211,
then advanced as viewer.py's branch-and-play does), changes one star's photon rate or the
wind by a factor, and runs a number of steps.  The server admits queued requests whenever a
slot and HBM (under a byte budget at a stated cost per cell) are free, advances every admitted
request together in one batch (BatchSim: persistent kernels, CUDA graphs) one step per tick,
retires finished requests at once and admits new ones at the next tick, so work that arrives
while others run overlaps with them on the device.  Each request's result is bit-identical to
running it alone.
"""
import collections
import time

import numpy as np

from .batch import BatchSim
from .sim import Sim


class Snapshot:
    """A full-precision device snapshot of a Sim (fields, clock, stars, parameters)."""

    def __init__(self, sim):
        sim._sync()
        self.shape, self.dx, self.device = sim.shape, sim.dx, sim.device
        self.fields = {k: getattr(sim, "_" + k).clone() for k in ("rho", "mx", "my", "mz", "xi", "dfront", "g0")}
        self.meta = sim.get_state_meta()
        self.rays, self.fuv = sim.rfront.shape, sim.att.shape
        self.ion_every, self.fast, self.arith = sim.ion_every, sim.fast, sim.arith
        self.torus = sim.torus0 if sim.phase == "pre" else None          # joins when the stirring phase ends
        self.stir_grid = (sim.sshape, sim.dxs)

    @property
    def cells(self):
        return int(np.prod(self.shape))

    def branch(self, mod=None):
        """a new Sim resuming from this snapshot; mod = ("q", star_index, factor) | ("wind", factor)"""
        m = self.meta
        f = self.fields
        s = Sim.from_state(self.shape, self.dx, f["rho"], m["stars"], m["kinds"], m["jets"], m["jkinds"], m["P"],
                           mom=[f["mx"], f["my"], f["mz"]], rays=self.rays, fuv_grid=self.fuv,
                           ion_every=self.ion_every, fast=self.fast, device=self.device, start_main=False,
                           torus=self.torus, stir_grid=self.stir_grid, arith=self.arith)
        s._xi.copy_(f["xi"])
        s._dfront.copy_(f["dfront"])
        s._g0.copy_(f["g0"])
        s.set_state_meta(m)
        if mod is not None:
            if mod[0] == "q":
                i, fac = int(mod[1]), float(mod[2])
                st = list(s.stars[i])
                st[3] = st[3] * fac
                s.stars[i] = tuple(st)
            elif mod[0] == "wind":
                s.set_param("wind", s.P["wind"] * float(mod[1]))
            else:
                raise ValueError(f"unknown modification {mod!r}")
        return s


class Request:
    def __init__(self, rid, t_arrive, snap, mod, nsteps):
        if int(nsteps) < 0:
            raise ValueError(f"a request runs nsteps >= 0 steps, not {nsteps}")
        self.rid, self.t_arrive, self.snap, self.mod, self.nsteps = rid, t_arrive, snap, mod, int(nsteps)
        self.sim = None
        self.left = self.nsteps
        self.t_admit = self.t_done = None
        self.result = None


def poisson_requests(snapshots, n, rate, seed=0, steps=(10, 100), factor=0.5):
    """n requests with exponential inter-arrival times (rate per second); each picks a
    snapshot, a +-factor change of one star's photon rate or of the wind, and a step count"""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for rid in range(n):
        t += float(rng.exponential(1.0 / rate))
        si = int(rng.integers(len(snapshots)))
        sign = 1.0 if rng.random() < 0.5 else -1.0
        fac = 1.0 + sign * factor
        if rng.random() < 0.5:
            mod = ("q", int(rng.integers(len(snapshots[si].meta["stars"]))), fac)
        else:
            mod = ("wind", fac)
        out.append(Request(rid, t, si, mod, int(rng.integers(steps[0], steps[1] + 1))))
    return out


def result_of(sim):
    """what a finished request returns: the clock, FP64 totals and a digest of the fields"""
    c = sim._clock()
    tot = sim.conservation()
    xi = sim._xi
    return dict(t=c.t, it=int(c.it), totals=tot, xi_mean=float(xi.double().mean()),
                state=[t.clone() for t in (sim._rho, sim._mx, sim._my, sim._mz, sim._xi)])


class Server:
    """Continuous batching under an HBM budget."""

    def __init__(self, snapshots, budget_bytes=150e9, bytes_per_cell=48, max_slots=64, keep_state=False):
        self.snaps = snapshots
        self.budget = float(budget_bytes)
        self.bpc = float(bytes_per_cell)
        self.max_slots = int(max_slots)
        self.keep_state = keep_state
        self.ticks = 0
        self.rebuilds = 0

    def _cost(self, req):
        return self.snaps[req.snap].cells * self.bpc

    def run(self, requests, realtime=True):
        """serve `requests` (in arrival order; realtime=False admits each as soon as it fits);
        returns (stats, the finished requests in completion order).  On an error every instance and
        batch still open is closed before it propagates."""
        pending = collections.deque(sorted(requests, key=lambda r: r.t_arrive))
        queue = collections.deque()
        active, done = [], []
        used = 0.0
        batch = None
        t0 = time.perf_counter()
        cell_steps = 0

        def finish(r):                       # the result, then the instance is closed whatever happens
            try:
                r.result = result_of(r.sim)
                if not self.keep_state:
                    r.result.pop("state")
            finally:
                r.sim.close()
                r.sim = None
            r.t_done = time.perf_counter() - t0
            done.append(r)

        try:
            while pending or queue or active:
                now = time.perf_counter() - t0
                while pending and (pending[0].t_arrive <= now or not realtime):
                    queue.append(pending.popleft())
                changed = False
                while queue and len(active) < self.max_slots and used + self._cost(queue[0]) <= self.budget:
                    r = queue.popleft()
                    r.sim = self.snaps[r.snap].branch(r.mod)
                    r.t_admit = time.perf_counter() - t0
                    if r.left == 0:                    # nothing to run: the branched state is the result
                        finish(r)
                        continue
                    used += self._cost(r)
                    active.append(r)
                    changed = True
                if queue and not active:
                    raise RuntimeError("a request does not fit the HBM budget on its own")
                if not active:
                    if pending:
                        time.sleep(max(0.0, min(pending[0].t_arrive - now, 0.01)))
                    continue
                if changed or batch is None:
                    if batch is not None:
                        batch.close()
                        batch = None
                    batch = BatchSim([r.sim for r in active])
                    self.rebuilds += 1
                batch.step(1)                          # one tick: every active request advances one step
                self.ticks += 1
                fin = []
                for r in active:
                    r.left -= 1
                    cell_steps += r.sim._n
                    if r.left == 0:
                        fin.append(r)
                if fin:
                    batch.close()
                    batch = None
                    for r in fin:
                        active.remove(r)
                        used -= self._cost(r)
                        finish(r)
        finally:
            if batch is not None:
                batch.close()
            for r in active:
                if r.sim is not None:
                    r.sim.close()
                    r.sim = None
        wall = time.perf_counter() - t0
        lat = np.array([r.t_done - r.t_arrive for r in done])
        pct = (lambda q: float(np.percentile(lat, q) * 1e3)) if len(lat) else (lambda q: None)
        return dict(requests=len(done), wall_s=wall, cell_steps=cell_steps, gcells_per_s=cell_steps / wall / 1e9,
                    p50_ms=pct(50), p99_ms=pct(99), ticks=self.ticks, batch_rebuilds=self.rebuilds), done


def run_alone(snapshot, req):
    """the same request on its own (the equivalence check)"""
    s = snapshot.branch(req.mod)
    s.step(req.nsteps)
    out = result_of(s)
    s.close()
    return out

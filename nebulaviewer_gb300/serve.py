"""Serving branch requests from device snapshots with continuous batching.

A request branches from a device snapshot of an instance (the state the reference keeps in
its timeline, timeline.py:95-203, restored through Sim.set_state_meta, sim.py:1185-1211,
then advanced as viewer.py's branch-and-play does, viewer.py:257-266), changes one star's
photon rate or the wind by a factor, and runs a number of steps.

The server keeps a pool of instances.  A request for a snapshot takes an idle instance built
from that snapshot if there is one and branches into it by device copies (no allocation);
otherwise a new instance is built, if its true device footprint -- its fields and the
library's scratch for it (nb_instance_bytes: ray and FUV tables sized for its stars, tensor
maps, ...) -- fits the HBM budget next to every instance already pooled, busy or idle; idle
instances of other snapshots are closed first, least recently used first, when that makes
room.  A server may also build a warm pool before traffic starts (run's `warm`: idle instances
per snapshot, within the budget).  The pooled instances below `solo_cells` cells live in one
BatchSim (persistent kernels, CUDA graphs): a request joins the stepping set when it is admitted
and leaves it when it has run its steps, through the batch's slot flags, so admissions and
retirements rebuild nothing; the batch and its graphs are rebuilt only when the set of small
instances in the pool changes.  An instance of `solo_cells` cells or more fills the GPU on its own, where the batched
kernels would only add their per-cell cost (the instance records they index, the work-list
walk), so it is stepped through its own Sim.step in the same tick.  The large instances share a
CUDA stream apart from the batch's: the batch and the large instances are launched together and
the small instances' kernels fill the large ones' tail waves, while the large instances still
run one after another (with a stream each, two of them side by side compete for the L2 their
ray casts and tile marches read from: the served mix then swung between 0.97x and 1.02x of the
requests run one at a time, from run to run; with one shared stream it stays at 0.99x).  Every tick advances all busy instances one step, so work that arrives while others
run overlaps with them on the device; a host round trip runs as many ticks as no busy request
finishes within (and, while arrivals are pending, as fit before the next one).
Each request's result is the same as running it alone (bit-identical with the exact build).
"""
import collections
import contextlib
import time

import numpy as np
import torch

from .batch import BatchSim
from .sim import Sim, footprint_bytes


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
        # device bytes of an instance branched from this snapshot, known before it is built
        self.footprint = footprint_bytes(self.shape, self.dx, self.meta["P"], self.rays, self.fuv, self.fast,
                                         len(self.meta["stars"]), self.arith)

    @property
    def cells(self):
        return int(np.prod(self.shape))

    def branch(self, mod=None, stream=None):
        """a new Sim resuming from this snapshot; mod = ("q", star_index, factor) | ("wind", factor);
        stream: the CUDA stream the instance works on (default: the current one)"""
        m = self.meta
        f = self.fields
        with on_stream(stream):
            s = Sim.from_state(self.shape, self.dx, f["rho"], m["stars"], m["kinds"], m["jets"], m["jkinds"],
                               m["P"], mom=[f["mx"], f["my"], f["mz"]], rays=self.rays, fuv_grid=self.fuv,
                               ion_every=self.ion_every, fast=self.fast, device=self.device, start_main=False,
                               torus=self.torus, stir_grid=self.stir_grid, arith=self.arith)
            self._resume(s, mod)
        return s

    def branch_into(self, sim, mod=None):
        """resume this snapshot in `sim`, an instance built from it before (Snapshot.branch) and
        since used for another request: device copies of the fields and the state meta, no
        allocation -- the same state a fresh branch starts from"""
        if tuple(sim.shape) != tuple(self.shape) or len(sim.stars) != len(self.meta["stars"]):
            raise ValueError("branch_into needs an instance built from this snapshot")
        sim.events = []
        with on_stream(getattr(sim, "_stream", None)):       # in order with the instance's earlier work
            self._resume(sim, mod)
        return sim

    def _resume(self, s, mod):
        for k in ("rho", "mx", "my", "mz", "xi", "dfront", "g0"):
            getattr(s, "_" + k).copy_(self.fields[k])
        s.set_state_meta(self.meta)
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


def on_stream(stream):
    """a context placing torch's work on `stream` (None: leave the current stream)"""
    return torch.cuda.stream(stream) if stream is not None else contextlib.nullcontext()


def result_of(sim, keep_state=True):
    """what a finished request returns: the clock, FP64 totals, a digest of the fields and (keep_state)
    a copy of the state (complete when this returns, whichever stream the instance works on)"""
    with on_stream(getattr(sim, "_stream", None)):
        c = sim._clock()
        tot = sim.conservation()
        xi = sim._xi
        out = dict(t=c.t, it=int(c.it), totals=tot, xi_mean=float(xi.sum(dtype=torch.float64)) / xi.numel())
        if keep_state:
            out["state"] = [t.clone() for t in (sim._rho, sim._mx, sim._my, sim._mz, sim._xi)]
            sim._sync()
    return out


class _Slot:
    """a pooled instance: the snapshot it was built from, the request it serves (None: idle), and
    the tick it was last released at"""

    def __init__(self, snap, sim, nbytes):
        self.snap, self.sim, self.nbytes = snap, sim, nbytes
        self.req = None
        self.last = -1


# Instances of at least this many cells are stepped alone (Sim.step) rather than in the batch:
# 8 Mi cells is ~2.7 waves of the stage kernels' resident 32 x 8 x 20-cell tiles on 152 SMs, past
# which a batch no longer fills idle SMs and its kernels cost ~5% more per cell than the
# single-instance ones (measured on the served mix: 96^3-320^3 snapshots).
SOLO_CELLS = 8 * 2 ** 20


class Server:
    """Continuous batching over a pool of instances under an HBM budget (see the module text)."""

    def __init__(self, snapshots, budget_bytes=150e9, max_slots=64, keep_state=False, solo_cells=SOLO_CELLS,
                 solo_streams=True):
        self.snaps = snapshots
        self.budget = float(budget_bytes)
        self.max_slots = int(max_slots)
        self.keep_state = keep_state
        self.solo_cells = solo_cells          # None: every instance in the batch
        self.solo_streams = solo_streams      # the instances stepped alone work on a stream apart from the batch's
        self._solo_stream = {}                # device -> that stream
        self.ticks = 0
        self.round_trips = 0         # host round trips (each advances one or more ticks)
        self.solo_ticks = 0          # instance-ticks stepped alone (instances of solo_cells or more)
        self.rebuilds = 0
        self.built = 0               # instances built
        self.reused = 0              # requests branched into a pooled instance
        self.evicted = 0             # idle instances closed to make room
        self.prewarmed = 0           # idle instances built before the clock started (run's `warm`)
        self.peak_bytes = 0

    def run(self, requests, realtime=True, warm=None):
        """serve `requests` (in arrival order; realtime=False admits each as soon as it fits);
        returns (stats, the finished requests in completion order).  warm = {snapshot index: n}
        builds up to n idle instances of each snapshot before the clock starts (as far as the
        budget allows), the warm pool a server keeps for the traffic it expects, so that requests
        branch into them by device copies.  On an error every instance and batch still open is
        closed before it propagates."""
        pending = collections.deque(sorted(requests, key=lambda r: r.t_arrive))
        queue = collections.deque()
        pool, done = [], []
        batch, batch_pool = None, []

        def solo(p):
            return self.solo_cells is not None and p.sim._n >= self.solo_cells

        def build(snap, mod):
            """a new instance of snap: one to be stepped alone works on the stream of those"""
            dev = getattr(snap, "device", None)
            if (self.solo_streams and self.solo_cells is not None and snap.cells >= self.solo_cells
                    and dev is not None and torch.device(dev).type == "cuda"):
                key = str(torch.device(dev))
                if key not in self._solo_stream:
                    self._solo_stream[key] = torch.cuda.Stream(device=dev)
                return snap.branch(mod, stream=self._solo_stream[key])
            return snap.branch(mod)

        dirty = False                # the pool changed since the batch was built
        cell_steps = 0
        tick_s = 0.0                 # wall time per tick of the last round trip
        self.prewarmed = 0
        try:
            for si, n in sorted((warm or {}).items()):
                snap = self.snaps[si]
                for _ in range(int(n)):
                    if sum(p.nbytes for p in pool) + snap.footprint > self.budget:
                        break
                    sim = build(snap, None)
                    pool.append(_Slot(si, sim, sim.footprint()))
                    self.prewarmed += 1
            self.peak_bytes = max(self.peak_bytes, sum(p.nbytes for p in pool))
        except BaseException:
            for p in pool:
                p.sim.close()
            raise
        dirty = bool(pool)
        t0 = time.perf_counter()

        def pool_bytes():
            return sum(p.nbytes for p in pool)

        def finish(slot):            # the result; the instance stays in the pool, idle
            r = slot.req
            r.result = result_of(slot.sim, self.keep_state)
            r.sim = None
            r.t_done = time.perf_counter() - t0
            done.append(r)
            slot.req = None
            slot.last = self.ticks

        def admit(r):
            """an instance for r (reused, or built within the budget); False when r must wait"""
            nonlocal dirty
            snap = self.snaps[r.snap]
            idle = [p for p in pool if p.req is None and p.snap == r.snap]
            if idle:
                slot = max(idle, key=lambda p: p.last)
                snap.branch_into(slot.sim, r.mod)
                self.reused += 1
            else:
                cost = snap.footprint
                others = sorted((p for p in pool if p.req is None), key=lambda p: p.last)
                if pool_bytes() + cost > self.budget and pool_bytes() - sum(p.nbytes for p in others) + cost > self.budget:
                    return False                     # even closing every idle instance makes no room
                while pool_bytes() + cost > self.budget:
                    p = others.pop(0)                # least recently used idle instance
                    pool.remove(p)
                    p.sim.close()
                    self.evicted += 1
                    dirty = True
                sim = build(snap, r.mod)
                slot = _Slot(r.snap, sim, sim.footprint())
                pool.append(slot)
                self.built += 1
                dirty = True
                if slot.nbytes > cost:
                    raise RuntimeError(f"an instance holds {slot.nbytes} bytes, more than the {cost} it was admitted for")
            slot.req = r
            r.sim = slot.sim
            r.t_admit = time.perf_counter() - t0
            self.peak_bytes = max(self.peak_bytes, pool_bytes())
            return slot

        try:
            while pending or queue or any(p.req is not None for p in pool):
                now = time.perf_counter() - t0
                while pending and (pending[0].t_arrive <= now or not realtime):
                    queue.append(pending.popleft())
                while queue and sum(p.req is not None for p in pool) < self.max_slots:
                    slot = admit(queue[0])
                    if not slot:
                        break
                    queue.popleft()
                    if slot.req.left == 0:             # nothing to run: the branched state is the result
                        finish(slot)
                busy = [p for p in pool if p.req is not None]
                if queue and not busy:
                    raise RuntimeError("a request does not fit the HBM budget on its own")
                if not busy:
                    if pending:
                        time.sleep(max(0.0, min(pending[0].t_arrive - now, 0.01)))
                    continue
                if dirty:
                    # the batch holds the smaller instances only: a large one joining or leaving the
                    # pool rebuilds nothing
                    small = [p for p in pool if not solo(p)]
                    if [id(p) for p in small] != [id(p) for p in batch_pool] or (small and batch is None):
                        if batch is not None:
                            batch.close()
                            batch = None
                        batch_pool = small
                        if batch_pool:
                            batch = BatchSim([p.sim for p in batch_pool])
                            self.rebuilds += 1
                    dirty = False
                flags = [p.req is not None for p in batch_pool]
                alone = [p for p in busy if solo(p)]
                # ticks: every busy instance advances one step per tick.  As many ticks per host round
                # trip as no busy request finishes within and, while arrivals are pending, as fit before
                # the next one is due (at the last round trip's time per tick)
                k = min(p.req.left for p in busy)
                if pending and realtime:
                    k = min(k, max(1, int((pending[0].t_arrive - now) / max(tick_s, 1e-4))))
                t_tick = time.perf_counter()
                # the batch and the instances stepped alone are all launched before any of them is
                # waited for: on two streams, the batch runs beside the large instances
                if any(flags):
                    if flags != list(batch.active):
                        batch.set_active(flags)
                    batch.step(k, sync=False)
                for p in alone:
                    p.sim.step(k, sync=False)
                for p in alone:
                    p.sim.step(0)                    # its clock mirrored and read: raises if a TMA wait gave up
                if any(flags):
                    batch.sync()
                self.solo_ticks += k * len(alone)
                tick_s = (time.perf_counter() - t_tick) / k
                self.ticks += k
                self.round_trips += 1
                for p in busy:
                    p.req.left -= k
                    cell_steps += p.sim._n * k
                    if p.req.left == 0:
                        finish(p)
        finally:
            if batch is not None:
                batch.close()
            for p in pool:
                if p.req is not None:
                    p.req.sim = None
                p.sim.close()
        wall = time.perf_counter() - t0
        lat = np.array([r.t_done - r.t_arrive for r in done])
        pct = (lambda q: float(np.percentile(lat, q) * 1e3)) if len(lat) else (lambda q: None)
        return dict(requests=len(done), wall_s=wall, cell_steps=cell_steps, gcells_per_s=cell_steps / wall / 1e9,
                    p50_ms=pct(50), p99_ms=pct(99), ticks=self.ticks, round_trips=self.round_trips,
                    solo_ticks=self.solo_ticks,
                    batch_rebuilds=self.rebuilds,
                    instances_built=self.built, instances_prewarmed=self.prewarmed, branches_in_place=self.reused,
                    evicted=self.evicted, peak_pool_bytes=self.peak_bytes, budget_bytes=self.budget), done


def run_alone(snapshot, req):
    """the same request on its own (the equivalence check)"""
    s = snapshot.branch(req.mod)
    s.step(req.nsteps)
    out = result_of(s)
    s.close()
    return out

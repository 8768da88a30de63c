"""Timeline cache: device snapshots of a running simulation for scrubbing back, replaying and
branching -- the role of the reference's Timeline (timeline.py:95-203).  The method names are
the ones the reference's viewer calls (viewer.py:84-298, 422-429): clear, maybe_capture,
capture, restore, nearest, index_at_or_before, truncate_after, set_budget, status, taus and
`snaps[i]["tau"]`; the snapshot itself is the reference's 13 B/cell format (timeline.py:19-89),
packed on the device (Sim.snapshot_pack).

How it keeps snapshots (this package's own scheme):

* Slots.  Each snapshot occupies one slot: a device buffer of 13 bytes per cell.  Slots are made
  on demand until the byte budget is reached and then reused from a free list, so once the cache
  has filled a capture, a thinning or a truncation never allocates device memory.
* Lattice.  Simulated time (tau: negative in the stirring phase, sim.tau()) is cut into bins of
  `base` = t_end / 256, counted from the time of clear() (or of the first capture), so bins are
  never negative.  At retention level L a group spans 2^L bins; the cache keeps the earliest
  snapshot of every group and the newest snapshot (the live end of the run).
* Coarsening.  When every slot is taken and a new snapshot comes, the level rises until the kept
  set leaves a slot free; the snapshots that lose their place give their slots back.  Because
  the rule is tied to the lattice, not to positions in the list, the survivors stay on a regular
  grid of simulated time however many times the cache was coarsened, and a snapshot made off the
  lattice (a direct capture) is treated like any other.
* Captures.  maybe_capture takes a snapshot once tau reaches the start of the next bin of the
  current level after the newest snapshot.
"""
import bisect
import math

import torch

BYTES_PER_CELL = 13                  # timeline.py:19-89: fp16 rho, m (x3), uint8 xi, fp16 dfront, g0
LATTICE_POINTS = 256                 # lattice bins over t_end


class Timeline:
    def __init__(self, budget_gb=8.0, device="cuda:0"):
        self.device = torch.device(device)
        self.budget = float(budget_gb) * 1e9
        self.snaps = []              # sorted by tau: dict(tau, bin, slot, buf, shape, meta)
        self.base = 1e-3             # lattice bin width (clear() sets it from t_end)
        self.origin = None           # tau of bin 0 (clear(sim), else the first capture)
        self.level = 0               # kept: the earliest snapshot per 2^level bins, and the newest
        self.ncells = 0
        self._slots = []             # device buffers, BYTES_PER_CELL * ncells bytes each
        self._free = []              # indices of unused slots
        self._next_bin = None        # maybe_capture waits for tau to reach this bin (None: any)

    # ---------------------------------------------------------------- sizes
    def _slot_bytes(self):
        return BYTES_PER_CELL * max(self.ncells, 1)

    def capacity(self):
        return max(1, int(self.budget // self._slot_bytes()))

    def bytes_used(self):
        return len(self.snaps) * self._slot_bytes()

    @property
    def stride(self):
        """simulated time between kept snapshots at the current level"""
        return self.base * (1 << self.level)

    # ---------------------------------------------------------------- lattice
    def _bin(self, tau):
        return max(0, math.floor((tau - self.origin) / self.base + 1e-9))

    def _group(self, b, level=None):
        return b >> (self.level if level is None else level)

    def _kept(self, snaps, level):
        """the snapshots a level keeps: the earliest of each group of 2^level bins, and the newest"""
        out, seen = [], set()
        for k, s in enumerate(snaps):
            g = self._group(s["bin"], level)
            if g not in seen or k == len(snaps) - 1:
                out.append(s)
                seen.add(g)
        return out

    def _coarsen_to(self, n_max):
        """raise the level until at most n_max snapshots are kept (bins are not negative, so at a
        high enough level one group holds them all and two are kept: the first and the newest);
        release the others' slots.  With room for fewer than two, only the newest stays."""
        keep = self.snaps
        while len(keep) > n_max >= 2:
            self.level += 1
            keep = self._kept(keep, self.level)
        if len(keep) > n_max:
            keep = keep[len(keep) - n_max:] if n_max > 0 else []
        ids = {id(s) for s in keep}
        self._free.extend(s["slot"] for s in self.snaps if id(s) not in ids)
        self.snaps = keep

    # ---------------------------------------------------------------- the viewer's calls
    def clear(self, sim=None):
        """forget every snapshot (the slots stay for reuse); with a sim: size the cache for its grid
        and start the lattice at its current time"""
        self._free.extend(s["slot"] for s in self.snaps)
        self.snaps = []
        self.level = 0
        self._next_bin = None
        self.origin = None
        if sim is not None:
            self.origin = sim.tau()
            n = sim.shape[0] * sim.shape[1] * sim.shape[2]
            if n != self.ncells:                     # another grid: the slots no longer fit
                self._slots, self._free = [], []
                self.ncells = n
            self.base = max(float(sim.P.get("t_end", 0.25)) / LATTICE_POINTS, 1e-6)

    def set_budget(self, gb):
        """change the byte budget; above the new capacity the cache coarsens and drops slots"""
        self.budget = float(gb) * 1e9
        cap = self.capacity()
        self._coarsen_to(cap)
        if len(self._slots) > cap:                   # give the unused slots' memory back
            self._slots = [self._slots[s["slot"]] for s in self.snaps]
            for k, s in enumerate(self.snaps):
                s["slot"] = k
            self._free = []

    def taus(self):
        return [s["tau"] for s in self.snaps]

    def nearest(self, tau):
        if not self.snaps:
            return None
        t = self.taus()
        k = bisect.bisect_left(t, tau)
        cands = [i for i in (k - 1, k) if 0 <= i < len(t)]
        return min(cands, key=lambda i: abs(t[i] - tau))

    def index_at_or_before(self, tau):
        k = bisect.bisect_right(self.taus(), tau + 1e-12)
        return k - 1 if k > 0 else None

    def maybe_capture(self, sim):
        """after a step: a snapshot when tau has reached the next bin of the current level"""
        tau = sim.tau()
        if self.snaps and tau <= self.snaps[-1]["tau"] + 1e-12:
            return False
        if self._next_bin is not None and self.origin is not None and self._bin(tau) < self._next_bin:
            return False
        self.capture(sim)
        return True

    def capture(self, sim):
        """a snapshot of the sim now (G0 brought up to date first, as the renderer shows it)"""
        if not self.ncells:
            self.ncells = sim._n
        tau = sim.tau()
        if self.origin is None or (not self.snaps and tau < self.origin):
            self.origin = tau
        if self.snaps and tau <= self.snaps[-1]["tau"] + 1e-12:      # keep the list in time order
            self.truncate_after(tau - 1e-12)
        self._coarsen_to(self.capacity() - 1)
        sim.update_render_fields()
        slot = self._take_slot(sim)
        buf = self._slots[slot]
        sim.snapshot_pack(buf)
        b = self._bin(tau)
        self.snaps.append(dict(tau=tau, bin=b, slot=slot, buf=buf, shape=tuple(sim.shape),
                               meta=sim.get_state_meta()))
        self._next_bin = (self._group(b) + 1) << self.level
        return len(self.snaps) - 1

    def _take_slot(self, sim):
        if self._free:
            return self._free.pop()
        self._slots.append(torch.empty(self._slot_bytes(), dtype=torch.uint8, device=sim.device))
        return len(self._slots) - 1

    def restore(self, sim, i):
        """the sim's fields and state from snapshot i (False when it was taken on another grid)"""
        s = self.snaps[i]
        if tuple(s["shape"]) != tuple(sim.shape):
            return False
        sim.snapshot_unpack(s["buf"])
        sim.set_state_meta(s["meta"])
        return True

    def truncate_after(self, tau):
        """branch: forget every snapshot later than tau (the run continues from there anew)"""
        keep = [s for s in self.snaps if s["tau"] <= tau + 1e-12]
        self._free.extend(s["slot"] for s in self.snaps[len(keep):])
        self.snaps = keep
        if self.origin is not None:
            self._next_bin = (self._group(self._bin(tau)) + 1) << self.level

    def status(self):
        n = len(self.snaps)
        if not n:
            return "timeline empty"
        return (f"{n} snapshots of {self.capacity()}, {self.bytes_used() / 1e9:.2f}/{self.budget / 1e9:.1f} GB, "
                f"one per {self.stride:.4g} time units (level {self.level})")

"""Timeline cache: device snapshots of a simulation for scrubbing, playback and branching.

The reference's Timeline (timeline.py:95-203) over this package's `Sim`: the same methods
(clear, bytes_used, capacity, set_budget, taus, nearest, index_at_or_before, maybe_capture,
capture, restore, truncate_after, status) and the same 13 B/cell format (fp16 state, uint8
xi, fp16 dfront / g0; timeline.py:19-89), packed on the device by one kernel into one buffer
per snapshot; thinning under a byte budget keeps every other snapshot and doubles the spacing.
"""
import math

import torch

BYTES_PER_CELL = 13


class Timeline:
    def __init__(self, budget_gb=8.0, device="cuda:0"):
        self.device = torch.device(device)
        self.budget = budget_gb * 1e9
        self.snaps = []          # sorted by tau: dict(tau, buf, shape, meta)
        self.dtau = 0.002
        self.next_tau = -1e9
        self.ncells = 0
        self.thinned = 0

    def clear(self, sim=None):
        self.snaps = []
        self.thinned = 0
        if sim is not None:
            self.ncells = sim.shape[0] * sim.shape[1] * sim.shape[2]
            self.dtau = max(sim.P["t_end"] / 200.0, 1e-4)
            self.next_tau = sim.tau()

    def bytes_used(self):
        return len(self.snaps) * self.ncells * BYTES_PER_CELL

    def capacity(self):
        return max(1, int(self.budget // max(self.ncells * BYTES_PER_CELL, 1)))

    def set_budget(self, gb):
        self.budget = gb * 1e9
        while len(self.snaps) > self.capacity():
            self._thin()

    def taus(self):
        return [s["tau"] for s in self.snaps]

    def nearest(self, tau):
        if not self.snaps:
            return None
        return min(range(len(self.snaps)), key=lambda i: abs(self.snaps[i]["tau"] - tau))

    def index_at_or_before(self, tau):
        idx = None
        for i, s in enumerate(self.snaps):
            if s["tau"] <= tau + 1e-12:
                idx = i
        return idx

    def maybe_capture(self, sim):
        """call after sim steps: takes a snapshot when sim time crosses the next grid point"""
        tau = sim.tau()
        if tau + 1e-12 < self.next_tau:
            return False
        if self.snaps and tau <= self.snaps[-1]["tau"] + 1e-12:
            return False
        self.capture(sim)
        self.next_tau = (math.floor(tau / self.dtau + 1e-9) + 1) * self.dtau
        return True

    def capture(self, sim):
        if not self.ncells:
            self.ncells = sim._n
        sim.update_render_fields()           # g0 up to date with this state
        buf = torch.empty(BYTES_PER_CELL * sim._n, dtype=torch.uint8, device=sim.device)
        sim.snapshot_pack(buf)
        self.snaps.append(dict(tau=sim.tau(), buf=buf, shape=sim.shape, meta=sim.get_state_meta()))
        while len(self.snaps) > self.capacity():
            self._thin()

    def _thin(self):
        """drop every other snapshot (keep first and last), double the spacing"""
        if len(self.snaps) < 3:
            self.snaps = self.snaps[-1:]
            return
        keep = self.snaps[::2]
        if keep[-1] is not self.snaps[-1]:
            keep.append(self.snaps[-1])
        self.snaps = keep
        self.dtau *= 2.0
        self.thinned += 1
        if self.snaps:
            self.next_tau = (math.floor(self.snaps[-1]["tau"] / self.dtau + 1e-9) + 1) * self.dtau

    def restore(self, sim, i):
        s = self.snaps[i]
        if tuple(s["shape"]) != tuple(sim.shape):
            return False
        sim.snapshot_unpack(s["buf"])
        sim.set_state_meta(s["meta"])
        return True

    def truncate_after(self, tau):
        """branch: forget everything later than tau (the sim continues from there with new parameters)"""
        self.snaps = [s for s in self.snaps if s["tau"] <= tau + 1e-12]
        self.next_tau = (math.floor(tau / self.dtau + 1e-9) + 1) * self.dtau

    def status(self):
        n = len(self.snaps)
        if not n:
            return "cache empty"
        return (f"{n} frames  {self.bytes_used()/1e9:.1f}/{self.budget/1e9:.0f} GB  "
                f"every {self.dtau:.4g}{'  (thinned x' + str(2 ** self.thinned) + ')' if self.thinned else ''}")

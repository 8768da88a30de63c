"""Batched simulation: many `Sim` instances of different sizes advanced together on one GPU.

Each batch step is one control launch for all instances, the ionization of every instance
that is due (each keeps its own `it % ion_every` cadence, sim.py:1102), and one persistent
launch per RK2 stage walking a tile work-list spanning every instance, largest first; the
step is replayed as a CUDA graph.  Each instance keeps its own clock, CFL dt, stars and live
parameters, and its results are bit-identical to stepping it alone.
"""
import ctypes as C
import time

from . import _lib
from . import ics as _ics
from .sim import Sim


class BatchSim:
    def __init__(self, sims, graphs=True):
        if not sims:
            raise ValueError("a batch needs at least one Sim")
        self.sims = list(sims)
        for s in self.sims:
            if s.phase != "main" or s._stirring():
                raise NotImplementedError("batched steps are main-phase steps without stirring: step stirred "
                                          "instances alone (Sim.step)")
        if len({s.arith for s in self.sims}) != 1:
            raise ValueError("the instances of a batch must come from one library build (same arith)")
        self._lib = self.sims[0]._lib
        n = len(self.sims)
        for s in self.sims:
            s._push()
        hs = (C.c_void_p * n)(*[s._h.value for s in self.sims])
        ie = (C.c_int * n)(*[int(s.ion_every) for s in self.sims])
        b = C.c_void_p()
        rc = self._lib.nb_batch_create(hs, ie, n, C.byref(b))
        if rc != 0:
            raise _lib.NebulaError(f"nb_batch_create: {_lib.ERRORS.get(rc, rc)}: "
                                   f"{self._lib.nb_batch_last_error(None).decode()}")
        self._b = b
        self.active = [True] * n
        self.set_option("graphs", 1 if graphs else 0)
        self.prof = {}

    def _chk(self, rc, what):
        if rc != 0:
            raise _lib.NebulaError(f"{what}: {_lib.ERRORS.get(rc, rc)}: {self._lib.nb_batch_last_error(self._b).decode()}")

    def set_option(self, key, value):
        keys = {"graphs": 0, "grid": 1, "ray_group": 2}
        self._chk(self._lib.nb_batch_set_option(self._b, keys[key], int(value)), "nb_batch_set_option")

    @property
    def cells(self):
        """cells of the active instances (those a step advances)"""
        return sum(s._n for s, a in zip(self.sims, self.active) if a)

    def set_active(self, active):
        """which instances step (one flag per Sim, in the batch's order): an idle one is left as it
        is, so instances join and leave the stepping set without rebuilding the batch or its graphs"""
        flags = [bool(a) for a in active]
        if len(flags) != len(self.sims):
            raise ValueError(f"one flag per instance ({len(self.sims)}), not {len(flags)}")
        arr = (C.c_int * len(flags))(*[int(a) for a in flags])
        self._chk(self._lib.nb_batch_set_active(self._b, arr, len(flags)), "nb_batch_set_active")
        self.active = flags

    def step(self, k=1, sync=True):
        """advance every active instance k steps (the live parameters / stars of each Sim are pushed
        first)"""
        t0 = time.perf_counter()
        live = [s for s, a in zip(self.sims, self.active) if a]
        for s in live:
            s._push()
            s._clock_fresh = False               # the batch advances the clocks: read them from the device
        self._chk(self._lib.nb_batch_step(self._b, int(k)), "nb_batch_step")
        for s in live:
            s._it += int(k)
            s.version += int(k)
        if sync:
            self.sync()
        self.prof["step"] = self.prof.get("step", 0.0) + time.perf_counter() - t0
        return time.perf_counter() - t0

    def sync(self):
        """wait for the batch's steps (the instances' stream follows the batch's), then check_status"""
        self.sims[0]._sync()
        self.check_status()

    def check_status(self):
        """raise if a batched hydro stage's bounded TMA wait gave up on the device for any instance
        (its fields are incomplete from then on), as a synchronized Sim.step does; step(sync=True)
        calls it after the batch's steps"""
        st = C.c_int()
        bad = []
        for i, s in enumerate(self.sims):
            s._chk(s._lib.nb_device_status(s._h, C.byref(st)), "nb_device_status")
            if st.value & _lib.NB_DEV_TMA_TIMEOUT:
                bad.append(i)
        if bad:
            raise _lib.NebulaError(f"nb_batch_step: NB_ERR_TIMEOUT: a bounded TMA wait in a batched hydro stage "
                                   f"gave up on the device; instances {bad} have incomplete fields")

    def launches(self):
        v = C.c_longlong()
        self._chk(self._lib.nb_batch_counters(self._b, C.byref(v)), "nb_batch_counters")
        return int(v.value)

    def close(self):
        if getattr(self, "_b", None):
            self.sims[0]._sync()
            self._lib.nb_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_workload(n=32, seed=7, device="cuda", lo=64, hi=192, **sim_kw):
    """the batched workload as a list of Sims (see ics.batch_scenes)"""
    sims = []
    for ic in _ics.batch_scenes(n=n, seed=seed, device=device, lo=lo, hi=hi):
        sims.append(Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"],
                                   ic["jkinds"], ic["P"], mom=ic["mom"], device=device, **sim_kw))
    return sims

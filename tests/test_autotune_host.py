"""The autotuner's host logic on a fake instance: it keeps the fastest candidate of each knob,
leaves the state as it found it, and when a candidate run fails it puts the original launch
shapes back, restores the state and switches the kernel timers off.  No GPU."""
import ctypes as C

import pytest

torch = pytest.importorskip("torch")
autotune = pytest.importorskip("nebulaviewer_gb300.autotune")
from nebulaviewer_gb300 import _lib  # noqa: E402


class FakeLib:
    def __init__(self, sim):
        self.sim = sim
        self.tuning = {i: 0 for i in _lib.TUNE.values()}
        self.profiling = 0

    def nb_get_tuning(self, h, key, out):
        out._obj.value = self.tuning[key]
        return 0

    def nb_set_tuning(self, h, key, value):
        self.tuning[key] = value
        return 0

    def nb_profile(self, h, on):
        self.profiling = on
        return 0

    def nb_profile_read(self, h, ms, n):
        # the hydro stages take (chunk_i - 24)^2 + 1 ms per launch: 24 is the fastest depth
        c = self.tuning[_lib.TUNE["chunk_i"]]
        for k in ("stage1", "stage2"):
            i = _lib.PROF_KINDS.index(k)
            ms[i] = float((c - 24) ** 2 + 1)
            n[i] = 1
        return 0


class Shape:
    def __init__(self, *s):
        self.shape = s


class FakeSim:
    def __init__(self, fail_at_chunk=None):
        self.shape, self.stars, self.P, self.arith = (8, 8, 8), [], {"solver": "hll"}, "exact"
        self.rfront, self.att = Shape(4, 4), Shape(2, 2, 2)
        self._h = C.c_void_p(1)
        self._lib = FakeLib(self)
        for k in ("rho", "mx", "my", "mz", "xi", "dfront", "g0"):
            setattr(self, "_" + k, torch.zeros(8))
        self._it, self.version, self.meta = 5, 5, {"t": 1.0}
        self.fail_at_chunk = fail_at_chunk

    def _sync(self):
        pass

    def get_state_meta(self):
        return dict(self.meta)

    def set_state_meta(self, m):
        self.meta = dict(m)

    def step(self, k, sync=True):
        if self._lib.tuning[_lib.TUNE["chunk_i"]] == self.fail_at_chunk:
            raise RuntimeError("injected step failure")
        self._rho += 1.0                              # a step changes the state
        self._it += k
        self.version += k
        self.meta["t"] += 0.5


def test_keeps_the_fastest_candidate_and_the_state():
    s = FakeSim()
    res = autotune.autotune(s, knobs=["chunk_i"], use_cache=False)
    assert res["chunk_i"][0] == 24 and autotune.get(s, "chunk_i") == 24
    assert torch.equal(s._rho, torch.zeros(8)) and s._it == 5 and s.version == 5 and s.meta == {"t": 1.0}
    assert s._lib.profiling == 0


def test_a_failed_candidate_restores_shapes_state_and_timers():
    s = FakeSim(fail_at_chunk=24)
    autotune.put(s, "chunk_i", 20)
    with pytest.raises(RuntimeError, match="injected"):
        autotune.autotune(s, knobs=["chunk_i"], use_cache=False)
    assert autotune.get(s, "chunk_i") == 20
    assert torch.equal(s._rho, torch.zeros(8)) and s._it == 5 and s.version == 5 and s.meta == {"t": 1.0}
    assert s._lib.profiling == 0

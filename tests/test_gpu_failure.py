"""The bounded-wait failure path on the GPU, without faulting it.

The reference reads the CFL max speed back to the host every step (sim.py:1009-1012), so a
stuck step would block the caller.  Here the step never waits for the host, and every device-side
wait of the hydro stages (the mbarrier a tile's TMA copies complete) is bounded: when it runs
out, the stage records NB_DEV_TMA_TIMEOUT in the instance's device status word, writes nothing
more and returns.  These tests make that wait run out on purpose in the one allowed form -- a
short poll limit (64 polls) and a stage that issues no tile copy at all, so nothing is left in
flight -- and check that the failure reaches the caller: nb_device_status has the bit,
nb_get_clock and nb_peek_clock return NB_ERR_TIMEOUT, a synchronized Sim.step and BatchSim.step
raise, and the CUDA context stays usable for a fresh instance.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

NB_ERR_TIMEOUT = -5


@pytest.fixture(scope="module")
def nb():
    from nebulaviewer_gb300 import build
    build.build(verbose=False)
    from nebulaviewer_gb300 import _lib, autotune, ics, sim
    assert torch.cuda.is_available(), "the gpu tests need a CUDA device"
    return _lib, autotune, ics, sim


def _sheet(nb, res=32, seed=3, arith=None):
    _lib, _, ics, S = nb
    ic = ics.sheet(res=res, seed=seed, nstars=2)
    return S.Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                            ic["P"], mom=ic["mom"], rays=(32, 64), fuv_grid=(8, 8, 16), arith=arith)


def _status(sim):
    st = C.c_int()
    assert sim._lib.nb_device_status(sim._h, C.byref(st)) == 0
    return st.value


@pytest.mark.parametrize("arith", ("exact", "fast"))
def test_expired_hydro_wait_is_reported(nb, arith):
    _lib, at, _, S = nb
    sim = _sheet(nb, arith=arith)
    sim.step(1)                                   # a normal step first: no status bit
    assert _status(sim) == 0
    rho0 = sim._rho.clone()
    at.put(sim, "wait_limit", 64)
    at.put(sim, "stall_test", 1)
    assert at.get(sim, "wait_limit") == 64 and at.get(sim, "stall_test") == 1
    with pytest.raises(_lib.NebulaError, match="NB_ERR_TIMEOUT"):
        sim.step(1)                               # synchronized: reads the clock copy and raises
    assert _status(sim) & _lib.NB_DEV_TMA_TIMEOUT
    c = _lib.NbClock()
    assert sim._lib.nb_get_clock(sim._h, C.byref(c)) == NB_ERR_TIMEOUT
    assert sim._lib.nb_peek_clock(sim._h, C.byref(c)) == NB_ERR_TIMEOUT
    assert b"TMA wait" in sim._lib.nb_last_error(sim._h)
    # stage 2 wrote nothing over U^n either: the density is the last good step's
    assert torch.equal(sim._rho, rho0)
    sim.close()
    # the context is still usable: a fresh instance steps and matches a second fresh one bit for bit
    a, b = _sheet(nb, arith=arith), _sheet(nb, arith=arith)
    a.step(3)
    b.step(3)
    assert _status(a) == 0 and torch.equal(a._rho, b._rho) and torch.equal(a._xi, b._xi)
    a.close()
    b.close()


def test_limit_and_switch_are_checked(nb):
    _lib, at, _, _ = nb
    sim = _sheet(nb, res=16)
    for key, bad in (("wait_limit", 0), ("wait_limit", (1 << 22) + 1), ("stall_test", 2)):
        with pytest.raises(_lib.NebulaError, match="NB_ERR_ARG"):
            at.put(sim, key, bad)
    assert at.get(sim, "wait_limit") == 1 << 22 and at.get(sim, "stall_test") == 0
    sim.close()


def test_expired_wait_in_a_batch_is_reported(nb):
    """a batched hydro stage: the instance whose copies never come is flagged, the batch step
    raises after synchronizing, and an instance that only the other blocks stepped stays right"""
    _lib, at, _, S = nb
    from nebulaviewer_gb300.batch import BatchSim
    good, bad = _sheet(nb, res=48, seed=4, arith="exact"), _sheet(nb, res=32, seed=5, arith="exact")
    alone = _sheet(nb, res=48, seed=4, arith="exact")
    at.put(bad, "wait_limit", 64)
    at.put(bad, "stall_test", 1)
    B = BatchSim([good, bad], graphs=False)
    with pytest.raises(_lib.NebulaError, match="NB_ERR_TIMEOUT"):
        B.step(1)
    assert _status(bad) & _lib.NB_DEV_TMA_TIMEOUT
    # a block that failed leaves the rest of its work undone and flags the instance of each item it
    # skips; the good instance is either flagged or stepped exactly as alone
    alone.step(1)
    if not _status(good) & _lib.NB_DEV_TMA_TIMEOUT:
        assert np.array_equal(good.rho.numpy().view(np.uint32), alone.rho.numpy().view(np.uint32))
    B.close()
    for s in (good, bad, alone):
        s.close()

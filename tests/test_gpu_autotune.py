"""The launch-shape autotuner leaves the instance's state and clock unchanged and keeps the
hydro result independent of the shapes it picks."""
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_autotune_preserves_state_and_hydro_result():
    from nebulaviewer_gb300 import autotune, build, ics
    from nebulaviewer_gb300.sim import Sim
    build.build(verbose=False)
    ic = ics.sheet(res=48, seed=8, nstars=3, device="cuda", shape=(48, 40, 64))

    def make():
        return Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                              ic["P"], mom=ic["mom"], rays=(64, 128), fuv_grid=(16, 16, 32))
    a = make()
    a.step(2)
    before = [t.clone() for t in (a._rho, a._mx, a._xi, a._dfront)] + [a.t, a.it]
    res = autotune.autotune(a, use_cache=False)
    assert set(res) == set(autotune.CANDIDATES)
    after = [t.clone() for t in (a._rho, a._mx, a._xi, a._dfront)] + [a.t, a.it]
    for x, y in zip(before[:4], after[:4]):
        assert torch.equal(x, y)
    assert before[4:] == after[4:]
    # with the same ray lanes, the hydro shapes picked do not change the result
    b = make()
    b.step(2)
    autotune.put(b, "ray_group", autotune.get(a, "ray_group"))
    autotune.put(b, "fuv_group", autotune.get(a, "fuv_group"))
    a.step(4)
    b.step(4)
    assert torch.equal(a._rho, b._rho) and torch.equal(a._xi, b._xi) and a.t == b.t
    a.close()
    b.close()

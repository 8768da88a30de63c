"""Batched instances (persistent stage kernels over a multi-instance tile work-list, batched
control and ionization, CUDA graphs): every instance's result equals stepping it alone, whatever
the batch composition, cadence mix or graph use -- bit for bit with the exact build, within the
path's tolerance (rel-L_inf 1e-5) with the fast build, whose batched and single-instance
kernels may contract multiply-adds differently."""
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nb():
    from nebulaviewer_gb300 import build
    build.build(verbose=False)
    from nebulaviewer_gb300 import batch, ics, sim
    assert torch.cuda.is_available()
    return batch, ics, sim


SHAPES = [(24, 32, 40), (32, 32, 32), (16, 48, 24), (40, 24, 32)]


def scenes(ics):
    out = []
    for m, shape in enumerate(SHAPES):
        if m % 2 == 0:
            out.append(ics.torus(seed=10 + m, device="cuda", shape=shape, nstars=1 + m))
        else:
            out.append(ics.sheet(res=min(shape), seed=20 + m, nstars=2 + m, device="cuda", shape=shape))
    return out


def make(S, ic, ion_every=None, arith=None):
    return S.Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                            ic["P"], mom=ic["mom"], rays=(64, 128), fuv_grid=(16, 16, 32), ion_every=ion_every,
                            arith=arith)


def state(s):
    torch.cuda.synchronize()
    c = s._clock()
    return [t.clone() for t in (s._rho, s._mx, s._my, s._mz, s._xi, s._dfront)] + [c.t, c.dt, c.it]


def same(a, b, exact=True):
    for x, y in zip(a[:6], b[:6]):
        if exact:
            assert torch.equal(x, y)
        elif x.dtype == torch.float16:
            # an fp16 field (dfront): the fast build's last-bit float32 differences may cross an
            # fp16 rounding boundary; within 2 fp16 ulps (2^-9 relative, above the subnormals)
            xd, yd = x.double(), y.double()
            assert bool(((xd - yd).abs() <= 2.0 ** -9 * torch.clamp(yd.abs(), min=2.0 ** -14)).all())
        else:
            xd, yd = x.double(), y.double()
            assert float((xd - yd).abs().max()) <= 1e-5 * max(float(yd.abs().max()), 1e-30)
    if exact:
        assert a[6:] == b[6:]
    else:
        assert a[8] == b[8] and abs(a[6] - b[6]) <= 1e-6 * abs(b[6])


@pytest.mark.parametrize("arith", ("exact", "fast"))
@pytest.mark.parametrize("cadence,graphs", (("lockstep", True), ("lockstep", False), ("mixed", True)))
def test_batch_bit_identical_to_alone(nb, cadence, graphs, arith):
    batch, ics, S = nb
    ics_list = scenes(ics)
    ie = [None] * 4 if cadence == "lockstep" else [2, 3, 5, 1]
    steps = 7
    alone = []
    for ic, e in zip(ics_list, ie):
        s = make(S, ic, e, arith)
        s.step(steps)
        alone.append(state(s))
        s.close()
    sims = [make(S, ic, e, arith) for ic, e in zip(ics_list, ie)]
    B = batch.BatchSim(sims, graphs=graphs)
    B.step(3)
    B.step(steps - 3)
    for s, ref in zip(sims, alone):
        same(state(s), ref, arith == "exact")
    assert B.launches() > 0
    B.close()
    for s in sims:
        s.close()


def test_batch_instances_remain_usable_alone(nb):
    """a batched instance can be stepped and rendered on its own between batch steps"""
    batch, ics, S = nb
    ic = scenes(ics)
    a = [make(S, x, arith="exact") for x in ic[:2]]
    b = [make(S, x, arith="exact") for x in ic[:2]]
    B = batch.BatchSim(a)
    B.step(2)
    a[0].step(1)
    B.step(2)
    for s in b:
        s.step(2)
    b[0].step(1)
    for s in b:
        s.step(2)
    for x, y in zip(a, b):
        same(state(x), state(y))
    a[0].update_render_fields(force=True)
    b[0].update_render_fields(force=True)
    assert torch.equal(a[0]._g0, b[0]._g0)
    B.close()


@pytest.mark.parametrize("graphs", (True, False))
def test_idle_slots_are_left_untouched(nb, graphs):
    """a batch whose slots go idle and active again (nb_batch_set_active, as the server's pool does):
    an idle instance keeps every bit of its state and clock; an active one ends exactly where
    stepping it alone ends, across ionizing steps where only some active instances ionize"""
    batch, ics, S = nb
    ics_list = scenes(ics)
    ie = [2, 3, 5, 1]
    sims = [make(S, ic, e, "exact") for ic, e in zip(ics_list, ie)]
    alone = [make(S, ic, e, "exact") for ic, e in zip(ics_list, ie)]
    B = batch.BatchSim(sims, graphs=graphs)
    plan = [([1, 0, 1, 1], 3), ([0, 1, 0, 1], 2), ([1, 1, 1, 1], 2), ([0, 0, 0, 0], 1), ([0, 0, 1, 0], 4)]
    for flags, k in plan:
        before = [state(s) for s in sims]
        B.set_active(flags)
        B.step(k)
        for s, a, f, prev in zip(sims, alone, flags, before):
            if f:
                a.step(k)
                same(state(s), state(a))
            else:
                same(state(s), prev)
    assert B.cells == sims[2]._n
    B.close()
    for s in sims + alone:
        s.close()


def test_footprint_is_known_before_allocation_and_matches_the_device(nb):
    """Sim.footprint (fields + nb_instance_bytes of the live handle) equals the estimate made from the
    description alone before anything is allocated, and the device memory the instance takes"""
    _, ics, S = nb
    from nebulaviewer_gb300.sim import footprint_bytes
    ic = ics.sheet(res=160, nstars=6, seed=8, device="cuda")
    P = dict(ic["P"])
    from nebulaviewer_gb300.params import make_params
    est = footprint_bytes(ic["shape"], ic["dx"], make_params(base=P), (512, 1024), (128, 128, 256), True, 6)
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    free0 = torch.cuda.mem_get_info()[0]
    s = S.Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"], P,
                         mom=ic["mom"])
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    used = free0 - torch.cuda.mem_get_info()[0]
    fp = s.footprint()
    assert fp == est
    assert abs(used - fp) <= 0.03 * fp + (32 << 20), (used, fp)
    assert fp > 40 * s._n + 100e6                     # the FUV and front tables are most of it here
    s.close()


def test_batch_beyond_the_parameter_records(nb):
    """a batch of 130 instances: more than the 128 whose stage records the persistent kernel takes as
    its parameter, so it reads them from device memory (the other form of the kernel); every
    instance still ends exactly where stepping it alone ends, with a slot idle for part of it"""
    batch, ics, S = nb
    shapes = [(16, 16, 16), (16, 24, 20), (24, 16, 12)]
    ics_list = [ics.torus(seed=100 + m, device="cuda", shape=shapes[m % 3], nstars=1) if m % 2 == 0 else
                ics.sheet(res=16, seed=200 + m, nstars=1, device="cuda", shape=shapes[m % 3]) for m in range(130)]

    def mk(ic):
        return S.Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                                ic["P"], mom=ic["mom"], rays=(16, 32), fuv_grid=(8, 8, 16), arith="exact")

    sims = [mk(ic) for ic in ics_list]
    B = batch.BatchSim(sims)
    flags = [1] * 130
    flags[7] = 0
    B.set_active(flags)
    B.step(2)
    B.set_active([1] * 130)
    B.step(2)
    for m, (s, ic) in enumerate(zip(sims, ics_list)):
        a = mk(ic)
        a.step(2 if m == 7 else 4)
        same(state(s), state(a))
        a.close()
    B.close()
    for s in sims:
        s.close()

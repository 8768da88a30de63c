"""GPU parity of the turbulent stirring (nebula3d.py:165-179 drive; sim.py:1030-1059 the
stirring phase and its end; sim.py:1110-1111 main-phase stirring), through libnebula.so.

Tolerances: with the exact build the drive and add_torus kernels are bit-identical to the
reference's and a stirring-phase step (no rays) is bit-identical to the reference Sim's
(fields and clocks); once the first ionization ran, and for the fast build throughout, the
tolerances of the other end-to-end tests apply (state rel-L_inf 1e-5 per step, xi 1e-4,
ionized mask within 0.1% of cells).
"""
import ctypes as C

import numpy as np
import pytest

from conftest import bits_equal, golden, golden_sim, rel_linf

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nb():
    from nebulaviewer_gb300 import build
    build.build(verbose=False)
    from nebulaviewer_gb300 import _lib, sim
    assert torch.cuda.is_available(), "the gpu tests need a CUDA device"
    return _lib, sim


def t32(a):
    return torch.as_tensor(np.ascontiguousarray(a, np.float32), device="cuda")


def _plain_sim(S, rho, mom, dx, stir_grid, **P):
    P = dict(dict(ci_over_cn=12.0, pre_corr=0.06), **P)
    return S.Sim.from_state(rho.shape, dx, rho, [], [], [], [], P, mom=list(mom), start_main=False,
                            stir_grid=stir_grid, rays=(4, 8), fuv_grid=(4, 4, 8), arith="exact")


@pytest.mark.parametrize("tag", ("in", "out"))
def test_drive_kernel_bit_identical_to_reference(nb, tag):
    _, S = nb
    z = golden("stir.npz")
    A, B = z[f"d_{tag}_A"], z[f"d_{tag}_B"]
    blend, amp, dt, dx, dxs = (float(v) for v in z[f"d_{tag}_scalars"])
    sim = _plain_sim(S, z["d_rho"], z["d_mom"], dx, (A.shape[1:], dxs))
    sim._drive_new(0.0, fields=[A, B])                     # sets the forcing grid of the handle
    fa, fb = t32(A), t32(B)
    sim._chk(sim._lib.nb_drive_step(sim._h, C.c_void_p(fa.data_ptr()), C.c_void_p(fb.data_ptr()), blend, amp, dt),
             "nb_drive_step")
    torch.cuda.synchronize()
    for k, ref in zip(("mx", "my", "mz"), z[f"d_{tag}_out"]):
        assert bits_equal(getattr(sim, k).numpy(), ref), k
    assert bits_equal(sim.rho.numpy(), z["d_rho"])
    sim.close()


def test_add_torus_and_mach_sums(nb):
    _, S = nb
    z = golden("stir.npz")
    sim = _plain_sim(S, z["d_rho"], z["d_mom"], 0.125, ((4, 4, 4), 0.75))
    tq = t32(z["a_torus"])
    sim._chk(sim._lib.nb_add_torus(sim._h, C.c_void_p(tq.data_ptr())), "nb_add_torus")
    torch.cuda.synchronize()
    assert bits_equal(sim.rho.numpy(), z["a_rho"])
    for k, ref in zip(("mx", "my", "mz"), z["a_mom"]):
        assert bits_equal(getattr(sim, k).numpy(), ref), k
    s = (C.c_double * 2)()
    sim._chk(sim._lib.nb_mach_sums(sim._h, s), "nb_mach_sums")
    r = z["a_rho"]
    m2 = (z["a_mom"][0] * z["a_mom"][0] + z["a_mom"][1] * z["a_mom"][1] + z["a_mom"][2] * z["a_mom"][2]) / r
    assert abs(s[0] - m2.astype(np.float64).sum()) <= 1e-12 * abs(s[0])
    assert abs(s[1] - r.astype(np.float64).sum()) <= 1e-12 * abs(s[1])
    sim.close()


@pytest.mark.parametrize("arith", ("exact", "fast"))
def test_sim_through_stirring_phase_matches_reference_sim(nb, arith):
    """the drop-in Sim against the reference Sim: 9 stirring-phase steps with a forcing swap, the
    step that ends the phase (torus, Mach number, first ionization), main-phase stirring with
    another swap"""
    _, S = nb
    d, m = golden_sim("bipolar_pre")
    sim = S.Sim.from_state(m["shape"], m["dx"], d["rho_ic"], m["stars"], m["kinds"], m["jets"], m["jkinds"], m["P"],
                           rays=m["rays"], fuv_grid=m["fuv"], ion_every=m["ion_every"], fast=True, torus=d["torus"],
                           stir_fields=list(d["fields"]), stir_grid=(m["sshape"], m["dxs"]), arith=arith)
    assert sim.phase == "pre"
    ionized = arith != "exact"           # the fast build: tolerances from the first step
    for n, st in enumerate(m["steps"]):
        sim.step(1)
        c = sim._clock()
        assert sim.phase == st["phase"], n
        drv = sim.drv
        assert (drv is None) == (st["clock"] is None)
        if drv is not None:
            assert drv["clock"] == pytest.approx(st["clock"], rel=1e-6, abs=1e-12), n
        if not ionized:
            assert c.tp == st["tp"] and c.ip == st["ip"], n
            assert c.t == st["t"] and c.dt == st["dt"], n
            if st["phase"] == "pre":
                for k in ("rho", "mx", "my", "mz", "xi"):
                    assert bits_equal(getattr(sim, k).numpy(), d[f"s{n + 1}_{k}"]), (n, k)
        else:
            assert abs(c.tp - st["tp"]) <= 1e-6 * st["tp"] and c.ip == st["ip"], n
        if st["phase"] == "main" or ionized:
            ionized = True
            assert abs(sim.t - st["t"]) <= 1e-6 * max(st["t"], 1e-30)
            for k in ("rho", "mx", "my", "mz"):
                assert rel_linf(getattr(sim, k).numpy(), d[f"s{n + 1}_{k}"]) < 1e-5, (n, k)
            x = sim.xi.numpy()
            assert np.abs(x - d[f"s{n + 1}_xi"]).max() < 1e-4
            assert np.mean((x > 0.5) != (d[f"s{n + 1}_xi"] > 0.5)) <= 1e-3
        if st["mach"] is not None:
            assert abs(sim.mach - st["mach"]) <= 1e-5 * st["mach"]
    sim.close()


def _stirred_pair(nb, res=16, rays=(64, 128), fuv=(16, 16, 32), n_fields=60, arith="exact"):
    import oracle as O
    from nebulaviewer_gb300 import ics, stir
    from nebulaviewer_gb300.params import make_params, sound_speeds
    _, S = nb
    ic = ics.torus_stirred(res=res)
    g = S.Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                         ic["P"], rays=rays, fuv_grid=fuv, torus=ic["torus"], arith=arith)
    P = make_params(base=ic["P"])
    cn2, ci2, vmax = sound_speeds(P)
    rng = np.random.default_rng(P["seed"])               # the Sim's own forcing stream, drawn again
    fields = [np.stack(stir.solenoidal(g.sshape, rng, 1.0, P["pre_kmax"])) for _ in range(n_fields)]
    o = O.OracleSim(ic["shape"], ic["dx"], ic["rho"].numpy(), ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"], P,
                    rays=rays, fuv_grid=fuv, cn2=cn2, ci2=ci2, vmax=vmax, torus=ic["torus"].numpy(),
                    stir_fields=fields, stir_grid=(g.sshape, g.dxs))
    return g, o


@pytest.mark.parametrize("arith", ("exact", "fast"))
def test_stirred_torus_against_oracle(nb, arith):
    """torus_stirred at 32^3: the stirring phase (forcing drawn by the Sim's own generator) bit for
    bit against the oracle (exact build; the fast build within tolerance), then 30 main-phase steps
    with stirring within tolerance"""
    g, o = _stirred_pair(nb, arith=arith)
    n = 0
    while o.phase == "pre":
        g.step(1)
        o.step(1)
        n += 1
        assert g.phase == o.phase
        if o.phase == "pre" and arith == "exact":
            for k in ("rho", "mx", "my", "mz"):
                assert bits_equal(getattr(g, k).numpy(), getattr(o, k)), (n, k)
            assert g.tp == o.tp
        elif o.phase == "pre":
            for k in ("rho", "mx", "my", "mz"):
                assert rel_linf(getattr(g, k).numpy(), getattr(o, k)) < 1e-5 * n, (n, k)
    assert 5 < n < 40 and abs(g.mach - o.mach) <= 1e-5 * o.mach
    for s in range(30):
        g.step(1)
        o.step(1)
        if s < 3:
            for k in ("rho", "mx", "my", "mz"):
                assert rel_linf(getattr(g, k).numpy(), getattr(o, k)) < 1e-5, (s, k)
    assert abs(g.t - o.t) <= 1e-4 * o.t
    for k in ("rho", "mx", "my", "mz"):
        assert rel_linf(getattr(g, k).numpy(), getattr(o, k)) < 1e-3, k
    assert g.drv["clock"] == pytest.approx(o.drv["clock"], rel=1e-3, abs=1e-9)
    g.close()


@pytest.mark.parametrize("arith", ("exact", "fast"))
def test_chunked_steps_equal_single_steps_and_meta_roundtrip(nb, arith):
    """step(k) (device-side clock, forcing ring refilled in chunks across the end of the phase)
    is bit-identical to k x step(1); a state saved in the stirring phase (fields + meta with the
    forcing and the Generator state) resumes to the same bits"""
    from nebulaviewer_gb300 import ics
    _, S = nb
    ic = ics.torus_stirred(res=16)
    mk = lambda: S.Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"],  # noqa
                                  ic["jkinds"], ic["P"], rays=(64, 128), fuv_grid=(16, 16, 32), torus=ic["torus"],
                                  arith=arith)
    a, b = mk(), mk()
    for _ in range(70):
        a.step(1)
    b.step(70)
    for k in ("rho", "mx", "my", "mz", "xi"):
        assert bits_equal(getattr(a, k).numpy(), getattr(b, k).numpy()), k
    ca, cb = a._clock(), b._clock()
    assert (ca.t, ca.tp, ca.it, ca.ip) == (cb.t, cb.tp, cb.it, cb.ip)
    assert a.phase == b.phase == "main" and a.drv["clock"] == b.drv["clock"]
    a.close()
    b.close()
    # save after 5 stirring-phase steps, run 40 more, restore, run 40 again
    c = mk()
    c.step(5)
    saved = {k: getattr(c, "_" + k).clone() for k in ("rho", "mx", "my", "mz", "xi", "dfront", "g0")}
    meta = c.get_state_meta()
    assert meta["phase"] == "pre" and meta["drv"] is not None
    c.step(40)
    first = {k: getattr(c, k).numpy() for k in ("rho", "mx", "my", "mz", "xi")}
    for k, v in saved.items():
        getattr(c, "_" + k).copy_(v)
    c.set_state_meta(meta)
    c.step(40)
    for k, v in first.items():
        assert bits_equal(getattr(c, k).numpy(), v), k
    c.close()


def test_batch_refuses_stirred_instances(nb):
    from nebulaviewer_gb300 import ics
    from nebulaviewer_gb300.batch import BatchSim
    _, S = nb
    ic = ics.torus_stirred(res=8)
    s = S.Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                         ic["P"], rays=(16, 32), fuv_grid=(8, 8, 16), torus=ic["torus"])
    with pytest.raises(NotImplementedError):
        BatchSim([s])
    s.close()

"""GPU parity: the sm_103a kernels (through libnebula.so's C ABI) against
  * the golden fixtures made from the reference's own kernels and Sim driver,
  * the CPU oracle on seeded inputs,
  * size-independent properties at the benchmark size (256^3).

Both library builds are tested: "exact" (libnebula.so) where the assertions are bit for bit,
"exact" and "fast" (libnebula_fast.so: FMA, approximate division / square root) wherever the
path's tolerances apply.

Tolerances (stated by the specification of this path):
  hydro stage        bit-identical to the reference kernels (no fused multiply-add, IEEE
                     division / sqrt, the reference's operation order);
  one full step      FP32 fields within rel-L_inf 1e-5; 1e-3 after 100 steps;
  ionization         xi within 1e-4, ionized mask (xi > 0.5) identical except <= 0.1% of
                     cells (ray sums are scans, and CUDA's atan2f/expf differ from the C
                     library's by a few ulps);
  fp16 fields        within 2 fp16 ulps.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import bits_equal, golden_sim, rel_linf

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
ARITH = ("exact", "fast")


@pytest.fixture(scope="module")
def nb():
    from nebulaviewer_gb300 import build
    build.build(verbose=False)
    from nebulaviewer_gb300 import _lib, sim
    assert torch.cuda.is_available(), "the gpu tests need a CUDA device"
    return _lib, sim


def t32(a):
    return torch.as_tensor(np.ascontiguousarray(a, np.float32), device="cuda")


def kernel_sim(nb, d, P_extra=None, rays=(6, 12), fuv=(5, 4, 8), fast=True, rho=None, stars=None, kinds=None,
               jets=None, jkinds=None, arith="exact"):
    _lib, S = nb
    dx = float(d["k_scalars"][0])
    rho = d["k_rho"] if rho is None else rho
    P = dict(ci_over_cn=12.0, floor=2e-3, cfl=0.3, solver="hll", limiter="minmod", q_ramp=0.0, q_main=1.0,
             wind=0.5, jet=3.0, jet_proto=2.0, jet_r=0.3, jet_angle=30.0, kappa_fuv=10.0)
    P.update(P_extra or {})
    if stars is None:
        ks, kj = d["k_stars"], d["k_jets"]
        stars = [(float(s[0]), float(s[1]), float(s[2]), float(s[3]), 0.0) for s in ks]
        kinds = ["abs"] * 3
        jets = [tuple(float(v) for v in j[:3]) for j in kj]
        jkinds = ["jet", "none", "proto"]
    return S.Sim.from_state(rho.shape, dx, rho, stars, kinds, jets, jkinds, P, mom=None, rays=rays, fuv_grid=fuv,
                            fast=fast, start_main=False, arith=arith)


HYDRO = (("rus", "rusanov", "minmod"), ("hll0", "hll", "minmod"), ("hll1", "hll", "vanleer"), ("hll2", "hll", "mc"))


@pytest.mark.parametrize("name,solver,lim", HYDRO)
def test_hydro_stage_bit_identical_to_reference_kernels(nb, kernels_npz, name, solver, lim):
    _lib, _ = nb
    d = kernels_npz
    sim = kernel_sim(nb, d, dict(solver=solver, limiter=lim))
    dt, pulse = float(np.float32(d["k_scalars"][9])), float(np.float32(d["k_scalars"][7]))
    U = [t32(d["k_rho"])] + [t32(m) for m in d["k_mom"]]
    sim._xi.copy_(t32(d["k_xi"]))
    o1 = [torch.zeros_like(U[0]) for _ in range(4)]
    o2 = [torch.zeros_like(U[0]) for _ in range(4)]
    P = lambda ts: _lib.f4([t.data_ptr() for t in ts])  # noqa: E731
    _lib.check(sim._lib.nb_hydro_stage(sim._h, P(U), P(U), P(o1), 0.0, 1.0, dt, pulse), sim._h, "stage 1")
    _lib.check(sim._lib.nb_hydro_stage(sim._h, P(o1), P(U), P(o2), 0.5, 0.5, dt, pulse), sim._h, "stage 2")
    torch.cuda.synchronize()
    assert bits_equal(torch.stack(o1).cpu().numpy(), d[f"k_{name}_s1"])
    assert bits_equal(torch.stack(o2).cpu().numpy(), d[f"k_{name}_s2"])
    # stage 2 in place over U^n (sim.py:1026-1028) gives the same bits
    _lib.check(sim._lib.nb_hydro_stage(sim._h, P(o1), P(U), P(U), 0.5, 0.5, dt, pulse), sim._h, "stage 2 in place")
    torch.cuda.synchronize()
    assert bits_equal(torch.stack(U).cpu().numpy(), d[f"k_{name}_s2"])
    sim.close()


def test_max_speed_matches_reference(nb, kernels_npz):
    d = kernels_npz
    sim = kernel_sim(nb, d)
    sim._mx.copy_(t32(d["k_mom"][0]))
    sim._my.copy_(t32(d["k_mom"][1]))
    sim._mz.copy_(t32(d["k_mom"][2]))
    sim._xi.copy_(t32(d["k_xi"]))
    v = C.c_float()
    _lib = nb[0]
    _lib.check(sim._lib.nb_max_speed(sim._h, C.byref(v)), sim._h, "max_speed")
    assert np.float32(v.value) == d["k_smax"][0]
    sim.close()


@pytest.mark.parametrize("arith", ARITH)
@pytest.mark.parametrize("tag,fast", (("full", True), ("half", False)))
def test_ionize_matches_reference_kernels(nb, kernels_npz, tag, fast, arith):
    d = kernels_npz
    rs = d["r_stars"]
    stars = [(float(s[0]), float(s[1]), float(s[2]), float(s[3]), 0.0) for s in rs]
    sim = kernel_sim(nb, d, dict(q_main=0.1, wind=0.0), rho=d["r_rho"], fast=fast, stars=stars, kinds=["abs"] * 3,
                     jets=[(0.0, 0.0, 1.0)] * 3, jkinds=["none"] * 3, arith=arith)
    _lib = nb[0]
    # the ray kernel alone, one star at a time
    rf = torch.zeros((6, 12), device="cuda")
    for s, st in enumerate(rs):
        xyz = (C.c_double * 3)(*[float(v) for v in st[:3]])
        _lib.check(sim._lib.nb_cast_rays(sim._h, xyz, float(st[3]), C.c_void_p(rf.data_ptr())), sim._h, "rays")
        assert rel_linf(rf.cpu().numpy(), d[f"r_{tag}_rfront"][s]) < 1e-5
    sim.ionize()
    torch.cuda.synchronize()
    xi = sim.xi.numpy()
    assert np.abs(xi - d[f"r_{tag}_xi"]).max() < 1e-4
    assert np.mean((xi > 0.5) != (d[f"r_{tag}_xi"] > 0.5)) <= 1e-3
    df = sim.dfront.numpy().astype(np.float32)
    ref = d[f"r_{tag}_df"].astype(np.float16).astype(np.float32)
    # exact: 2 fp16 ulps; fast: plus rel-L_inf 1e-5 of the finite dfront values (the approximate
    # square root moves r - rf by a few 1e-6 at cells on the front, where dfront is near 0)
    fin = np.abs(ref[ref < 500.0]).max()
    slack = 1e-6 if arith == "exact" else 1e-5 * fin
    assert np.all(np.abs(df - ref) <= 2 * np.abs(ref) * 2.0 ** -10 + slack)
    if tag == "full":
        sim.fuv_field()
        torch.cuda.synchronize()
        g0 = sim.g0.numpy().astype(np.float32)
        assert rel_linf(g0, d["f_g0"]) < 2e-3
        # the FUV ray kernel alone (reference layout [b][iu][ip])
        fnr, fnu, fnp = (int(v) for v in d["f_meta"][:3])
        att = torch.zeros((fnr, fnu, fnp), device="cuda")
        for s, st in enumerate(rs):
            xyz = (C.c_double * 3)(*[float(v) for v in st[:3]])
            _lib.check(sim._lib.nb_cast_fuv(sim._h, xyz, C.c_void_p(att.data_ptr())), sim._h, "fuv rays")
            assert np.abs(att.cpu().numpy() - d["f_att"][s]).max() < 1e-4
    sim.close()


@pytest.mark.parametrize("arith", ARITH)
@pytest.mark.parametrize("name", ("bubbles", "bipolar", "cliff"))
def test_sim_matches_reference_sim_end_to_end(nb, name, arith):
    """the drop-in Sim against the reference Sim run by its own driver code"""
    d, m = golden_sim(name)
    _, S = nb
    sim = S.Sim.from_state(m["shape"], m["dx"], d["s0_rho"], m["stars"], m["kinds"], m["jets"], m["jkinds"], m["P"],
                           rays=m["rays"], fuv_grid=m["fuv"], ion_every=m["ion_every"], fast=m["fast"], arith=arith)
    torch.cuda.synchronize()
    assert np.abs(sim.xi.numpy() - d["s0_xi"]).max() < 1e-4
    n = 1
    while f"s{n}_rho" in d.files:
        sim.dt_cap = m["dt_caps"][n - 1]
        sim.step(1)
        assert abs(sim.t - float(d[f"s{n}_t"])) <= 1e-6 * abs(float(d[f"s{n}_t"]))
        for k in ("rho", "mx", "my", "mz"):
            assert rel_linf(getattr(sim, k).numpy(), d[f"s{n}_{k}"]) < 1e-5, (n, k)
        x = sim.xi.numpy()
        assert np.abs(x - d[f"s{n}_xi"]).max() < 1e-4
        assert np.mean((x > 0.5) != (d[f"s{n}_xi"] > 0.5)) <= 1e-3
        n += 1
    sim.update_render_fields(force=True)
    assert rel_linf(sim.g0.numpy().astype(np.float32), d["g0"].astype(np.float32)) < 2e-3
    sim.close()


def _oracle_pair(nb, scenario, res, rays=(128, 256), fuv=(32, 32, 64), arith="exact", **kw):
    import oracle as O
    from nebulaviewer_gb300 import ics
    _, S = nb
    ic = ics.SCENARIOS[scenario](res=res, **kw)
    g = S.Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                         ic["P"], mom=ic["mom"], rays=rays, fuv_grid=fuv, arith=arith)
    from nebulaviewer_gb300.params import make_params, sound_speeds
    P = make_params(base=ic["P"])
    cn2, ci2, vmax = sound_speeds(P)
    mom = None if ic["mom"] is None else [m.cpu().numpy() for m in ic["mom"]]
    o = O.OracleSim(ic["shape"], ic["dx"], ic["rho"].cpu().numpy(), ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"], P,
                    rays=rays, fuv_grid=fuv, mom=mom, cn2=cn2, ci2=ci2, vmax=vmax)
    return g, o


def _compare(g, o, tol_state, tol_xi=1e-4):
    for k in ("rho", "mx", "my", "mz"):
        assert rel_linf(getattr(g, k).numpy(), getattr(o, k)) < tol_state, k
    x = g.xi.numpy()
    assert np.abs(x - o.xi).max() < tol_xi
    assert np.mean((x > 0.5) != (o.xi > 0.5)) <= 1e-3


def _errors(g, o):
    """rel-L_inf of rho, mx, my, mz, max |xi - xi_oracle| and the share of cells whose ionized mask
    (xi > 0.5) differs"""
    e = {k: rel_linf(getattr(g, k).numpy(), getattr(o, k)) for k in ("rho", "mx", "my", "mz")}
    x = g.xi.numpy()
    e["xi"] = float(np.abs(x - o.xi).max())
    e["mask"] = float(np.mean((x > 0.5) != (o.xi > 0.5)))
    return e


def _set_from_oracle(g, o):
    """the oracle's state (fields, front distance, clock) into the GPU instance, so that the next
    step is measured alone"""
    for k in ("rho", "mx", "my", "mz", "xi"):
        getattr(g, "_" + k).copy_(torch.as_tensor(np.ascontiguousarray(getattr(o, k))))
    g._dfront.copy_(torch.as_tensor(np.ascontiguousarray(o.dfront)))
    g._set_clock(t=o.t, dt=o.dt, it=o.it)
    g.invalidate()


@pytest.mark.parametrize("arith", ARITH)
def test_torus_64_against_oracle_100_steps(nb, arith):
    """the plain-step workload at its stated size: torus 64^3 (R 0.4, tube 0.15, n 100 on n 1,
    log-normal sigma 0.3), one central star with a Stromgren radius of 0.25, HLL + minmod, RK2,
    CFL 0.3, the reference's ray budgets (512 x 1024 rays); 100 steps.  Every field within rel-L_inf
    1e-5 for the first steps and 1e-3 after 100 (xi included), the ionized mask identical but for
    <= 0.1% of the cells"""
    g, o = _oracle_pair(nb, "torus", 32, rays=None, fuv=None, arith=arith)
    assert g.shape == (64, 64, 64) and g.rfront.shape == (512, 1024)
    _compare(g, o, 1e-6)
    for n in range(100):
        g.step(1)
        o.step(1)
        if n < 3:
            _compare(g, o, 1e-5)
        assert abs(g.t - o.t) <= 1e-4 * o.t
    e = _errors(g, o)
    assert max(e[k] for k in ("rho", "mx", "my", "mz", "xi")) <= 1e-3, e
    assert e["mask"] <= 1e-3, e
    g.close()


@pytest.mark.parametrize("arith", ARITH)
def test_sheet_64_each_step_against_oracle(nb, arith):
    """the turbulent-sheet workload at 64^3 with the reference's ray budgets, 12 steps (4 of them
    ionizing): before every step the GPU instance takes the oracle's state, so each step's error
    is measured alone -- rel-L_inf <= 1e-5 on rho, mx, my, mz in every step"""
    g, o = _oracle_pair(nb, "sheet", 64, rays=None, fuv=None, shape=(64, 64, 64), arith=arith)
    for n in range(12):
        _set_from_oracle(g, o)
        g.step(1)
        o.step(1)
        e = _errors(g, o)
        assert max(e[k] for k in ("rho", "mx", "my", "mz")) <= 1e-5, (n, e)
        assert e["xi"] < 1e-4 and e["mask"] <= 1e-3, (n, e)
        assert abs(g.t - o.t) <= 1e-6 * o.t
    g.close()


@pytest.mark.parametrize("arith", ARITH)
def test_sheet_256_against_oracle(nb, arith):
    """the headline workload itself: the turbulent sheet at 256^3 (6 stars, wind, 512 x 1024 rays,
    FUV on 160 x 160 x 320), 3 main-phase steps from the same state (the first ionizes), then the
    FUV field: rel-L_inf <= 1e-5 per step on rho, mx, my, mz, xi within 1e-4 with the ionized mask
    identical but for <= 0.1% of the cells, G0 within fp16 rounding"""
    g, o = _oracle_pair(nb, "sheet", 256, rays=None, fuv=None, arith=arith, device="cuda")
    assert g.shape == (256, 256, 256) and g.rfront.shape == (512, 1024) and g.att.shape == (160, 160, 320)
    _compare(g, o, 1e-6)
    for n in range(3):
        g.step(1)
        o.step(1)
        e = _errors(g, o)
        assert max(e[k] for k in ("rho", "mx", "my", "mz")) <= 1e-5, (n, e)
        assert e["xi"] < 1e-4 and e["mask"] <= 1e-3, (n, e)
        assert abs(g.t - o.t) <= 1e-6 * o.t
    g.update_render_fields(force=True)
    o.update_render_fields(force=True)
    assert rel_linf(g.g0.numpy().astype(np.float32), o.g0.astype(np.float32)) < 2e-3
    g.close()


@pytest.mark.parametrize("arith", ARITH)
def test_sheet_against_oracle(nb, arith):
    """the turbulent-sheet workload (6 stars, wind, Mach 5) at 48^3 for 12 steps, FUV at the end"""
    g, o = _oracle_pair(nb, "sheet", 48, shape=(48, 48, 48), arith=arith)
    for n in range(12):
        g.step(1)
        o.step(1)
        _compare(g, o, 1e-4 if n >= 3 else 1e-5)
    g.update_render_fields(force=True)
    o.update_render_fields(force=True)
    assert rel_linf(g.g0.numpy().astype(np.float32), o.g0.astype(np.float32)) < 5e-3
    g.close()


@pytest.mark.parametrize("arith", ARITH)
def test_uniform_rest_state_stays_exactly_at_rest_256(nb, arith):
    """size-independent property at the benchmark size: a uniform gas at rest, no stars"""
    _, S = nb
    n = 256
    rho = torch.full((n, n, n), 3.0, device="cuda")
    sim = S.Sim.from_state((n, n, n), 1.0 / n, rho, [], [], [], [], dict(cn2=1.0, ci2=144.0, vmax=72.0), arith=arith)
    sim.step(4)
    assert torch.all(sim._rho == 3.0) and torch.all(sim._mx == 0) and torch.all(sim._my == 0)
    assert torch.all(sim._mz == 0) and torch.all(sim._xi == 0)
    assert sim.dt == 0.3 * (1.0 / n) / 1.0
    sim.close()


@pytest.mark.parametrize("arith", ARITH)
def test_stromgren_radius_uniform_gas(nb, arith):
    """known answer: the front radius in uniform density n is (3Q/n^2)^(1/3) within a ray step"""
    _, S = nb
    n = 128
    dens = 2.0
    rho = torch.full((n, n, n), dens, device="cuda")
    Q = 4.0 * 0.2 ** 3 / 3.0                             # R = 0.2 at n = 2
    star = (0.5, 0.5, 0.5, 1.0, 0.0)
    sim = S.Sim.from_state((n, n, n), 1.0 / n, rho, [star], ["main"], [(0, 0, 1.0)], ["none"],
                           dict(q_main=Q, q_ramp=0.0), rays=(64, 128), start_main=False, arith=arith)
    rf = torch.zeros((64, 128), device="cuda")
    xyz = (C.c_double * 3)(0.5, 0.5, 0.5)
    nb[0].check(sim._lib.nb_cast_rays(sim._h, xyz, Q, C.c_void_p(rf.data_ptr())), sim._h, "rays")
    R = (3 * Q / dens ** 2) ** (1.0 / 3.0)
    assert abs(R - 0.2) < 1e-12
    r = rf.cpu().numpy()
    assert np.abs(r - R).max() < 0.5 / n
    sim.close()


@pytest.mark.parametrize("arith", ARITH)
def test_sheet_256_deterministic_and_conserving(nb, arith):
    """benchmark size: two runs give identical bits; FP64 totals move only by boundary flux"""
    _, S = nb
    runs = []
    for _ in range(2):
        sim = S.Sim("sheet", res=256, verbose=False, arith=arith)
        m0 = sim.conservation()
        sim.step(6)
        m1 = sim.conservation()
        runs.append((sim._rho.clone(), sim._mx.clone(), sim._xi.clone(), m0, m1))
        sim.close()
    a, b = runs
    assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1]) and torch.equal(a[2], b[2])
    assert a[3] == b[3] and a[4] == b[4]
    assert abs(a[4][0] - a[3][0]) / a[3][0] < 5e-3


@pytest.mark.parametrize("arith", ARITH)
def test_cliffwall_plane_source_against_oracle(nb, arith):
    """the ionized cloud wall: a density step with clumps, 3 stars and the -x plane-parallel
    source (no reference counterpart: checked against the oracle's FP32 and FP64 restatement)"""
    import oracle as O
    g, o = _oracle_pair(nb, "cliffwall", 64, rays=(128, 256), fuv=(32, 32, 64), nclumps=8, arith=arith)
    from nebulaviewer_gb300 import ics
    from nebulaviewer_gb300.params import make_params, sound_speeds
    ic = ics.cliffwall(res=64, nclumps=8)
    P = make_params(base=ic["P"])
    cn2, ci2, vmax = sound_speeds(P)
    o64 = O.OracleSim(ic["shape"], ic["dx"], ic["rho"].numpy(), ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                      P, rays=(128, 256), fuv_grid=(32, 32, 64), cn2=cn2, ci2=ci2, vmax=vmax, dtype=np.float64)
    assert 0.3 < float((g.xi.numpy() > 0.5).mean()) < 0.8        # the plane source ionizes the n = 1 side
    _compare(g, o, 1e-6)
    for n in range(6):
        g.step(1)
        o.step(1)
        o64.step(1)
        _compare(g, o, 1e-5)
    g.update_render_fields(force=True)
    o.update_render_fields(force=True)
    assert rel_linf(g.g0.numpy().astype(np.float32), o.g0.astype(np.float32)) < 5e-3
    for k in ("rho", "mx"):
        assert rel_linf(getattr(g, k).numpy(), getattr(o64, k)) < 1e-5
    g.close()


def _front_fields(sim):
    sim.ionize()
    torch.cuda.synchronize()
    df = sim._dfront
    return (sim._xi.clone().view(torch.int32), df.clone().view(torch.int16 if df.dtype == torch.float16 else torch.int32))


@pytest.mark.parametrize("arith", ARITH)
@pytest.mark.parametrize("case", ("sheet12", "overlapping8"))
def test_front_culling_changes_no_bit(nb, arith, case):
    """apply_front's per-segment star culling (bounds from each star's front-radius range) gives
    the same xi and front distance, bit for bit, as merging every star in every cell: a 12-star
    sheet with small fronts (most stars culled) and 8 stars in thin gas whose fronts overlap"""
    from nebulaviewer_gb300 import autotune as at, ics
    _, S = nb
    if case == "sheet12":
        ic = ics.sheet(res=128, nstars=12)
        sim = S.Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                               ic["P"], mom=ic["mom"], rays=(128, 256), fuv_grid=(32, 32, 64), arith=arith)
        sim.step(9)
    else:
        n = 96
        g = torch.Generator().manual_seed(5)
        rho = (0.05 + 0.02 * torch.rand((n, n, n), generator=g)).to("cuda")
        pos = torch.rand((8, 3), generator=g).double() * 0.8 + 0.1
        stars = [(float(p[0]), float(p[1]), float(p[2]), 1.0, 0.0) for p in pos]
        sim = S.Sim.from_state((n, n, n), 1.0 / n, rho, stars, ["main"] * 8, [(0, 0, 1.0)] * 8, ["none"] * 8,
                               dict(q_main=1e-5, q_ramp=0.0), rays=(96, 192), fuv_grid=(16, 16, 32), arith=arith)
    at.put(sim, "front_cull", 0)
    xi0, df0 = _front_fields(sim)
    at.put(sim, "front_cull", 1)
    xi1, df1 = _front_fields(sim)
    assert at.get(sim, "front_cull") == 1
    assert torch.equal(xi0, xi1) and torch.equal(df0, df1)
    ion = (xi1.view(torch.float32) > 0.5).float().mean().item()
    assert (0.0 < ion < 0.2) if case == "sheet12" else (0.05 < ion < 0.95)
    sim.close()


@pytest.mark.parametrize("arith", ARITH)
def test_pair_tables_change_no_bit(nb, arith):
    """the front and attenuation tables stored as neighbour pairs (one 8-byte gather for two
    corners) give the same xi, front distance and G0, bit for bit, as the plain tables: a 12-star
    sheet (cells next to a star, where a corner index clamps below 0, included) and the batched
    ionization of two instances"""
    from nebulaviewer_gb300 import autotune as at, ics
    from nebulaviewer_gb300.batch import BatchSim
    _, S = nb

    def sheet(res, seed):
        ic = ics.sheet(res=res, nstars=12, seed=seed)
        s = S.Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                             ic["P"], mom=ic["mom"], rays=(128, 256), fuv_grid=(32, 32, 64), arith=arith)
        s.step(4)
        return s

    sim = sheet(128, 2)
    out = {}
    for pairs in (0, 1):
        at.put(sim, "front_pairs", pairs)
        at.put(sim, "fuv_pairs", pairs)
        xi, df = _front_fields(sim)
        sim.update_render_fields(force=True)
        torch.cuda.synchronize()
        out[pairs] = (xi, df, sim._g0.clone().view(torch.int16))
    assert at.get(sim, "front_pairs") == 1 and at.get(sim, "fuv_pairs") == 1
    for a, b in zip(out[0], out[1]):
        assert torch.equal(a, b)
    sim.close()
    # the batched ionization reads and writes the same layouts
    res = {}
    for pairs in (0, 1):
        sims = [sheet(64, 3), sheet(48, 4)]
        for s in sims:
            at.put(s, "front_pairs", pairs)
        B = BatchSim(sims, graphs=False)
        B.step(3)                                   # it = 4, 5, 6: the third step ionizes (ion_every 3)
        res[pairs] = [(s._xi.clone().view(torch.int32), s._rho.clone().view(torch.int32)) for s in sims]
        B.close()
        for s in sims:
            s.close()
    for (x0, r0), (x1, r1) in zip(res[0], res[1]):
        assert torch.equal(x0, x1) and torch.equal(r0, r1)


@pytest.mark.parametrize("arith", ARITH)
def test_fuv_cut_changes_no_bit(nb, arith):
    """a FUV ray that stops once its optical depth passes the cut (exp(-tau) is 0.0f from there
    on) leaves the same attenuation bins and the same G0, bit for bit, as marching to the edge;
    the dense 12-star sheet has rays well past the cut"""
    from nebulaviewer_gb300 import autotune as at, ics
    _lib, S = nb
    ic = ics.sheet(res=128, nstars=12)
    fg = (32, 32, 64)
    sim = S.Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                           ic["P"], mom=ic["mom"], rays=(128, 256), fuv_grid=fg, arith=arith)
    sim.step(3)
    out = {}
    for cut in (0, 1):
        at.put(sim, "fuv_cut", cut)
        tabs = []
        for st in sim.stars_absolute()[0]:
            a = torch.empty(fg[2], fg[0], fg[1], device="cuda")
            xyz = (C.c_double * 3)(*[float(v) for v in st[:3]])
            _lib.check(sim._lib.nb_cast_fuv(sim._h, xyz, C.c_void_p(a.data_ptr())), sim._h, "nb_cast_fuv")
            tabs.append(a.clone())
        sim.update_render_fields(force=True)
        torch.cuda.synchronize()
        out[cut] = (torch.stack(tabs).view(torch.int32), sim._g0.clone().view(torch.int16))
    assert torch.equal(out[0][0], out[1][0]) and torch.equal(out[0][1], out[1][1])
    dark = (out[1][0].view(torch.float32) == 0.0).float().mean().item()
    assert dark > 0.05                          # a good share of the bins lies past the cut
    sim.close()


@pytest.mark.parametrize("arith", ARITH)
def test_ray_lanes_per_ray_agree(nb, arith):
    """every lanes-per-ray shape of the ionizing rays (1 .. 32) gives the same fronts up to the
    rounding of the column sums, and the Stromgren radius of uniform gas within a ray step"""
    from nebulaviewer_gb300 import autotune as at, ics
    _lib, S = nb
    ic = ics.sheet(res=64, nstars=3)
    sim = S.Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                           ic["P"], mom=ic["mom"], rays=(64, 128), fuv_grid=(16, 16, 32), arith=arith)
    st = sim.stars_absolute()[0]
    fronts = {}
    for g in (1, 2, 4, 8, 16, 32):
        at.put(sim, "ray_group", g)
        rf = torch.zeros((len(st), 128, 64), device="cuda")
        for i, s in enumerate(st):
            xyz = (C.c_double * 3)(*[float(v) for v in s[:3]])
            _lib.check(sim._lib.nb_cast_rays(sim._h, xyz, float(s[3]), C.c_void_p(rf[i].data_ptr())), sim._h, "rays")
        fronts[g] = rf.cpu().numpy()
    for g, rf in fronts.items():
        assert rel_linf(rf, fronts[4]) < 1e-5, g
    sim.close()
    n, dens = 64, 2.0
    Q = 4.0 * 0.2 ** 3 / 3.0
    uni = S.Sim.from_state((n, n, n), 1.0 / n, torch.full((n, n, n), dens, device="cuda"), [(0.5, 0.5, 0.5, 1.0, 0.0)],
                           ["main"], [(0, 0, 1.0)], ["none"], dict(q_main=Q, q_ramp=0.0), rays=(32, 64),
                           start_main=False, arith=arith)
    for g in (1, 2):
        at.put(uni, "ray_group", g)
        rf = torch.zeros((32, 64), device="cuda")
        xyz = (C.c_double * 3)(0.5, 0.5, 0.5)
        _lib.check(uni._lib.nb_cast_rays(uni._h, xyz, Q, C.c_void_p(rf.data_ptr())), uni._h, "rays")
        assert np.abs(rf.cpu().numpy() - 0.2).max() < 0.5 / n
    uni.close()


@pytest.mark.parametrize("arith", ARITH)
def test_fuv_lanes_per_ray_agree(nb, arith):
    """every lanes-per-ray shape of the FUV rays (8, 16, 32) in both table layouts gives the same G0
    (float32 fields) up to the rounding of the optical-depth sums, and each shape gives the same bits
    in both layouts and with the optical-depth cut on and off; a dense 12-star sheet with rays past
    the cut"""
    from nebulaviewer_gb300 import autotune as at, ics
    _, S = nb
    ic = ics.sheet(res=96, nstars=12)
    sim = S.Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                           dict(ic["P"], fp32_fields=True), mom=ic["mom"], rays=(64, 128), fuv_grid=(24, 24, 48),
                           arith=arith)
    sim.step(3)
    out = {}
    for cut in (1, 0):
        at.put(sim, "fuv_cut", cut)
        for pairs in (0, 1):
            at.put(sim, "fuv_pairs", pairs)
            for g in (8, 16, 32):
                at.put(sim, "fuv_group", g)
                sim.fuv_field()
                torch.cuda.synchronize()
                out[cut, pairs, g] = sim.g0.numpy().astype(np.float32)
    assert out[1, 0, 16].dtype == np.float32 and np.isfinite(out[1, 0, 16]).all() and out[1, 0, 16].max() > 0
    for k, v in out.items():
        assert rel_linf(v, out[1, 0, 16]) < 1e-5, k
    for g in (8, 16, 32):
        for cut in (0, 1):
            assert np.array_equal(out[cut, 0, g].view(np.int32), out[cut, 1, g].view(np.int32)), (cut, g)
            assert np.array_equal(out[cut, 0, g].view(np.int32), out[1 - cut, 0, g].view(np.int32)), (cut, g)
    sim.close()


@pytest.mark.parametrize("solver,lim", (("hll", "minmod"), ("hll", "vanleer"), ("hll", "mc"), ("rusanov", "minmod")))
def test_ragged_grid_many_stars_stage_bit_identical(nb, solver, lim):
    """a 37 x 45 x 100 grid (partial j and k tiles, uneven i-chunks), dx = 0.01 (not a power of
    two), 40 stars with jets, proto-jets and wind (the per-tile jet list takes two ballot rounds):
    both RK2 stages bit-identical to the oracle's restatement of the reference kernel"""
    import math
    import oracle as O
    from nebulaviewer_gb300 import autotune as at
    from nebulaviewer_gb300.params import make_params, sound_speeds
    _lib, S = nb
    shape, dx = (37, 45, 100), 0.01
    rng = np.random.default_rng(11)
    rho = (0.5 + rng.random(shape)).astype(np.float32)
    mom = [(0.4 * rng.standard_normal(shape)).astype(np.float32) for _ in range(3)]
    xi = rng.random(shape).astype(np.float32)
    L = np.array(shape) * dx
    pos = rng.random((40, 3)) * L
    stars = [(float(p[0]), float(p[1]), float(p[2]), float(0.5 + rng.random()), 0.0) for p in pos]
    d = rng.standard_normal((40, 3))
    jets = [tuple(float(v) for v in a / np.linalg.norm(a)) for a in d]
    jkinds = [("jet", "proto", "none")[i % 3] for i in range(40)]
    P = dict(q_main=1.0, q_ramp=0.0, wind=0.5, jet=3.0, jet_proto=2.0, jet_r=0.12, jet_angle=35.0, max_stars=64,
             solver=solver, limiter=lim, floor=2e-3, cfl=0.3)
    sim = S.Sim.from_state(shape, dx, torch.as_tensor(rho, device="cuda"), stars, ["main"] * 40, jets, jkinds, P,
                           mom=[torch.as_tensor(m, device="cuda") for m in mom], rays=(16, 32), fuv_grid=(8, 8, 16),
                           start_main=False, arith="exact")
    at.put(sim, "chunk_i", 10)                            # 4 chunks of 9 or 10 planes
    sim._xi.copy_(t32(xi))
    Pm = make_params(base=P)
    cn2, ci2, vmax = sound_speeds(Pm)
    o = O.OracleSim(shape, dx, rho, stars, ["main"] * 40, jets, jkinds, Pm, rays=(16, 32), fuv_grid=(8, 8, 16),
                    mom=mom, start_main=False, cn2=cn2, ci2=ci2, vmax=vmax)
    o._set_star_weights()
    assert float((o.jet_arr[:40, 3] > 0).sum()) > 20
    dt, pulse = 2e-4, 1.3
    U = [t32(rho)] + [t32(m) for m in mom]
    g1 = [torch.zeros_like(U[0]) for _ in range(4)]
    g2 = [torch.zeros_like(U[0]) for _ in range(4)]
    F = lambda ts: _lib.f4([t.data_ptr() for t in ts])  # noqa: E731
    _lib.check(sim._lib.nb_hydro_stage(sim._h, F(U), F(U), F(g1), 0.0, 1.0, dt, pulse), sim._h, "stage 1")
    _lib.check(sim._lib.nb_hydro_stage(sim._h, F(g1), F(U), F(g2), 0.5, 0.5, dt, pulse), sim._h, "stage 2")
    torch.cuda.synchronize()
    Un = [rho] + mom
    o1 = [np.zeros(shape, np.float32) for _ in range(4)]
    o2 = [np.zeros(shape, np.float32) for _ in range(4)]
    common = dict(stars=o.star_arr, nstars=40, wind=0.5, jets=o.jet_arr, jet_cos=math.cos(math.radians(35.0)),
                  jet_r=0.12, pulse=pulse, dt=dt, dx=dx, floor_=2e-3, cn2=cn2, ci2=ci2, vmax=vmax,
                  solver=1 if solver == "hll" else 0, lim={"minmod": 0, "vanleer": 1, "mc": 2}[lim])
    o.K.hydro_stage(Un, xi, Un, o1, a=0.0, b=1.0, **common)
    o.K.hydro_stage(o1, xi, Un, o2, a=0.5, b=0.5, **common)
    assert bits_equal(torch.stack(g1).cpu().numpy(), np.stack(o1))
    assert bits_equal(torch.stack(g2).cpu().numpy(), np.stack(o2))
    sim.close()


@pytest.mark.parametrize("arith", ARITH)
@pytest.mark.parametrize("nstars", (0, 36))
def test_star_count_edges_against_oracle(nb, arith, nstars):
    """no stars at all (no rays, no fronts, no FUV sources), and 36 stars (more than a row table
    holds: the per-cell front and FUV forms, no culling) on a 40 x 24 x 44 grid, stepped and
    ionized against the oracle"""
    import oracle as O
    from nebulaviewer_gb300.params import make_params, sound_speeds
    _, S = nb
    shape, dx = (40, 24, 44), 1.0 / 48
    rng = np.random.default_rng(5 + nstars)
    rho = (0.05 + 0.5 * rng.random(shape) ** 4).astype(np.float32)
    L = np.array(shape) * dx
    pos = rng.random((nstars, 3)) * L * 0.9 + 0.05 * L
    stars = [(float(p[0]), float(p[1]), float(p[2]), float(0.5 + rng.random()), 0.0) for p in pos]
    P = dict(q_main=4e-6, q_ramp=0.0, wind=0.5, max_stars=64, solver="hll", limiter="minmod", cfl=0.3)
    g = S.Sim.from_state(shape, dx, torch.as_tensor(rho, device="cuda"), stars, ["main"] * nstars,
                         [(0.0, 0.0, 1.0)] * nstars, ["none"] * nstars, P, rays=(32, 64), fuv_grid=(16, 16, 32),
                         arith=arith)
    Pm = make_params(base=P)
    cn2, ci2, vmax = sound_speeds(Pm)
    o = O.OracleSim(shape, dx, rho, stars, ["main"] * nstars, [(0.0, 0.0, 1.0)] * nstars, ["none"] * nstars, Pm,
                    rays=(32, 64), fuv_grid=(16, 16, 32), cn2=cn2, ci2=ci2, vmax=vmax)
    _compare(g, o, 1e-6)
    for _ in range(4):
        g.step(1)
        o.step(1)
        _compare(g, o, 1e-5)
    g.update_render_fields(force=True)
    o.update_render_fields(force=True)
    g0 = g.g0.numpy().astype(np.float32)
    if nstars == 0:
        assert not g0.any() and not g.xi.numpy().any()
    else:
        assert rel_linf(g0, o.g0.astype(np.float32)) < 5e-3
        assert 0.0 < float((g.xi.numpy() > 0.5).mean()) < 0.9
    g.close()

"""The CPU oracle against the golden fixtures made from the reference's own kernel source
and its own Sim driver (tests/golden/make_golden.py).  This pins the oracle."""
import numpy as np
import pytest

import oracle as O
from conftest import bits_equal, golden_sim, rel_linf

HYDRO = (("rus", 0, 0), ("hll0", 1, 0), ("hll1", 1, 1), ("hll2", 1, 2))


@pytest.mark.parametrize("name,solver,lim", HYDRO)
def test_hydro_stage_bit_exact(kernels_npz, name, solver, lim):
    d = kernels_npz
    K = O.Kernels(np.float32)
    dx, cn2, ci2, floor, vmax, jet_cos, jet_r, pulse, wind, dt = d["k_scalars"]
    rho, mom, xi = d["k_rho"], d["k_mom"], d["k_xi"]
    U = [rho, mom[0], mom[1], mom[2]]
    o1 = np.zeros((4,) + rho.shape, np.float32)
    K.hydro_stage(U, xi, U, list(o1), d["k_stars"], 3, wind, d["k_jets"], jet_cos, jet_r, pulse, dt, dx, 0.0, 1.0,
                  floor, cn2, ci2, vmax, solver, lim)
    assert bits_equal(o1, d[f"k_{name}_s1"])
    o2 = np.zeros_like(o1)
    K.hydro_stage(list(o1), xi, U, list(o2), d["k_stars"], 3, wind, d["k_jets"], jet_cos, jet_r, pulse, dt, dx, 0.5,
                  0.5, floor, cn2, ci2, vmax, solver, lim)
    assert bits_equal(o2, d[f"k_{name}_s2"])


def test_hydro_stage_in_place_equals_out_of_place(kernels_npz):
    """sim.py:1026-1027: stage 2 over U^n in place is bit-identical to a separate output"""
    d = kernels_npz
    K = O.Kernels(np.float32)
    dx, cn2, ci2, floor, vmax, jet_cos, jet_r, pulse, wind, dt = d["k_scalars"]
    U = [d["k_rho"].copy(), *[m.copy() for m in d["k_mom"]]]
    U1 = [np.ascontiguousarray(x) for x in d["k_hll0_s1"]]
    args = (d["k_stars"], 3, wind, d["k_jets"], jet_cos, jet_r, pulse, dt, dx, 0.5, 0.5, floor, cn2, ci2, vmax, 1, 0)
    out = [np.zeros_like(U[0]) for _ in range(4)]
    K.hydro_stage(U1, d["k_xi"], U, out, *args)
    K.hydro_stage(U1, d["k_xi"], U, U, *args)
    assert bits_equal(np.stack(out), np.stack(U))


def test_max_speed(kernels_npz):
    d = kernels_npz
    K = O.Kernels(np.float32)
    _, cn2, ci2 = d["k_scalars"][:3]
    assert np.float32(K.max_speed(d["k_rho"], *d["k_mom"], d["k_xi"], cn2, ci2)) == d["k_smax"][0]


@pytest.mark.parametrize("tag,f", (("full", 1.0), ("half", 0.5)))
def test_rays_front_smooth(kernels_npz, tag, f):
    d = kernels_npz
    K = O.Kernels(np.float32)
    dx = d["k_scalars"][0]
    rr = d["r_rho"]
    nu, nphi, diag = d["r_meta"]
    L = np.array(rr.shape) * dx
    ns = int(d[f"r_{tag}_nsteps"][0])
    xa = np.zeros(rr.shape, np.float32)
    dfa = np.full(rr.shape, 1e3, np.float32)
    for s, st in enumerate(d["r_stars"]):
        rf = K.cast_rays(rr, st[:3], st[3], f * dx, ns, dx, diag, L, int(nu), int(nphi))
        # float32 cos/sin/atan2 of numpy vs the C library: a few ulps
        assert rel_linf(rf, d[f"r_{tag}_rfront"][s]) < 1e-6
        K.apply_front(rf, st[:3], dx, 1.2 * dx, xa, dfa)
    assert np.abs(xa - d[f"r_{tag}_xi_raw"]).max() < 1e-5
    assert np.abs(dfa - d[f"r_{tag}_df"]).max() < 1e-5
    assert np.abs(K.smooth_xi(xa) - d[f"r_{tag}_xi"]).max() < 1e-5
    # the smoothing itself is bit-exact on the same input
    assert bits_equal(K.smooth_xi(d[f"r_{tag}_xi_raw"]), d[f"r_{tag}_xi"])


def test_fuv(kernels_npz):
    d = kernels_npz
    K = O.Kernels(np.float32)
    dx = d["k_scalars"][0]
    rr = d["r_rho"]
    L = np.array(rr.shape) * dx
    fnr, fnu, fnp, kappa, binr, ns = d["f_meta"]
    g0 = np.zeros(rr.shape, np.float32)
    for s, st in enumerate(d["r_stars"]):
        att = K.cast_fuv(rr, d["r_full_xi"], st[:3], kappa, dx, int(ns), dx, binr, L, int(fnr), int(fnu), int(fnp))
        assert np.abs(att - d["f_att"][s]).max() < 1e-6
        K.apply_fuv(att, st[:3], st[3] / 0.1, dx, binr, g0)
    assert rel_linf(g0, d["f_g0"]) < 1e-6


def test_to_half(kernels_npz):
    d = kernels_npz
    assert np.array_equal(O.to_half(d["h_in"]).view(np.uint16), d["h_out"].view(np.uint16))
    x = np.random.default_rng(0).standard_normal(100000).astype(np.float32) * np.float32(3e4)
    with np.errstate(over="ignore"):            # values beyond 65504 round to +-inf on purpose
        ref = x.astype(np.float16)
    assert np.array_equal(O.to_half(x).view(np.uint16), ref.view(np.uint16))


@pytest.mark.parametrize("name", ("bubbles", "bipolar", "cliff"))
def test_oracle_sim_matches_reference_sim(name):
    """OracleSim (sim.py's driver restated) against the reference Sim run end to end"""
    d, m = golden_sim(name)
    sim = O.OracleSim(m["shape"], m["dx"], d["s0_rho"], m["stars"], m["kinds"], m["jets"], m["jkinds"], m["P"],
                      rays=m["rays"], fuv_grid=m["fuv"], ion_every=m["ion_every"], fast=m["fast"])
    assert np.abs(sim.xi - d["s0_xi"]).max() < 1e-5
    n = 1
    while f"s{n}_rho" in d.files:
        sim.dt_cap = m["dt_caps"][n - 1]
        sim.step(1)
        assert sim.t == float(d[f"s{n}_t"]) and sim.dt == float(d[f"s{n}_dt"])
        for k in ("rho", "mx", "my", "mz"):
            assert rel_linf(getattr(sim, k), d[f"s{n}_{k}"]) < 1e-5, (n, k)
        assert np.abs(sim.xi - d[f"s{n}_xi"]).max() < 1e-4
        n += 1
    sim.update_render_fields(force=True)
    assert rel_linf(sim.g0.astype(np.float32), d["g0"].astype(np.float32)) < 1e-3


def test_fp64_twin_runs_and_is_close(kernels_npz):
    """the FP64 re-run of the same scheme: close to FP32 on one stage"""
    d = kernels_npz
    dx, cn2, ci2, floor, vmax, jet_cos, jet_r, pulse, wind, dt = d["k_scalars"]
    U = [d["k_rho"], *d["k_mom"]]
    out = {}
    for T in (np.float32, np.float64):
        K = O.Kernels(T)
        o = np.zeros((4,) + d["k_rho"].shape, T)
        K.hydro_stage([u.astype(T) for u in U], d["k_xi"].astype(T), [u.astype(T) for u in U], list(o),
                      d["k_stars"].astype(T), 3, wind, d["k_jets"].astype(T), jet_cos, jet_r, pulse, dt, dx, 0.0,
                      1.0, floor, cn2, ci2, vmax, 1, 0)
        out[T] = o
    assert rel_linf(out[np.float32], out[np.float64]) < 1e-5


# ---------------------------------------------------------------------------- stirring
@pytest.mark.parametrize("tag", ("in", "out"))
def test_drive_bit_exact(tag):
    """nebula3d.py:165-179 drive; 'out': part of the domain lies outside the forcing grid (samples 0)"""
    from conftest import golden
    z = golden("stir.npz")
    m = [a.copy() for a in z["d_mom"]]
    blend, amp, dt, dx, dxs = z[f"d_{tag}_scalars"]
    O.Kernels().drive(z["d_rho"], *m, z[f"d_{tag}_A"], z[f"d_{tag}_B"], blend, amp, dt, dx, dxs)
    for a, b in zip(m, z[f"d_{tag}_out"]):
        assert bits_equal(a, b)


def test_add_torus_bit_exact():
    from conftest import golden
    z = golden("stir.npz")
    r, m = z["d_rho"].copy(), [a.copy() for a in z["d_mom"]]
    O.Kernels().add_torus(z["a_torus"], r, *m)
    assert bits_equal(r, z["a_rho"])
    for a, b in zip(m, z["a_mom"]):
        assert bits_equal(a, b)


@pytest.mark.parametrize("tag,shape,kmax", (("odd", (7, 6, 5), 4.0), ("even", (8, 6, 10), 6.0)))
def test_forcing_generator_reproduces_reference_draws(tag, shape, kmax):
    """the package's forcing generator: the reference's field bit for bit from an equal Generator
    state, and the Generator left in the same state"""
    from conftest import golden
    from nebulaviewer_gb300 import stir
    z = golden("stir.npz")
    g = np.random.default_rng(4242)
    assert bits_equal(np.stack(stir.solenoidal(shape, g, 1.0, kmax)), z[f"sol_{tag}"])
    assert np.array_equal(g.standard_normal(4), z[f"sol_{tag}_next"])


def test_matched_forcing_reproduces_reference_fields():
    """the reference's default "matched" mode draws its forcing fields from a per-call seeded
    spectrum (sim.py:270-337); the reference Sim of the bake fixture drew A and B that way right
    after its initial conditions (one call) -- three calls per field, so A used calls 2-4 and B 5-7"""
    import json
    from conftest import golden
    from nebulaviewer_gb300 import stir
    z = golden("bake_bipolar.npz")
    m = json.loads(str(z["meta"]))
    seed, calls, kmax = m["noise"]["seed"], m["noise"]["calls"], float(m["P"]["pre_kmax"])
    shape = tuple(m["sshape"])
    a = np.stack(stir.matched_solenoidal(shape, seed, calls - 6, 1.0, kmax, m["noise"]["K"]))
    b = np.stack(stir.matched_solenoidal(shape, seed, calls - 3, 1.0, kmax, m["noise"]["K"]))
    assert bits_equal(a, z["s_drv_A"]) and bits_equal(b, z["s_drv_B"])


def test_forcing_grid_rules():
    """sim.py:761-768: 24 cells per unit + 2 (resolution independent), or one per 6 cells + 2"""
    from nebulaviewer_gb300 import stir
    assert stir.forcing_grid((1.6, 1.6, 1.6), 1 / 128, (205, 205, 205)) == ((41, 41, 41), 1 / 24)
    assert stir.forcing_grid((2.0, 2.0, 2.0), 0.125, (16, 16, 16), physical=False) == ((4, 4, 4), 0.75)


def test_oracle_sim_through_stirring_phase_matches_reference_sim():
    """the oracle's Sim driver against the reference Sim: stirring phase with a field swap, its end
    (torus, first ionization), main-phase stirring with another swap -- every field bit for bit"""
    d, m = golden_sim("bipolar_pre")
    o = O.OracleSim(m["shape"], m["dx"], d["rho_ic"], m["stars"], m["kinds"], m["jets"], m["jkinds"], m["P"],
                    rays=m["rays"], fuv_grid=m["fuv"], ion_every=m["ion_every"], fast=True, torus=d["torus"],
                    stir_fields=list(d["fields"]), stir_grid=(m["sshape"], m["dxs"]), cn2=m["cn2"], ci2=m["ci2"])
    for n, st in enumerate(m["steps"]):
        o.step(1)
        assert o.phase == st["phase"] and o.tp == st["tp"] and o.t == st["t"] and o.dt == st["dt"]
        assert (o.drv is None) == (st["clock"] is None)
        if o.drv is not None:
            assert o.drv["clock"] == st["clock"]
        for f in ("rho", "mx", "my", "mz", "xi"):
            assert bits_equal(getattr(o, f), d[f"s{n + 1}_{f}"]), (n, f)
        if st["mach"] is not None:
            assert abs(o.mach - st["mach"]) <= 1e-5 * st["mach"]        # FP64 sum vs the reference's FP32 atomics


# ---------------------------------------------------------------------------- renderer pack
@pytest.mark.parametrize("tag", ("jwst", "sho", "nat"))
def test_render_pack_bit_exact(tag):
    """render.py:176-205 pack_volume_lm and the [1 4 1] prefilter of render.py:281-298"""
    from conftest import golden
    z = golden("render.npz")
    pp = z[f"p_{tag}_params"]
    a = O.render_pack(z["p_rho"], z["p_mom"], z["p_xi"], z["p_df"], z["p_g0"], pp, int(pp[22]), smooth=False)
    b = O.render_pack(z["p_rho"], z["p_mom"], z["p_xi"], z["p_df"], z["p_g0"], pp, int(pp[22]), smooth=True)
    assert np.array_equal(a.view(np.uint16), z[f"p_{tag}_packed"].view(np.uint16))
    assert np.array_equal(b.view(np.uint16), z[f"p_{tag}_smooth"].view(np.uint16))

"""Generate the golden fixtures under tests/golden/ by running the REFERENCE's own
kernel source and its `Sim` driver on small seeded inputs.

    python tests/golden/make_golden.py --ref <reference checkout>

(or set NEBULA_REFERENCE to the checkout instead of passing --ref)

The reference is NVIDIA-Warp Python; `warp` is absent here, so `warp_stub` supplies
a float32 restatement of the Warp builtins its kernels call (see that module's
docstring for exactly what it does and does not reproduce).  Everything else —
the kernel bodies, `Sim.reset/_start_main/step/ionize/fuv_field/_compute_dt/
_hydro/_set_star_weights`, the initial conditions — is the reference's code,
imported unmodified from the reference checkout.

Fixtures (all small, committed):
  kernels.npz      per-kernel inputs/outputs: hydro_stage (Rusanov), hydro_stage_hll
                   (minmod / van Leer / MC) for both RK2 stages, max_speed, cast_rays,
                   apply_front, smooth_xi, cast_fuv, apply_fuv, to_half.
  sim_<name>.npz   end-to-end reference `Sim` runs: the state after reset (first
                   ionization included) and after every step, clocks, the FUV field.
  stir.npz         the stirring kernels (drive, add_torus) and the solenoidal forcing
                   generator on a seeded Generator.
  render.npz       the renderer's voxel pack (pack_volume_lm) and [1 4 1] prefilter.
  sim_bipolar_pre.npz  a reference `Sim` run through the pre-turbulence (stirring) phase,
                   its end (torus added, first ionization) and main-phase stirring, with
                   every forcing field the run drew.
  bake_<scene>.npz bake.py's loop run by the reference on the bipolar (stirring phase) and
                   bubbles (main phase, winds, triggered formation switched off) presets in the
                   default matched mode (replace_stars, live events, dt_cap, frames), with the
                   reference Sim as constructed (what Sim.from_reference reads).
Test infrastructure only: nothing in the product reads these files.
"""
import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import warp_stub  # noqa: E402

warp_stub.install()


def import_reference(ref):
    sys.path.insert(0, ref)
    sys.dont_write_bytecode = True
    import nebula3d  # noqa: F401
    import sim as refsim
    return sys.modules["nebula3d"], refsim


def f32(x):
    return np.asarray(x, np.float32)


# ----------------------------------------------------------------------------- per-kernel cases
def kernel_cases(N, S, rng):
    wp = warp_stub
    out = {}
    nx, ny, nz = 10, 9, 8
    dx = 1.0 / nz
    shape = (nx, ny, nz)
    rho = np.exp(rng.normal(0.0, 1.2, shape)).astype(np.float32)
    rho[rng.random(shape) < 0.06] = 1e-3               # below the floor (2e-3): exercises max(rho, floor)
    vel = rng.normal(0.0, 1.5, (3,) + shape).astype(np.float32)
    vel[:, rng.random(shape) < 0.05] *= 8.0            # a few cells above vmax = 6
    mom = (vel * rho).astype(np.float32)
    xi = rng.random(shape).astype(np.float32)
    xi[rng.random(shape) < 0.2] = 0.0
    xi[rng.random(shape) < 0.1] = 1.0
    L = np.array(shape) * dx
    stars = np.array([[0.45 * L[0], 0.55 * L[1], 0.5 * L[2], 1.0],
                      [0.2 * L[0], 0.3 * L[1], 0.7 * L[2], 0.4],
                      [0.8 * L[0], 0.7 * L[1], 0.2 * L[2], 0.0]], np.float32)       # last one off
    ax = rng.normal(size=(3, 3))
    ax /= np.linalg.norm(ax, axis=1, keepdims=True)
    jets = np.concatenate([ax, np.array([[3.0], [0.0], [2.0]])], 1).astype(np.float32)
    cn2, ci2, floor, vmax = (1.0 / 12.0) ** 2, 1.0, 2e-3, 6.0
    jet_cos, jet_r, pulse, wind = math.cos(math.radians(30.0)), 0.3, 1.3, 0.5
    smax = np.zeros(1, np.float32)
    N.max_speed.run(shape, [rho, mom[0], mom[1], mom[2], xi, cn2, ci2, smax])
    dt = 0.3 * dx / float(smax[0])
    out.update(k_rho=rho, k_mom=mom, k_xi=xi, k_stars=stars, k_jets=jets, k_smax=smax.copy(),
               k_scalars=np.array([dx, cn2, ci2, floor, vmax, jet_cos, jet_r, pulse, wind, dt], np.float64))
    sv = [wp.vec4(*s) for s in stars]
    jv = [wp.vec4(*j) for j in jets]
    for name, kern, lim in (("rus", N.hydro_stage, None), ("hll0", S.hydro_stage_hll, 0),
                            ("hll1", S.hydro_stage_hll, 1), ("hll2", S.hydro_stage_hll, 2)):
        t0 = time.time()
        o1 = np.zeros((4,) + shape, np.float32)
        common = [sv, len(sv), wind, jv, jet_cos, jet_r, pulse, dt, dx]
        tail = [floor, cn2, ci2, vmax] + ([lim] if lim is not None else [])
        kern.run(shape, [rho, mom[0], mom[1], mom[2], xi, rho, mom[0], mom[1], mom[2],
                         o1[0], o1[1], o1[2], o1[3]] + common + [0.0, 1.0] + tail)
        o2 = np.zeros((4,) + shape, np.float32)
        kern.run(shape, [o1[0], o1[1], o1[2], o1[3], xi, rho, mom[0], mom[1], mom[2],
                         o2[0], o2[1], o2[2], o2[3]] + common + [0.5, 0.5] + tail)
        out[f"k_{name}_s1"] = o1
        out[f"k_{name}_s2"] = o2
        print(f"  hydro {name}: {time.time() - t0:.1f}s", flush=True)

    # ---- ionization: a dense blob so some rays stop and some reach rcap
    g = (np.indices(shape).transpose(1, 2, 3, 0) + 0.5) * dx
    blob = 30.0 * np.exp(-np.sum((g - np.array([0.6, 0.5, 0.45]) * L) ** 2, -1) / (2 * 0.12 ** 2))
    rrho = (rho * 0.5 + blob).astype(np.float32)
    diag = float(math.sqrt(float(np.sum(L ** 2))) + 0.6)
    bmax = wp.vec3(*L)
    ray_stars = [(0.45 * L[0], 0.55 * L[1], 0.5 * L[2], 2e-2),
                 (0.15 * L[0], 0.8 * L[1], 0.3 * L[2], 4e-1),
                 (-0.3, 0.4 * L[1], 0.5 * L[2], 3.0)]          # outside the box: t_in > 0
    nu, nphi = 6, 12
    out["r_rho"] = rrho
    out["r_stars"] = np.array(ray_stars, np.float64)
    out["r_meta"] = np.array([nu, nphi, diag], np.float64)
    for tag, drf in (("full", 1.0), ("half", 0.5)):
        dr = drf * dx
        nsteps = int(diag / dr) + 1
        xi_a = np.zeros(shape, np.float32)
        df_a = np.full(shape, 1e3, np.float32)
        rfs = []
        for (sx, sy, sz, Q) in ray_stars:
            rf = np.zeros((nu, nphi), np.float32)
            svec = wp.vec3(sx, sy, sz)
            N.cast_rays.run((nu, nphi), [rrho, svec, Q, dr, nsteps, dx, diag, bmax, rf])
            N.apply_front.run(shape, [rf, svec, dx, 1.2 * dx, xi_a, df_a])
            rfs.append(rf)
        xi_raw = xi_a.copy()
        xs = np.zeros(shape, np.float32)
        N.smooth_xi.run(shape, [xi_a, xs])
        out[f"r_{tag}_rfront"] = np.stack(rfs)
        out[f"r_{tag}_xi_raw"] = xi_raw
        out[f"r_{tag}_df"] = df_a
        out[f"r_{tag}_xi"] = xs
        out[f"r_{tag}_nsteps"] = np.array([nsteps])
    print("  rays done", flush=True)

    # ---- FUV: reuse the smoothed xi from the full-step ionization
    fnr, fnu, fnp = 5, 4, 8
    binr = diag / fnr
    kappa = 10.0
    g0 = np.zeros(shape, np.float32)
    atts = []
    dr = dx
    nsteps = int(diag / dr) + 1
    for (sx, sy, sz, Q) in ray_stars:
        att = np.zeros((fnr, fnu, fnp), np.float32)
        svec = wp.vec3(sx, sy, sz)
        N.cast_fuv.run((fnu, fnp), [rrho, out["r_full_xi"], svec, kappa, dr, nsteps, dx, binr, bmax, att])
        N.apply_fuv.run(shape, [att, svec, Q / 0.1, dx, binr, g0])
        atts.append(att)
    out["f_att"] = np.stack(atts)
    out["f_g0"] = g0
    out["f_meta"] = np.array([fnr, fnu, fnp, kappa, binr, nsteps], np.float64)
    h = np.array([0.0, -0.0, 1e-8, 3.14159, 65504.0, 65519.0, 65520.0, 1e6, -2.5e-5, 1000.0, 0.1],
                 np.float32).reshape(1, 1, 11)
    ho = np.zeros(h.shape, np.float16)
    S.to_half.run(h.shape, [h, ho])
    out["h_in"], out["h_out"] = h, ho
    print("  fuv / to_half done", flush=True)
    return out


# ----------------------------------------------------------------------------- reference Sim runs
def sim_case(S, scenario, res, overrides, nsteps, fast, rays, fuv, ion_every=None, dt_cap_at=None):
    P = S.make_params(scenario, overrides)
    t0 = time.time()
    sim = S.Sim(scenario, res=res, params=P, ic_mode="matched", rays=rays, fuv_grid=fuv,
                ion_every=ion_every, device="cpu", verbose=False, fast=fast)
    print(f"  {scenario} {sim.shape} reset {time.time() - t0:.1f}s, {len(sim.stars)} stars", flush=True)

    def snap():
        return dict(rho=sim.rho.numpy(), mx=sim.mx.numpy(), my=sim.my.numpy(), mz=sim.mz.numpy(),
                    xi=sim.xi.numpy(), dfront=sim.dfront.numpy())

    s0 = snap()
    rho0 = s0["rho"]
    meta = dict(scenario=scenario, res=res, shape=list(sim.shape), dx=sim.dx, L=list(sim.L), fast=fast,
                rays=list(rays), fuv=list(fuv), ion_every=sim.ion_every, fuv_every=sim.fuv_every,
                stars=[list(map(float, s)) for s in sim.stars], kinds=list(sim.kinds),
                jets=[list(map(float, j)) for j in sim.jets], jkinds=list(sim.jkinds),
                P={k: v for k, v in sim.P.items() if isinstance(v, (int, float, str, bool, type(None), list))},
                dr=sim.dr, nsteps=sim.nsteps, diag=sim.diag, cap=sim.cap, cn2=sim.cn2, ci2=sim.ci2,
                dt_caps=[])
    steps = []
    for n in range(nsteps):
        cap = None
        if dt_cap_at is not None and n == dt_cap_at:
            cap = 0.5 * sim.P["cfl"] * sim.dx / 12.0
        sim.dt_cap = cap
        meta["dt_caps"].append(cap)
        t1 = time.time()
        sim.step(1)
        st = snap()
        st.update(t=sim.t, dt=sim.dt, it=sim.it)
        steps.append(st)
        print(f"    step {n}: t={sim.t:.6g} dt={sim.dt:.6g} ({time.time() - t1:.1f}s)", flush=True)
    sim.dt_cap = None
    sim.update_render_fields(force=True)
    g0 = sim.g0.numpy()
    out = {"meta": np.array(json.dumps(meta)), "rho_ic": rho0}
    # the state right after reset (includes _start_main's first ionization)
    for k, v in s0.items():
        out[f"s0_{k}"] = v
    for n, st in enumerate(steps):
        for k, v in st.items():
            out[f"s{n + 1}_{k}"] = np.asarray(v)
    out["g0"] = g0
    return out


def timeline_cases(ref, rng):
    """timeline.py:19-89: the 13 B/cell snapshot pack / unpack of the reference (k_pack_lm /
    k_unpack_lm for fp16 dfront / g0, k_pack / k_unpack for fp32)"""
    sys.path.insert(0, ref)
    import timeline as T
    shape = (6, 5, 8)
    rho = np.exp(rng.normal(0, 3.0, shape)).astype(np.float32)
    rho.flat[:4] = [70000.0, 1e-9, 65504.0, 3.0e4]
    mom = (rng.normal(0, 1.0, (3,) + shape) * np.exp(rng.normal(0, 4.0, (3,) + shape))).astype(np.float32)
    mom[0].flat[:3] = [-1e6, 1e6, -0.0]
    xi = rng.uniform(-0.2, 1.2, shape).astype(np.float32)
    xi.flat[:6] = [0.0, 1.0, 0.5 / 255, 1.5 / 255, 254.5 / 255, 0.99999]
    df32 = rng.normal(0, 2.0, shape).astype(np.float32) * np.float32(1e3)
    df32.flat[:2] = [1e3, -7e4]
    g032 = np.exp(rng.normal(0, 5.0, shape)).astype(np.float32)
    df16, g016 = df32.astype(np.float16), g032.astype(np.float16)
    out = {"t_rho": rho, "t_mom": mom, "t_xi": xi, "t_df16": df16, "t_g016": g016, "t_df32": df32, "t_g032": g032}
    for tag, kp, ku, df, g0 in (("lm", T.k_pack_lm, T.k_unpack_lm, df16, g016), ("f32", T.k_pack, T.k_unpack, df32,
                                                                             g032)):
        o = [np.zeros(shape, np.float16) for _ in range(4)] + [np.zeros(shape, np.uint8)] + \
            [np.zeros(shape, np.float16) for _ in range(2)]
        kp.run(shape, [rho, mom[0], mom[1], mom[2], xi, df, g0] + o)
        for name, a in zip(("r", "mx", "my", "mz", "xi", "df", "g0"), o):
            out[f"t_{tag}_pack_{name}"] = a
        fdt = np.float16 if tag == "lm" else np.float32
        u = [np.zeros(shape, np.float32) for _ in range(5)] + [np.zeros(shape, fdt) for _ in range(2)]
        ku.run(shape, o + [2e-3] + u)
        for name, a in zip(("rho", "mx", "my", "mz", "xi", "df", "g0"), u):
            out[f"t_{tag}_unpack_{name}"] = a
    # nebula3d.py:182-191 shock_field on a positive-density state
    rr = np.exp(rng.normal(0, 1.0, shape)).astype(np.float32) + np.float32(0.01)
    sh = np.zeros(shape, np.float32)
    T.N.shock_field.run(shape, [rr, mom[0], mom[1], mom[2], 0.125, sh])
    out["t_shock_rho"], out["t_shock"] = rr, sh
    return out


# ----------------------------------------------------------------------------- stirring
def stir_cases(N, S, rng):
    """nebula3d.py:165-179 drive, sim.py:352-363 add_torus, nebula3d.py:514-525 solenoidal"""
    out = {}
    shape = (10, 9, 8)
    dx = 1.0 / 8.0
    rho = np.exp(rng.normal(0.0, 1.0, shape)).astype(np.float32)
    mom = (rng.normal(0.0, 1.0, (3,) + shape) * rho).astype(np.float32)
    # coarse grids: one covering the domain, one too short along y (samples outside read 0)
    for tag, sshape, dxs in (("in", (7, 6, 5), 0.23), ("out", (6, 3, 5), 0.3)):
        A = [rng.normal(0.0, 1.0, sshape).astype(np.float32) for _ in range(3)]
        B = [rng.normal(0.0, 1.0, sshape).astype(np.float32) for _ in range(3)]
        m = [a.copy() for a in mom]
        blend, amp, dt = 0.37, 7.0, 1.3e-3
        N.drive.run(shape, [rho, m[0], m[1], m[2]] + A + B + [blend, amp, dt, dx, dxs])
        out[f"d_{tag}_A"], out[f"d_{tag}_B"] = np.stack(A), np.stack(B)
        out[f"d_{tag}_out"] = np.stack(m)
        out[f"d_{tag}_scalars"] = np.array([blend, amp, dt, dx, dxs], np.float64)
    out["d_rho"], out["d_mom"] = rho, mom
    # add_torus
    tq = (np.exp(rng.normal(0.0, 2.0, shape)) * (rng.random(shape) < 0.5)).astype(np.float32)
    r2, m2 = rho.copy(), [a.copy() for a in mom]
    S.add_torus.run(shape, [r2, m2[0], m2[1], m2[2], tq])
    out["a_torus"], out["a_rho"], out["a_mom"] = tq, r2, np.stack(m2)
    # the forcing generator on a seeded Generator, odd and even grid sizes
    for tag, sshape, kmax in (("odd", (7, 6, 5), 4.0), ("even", (8, 6, 10), 6.0)):
        g = np.random.default_rng(4242)
        v = N.solenoidal(sshape, g, 1.0, kmax)
        out[f"sol_{tag}"] = np.stack(v)
        out[f"sol_{tag}_next"] = g.standard_normal(4)          # the Generator state it leaves behind
    return out


def sim_pre_case(S, scenario, res, overrides, nsteps, rays, fuv, ic_mode):
    """a reference Sim through the stirring phase and into the main phase (sim.py:1044-1059, 1099-1114)"""
    P = S.make_params(scenario, overrides)
    sim = S.Sim(scenario, res=res, params=P, ic_mode=ic_mode, rays=rays, fuv_grid=fuv, device="cpu",
                verbose=False, fast=True)
    print(f"  {scenario} {sim.shape} phase {sim.phase}, {len(sim.stars)} stars", flush=True)
    fields = []                                    # every forcing field the run drew, in order

    def note():
        for F in (sim.drv["A"], sim.drv["B"]) if sim.drv else ():
            a = np.stack([c.numpy() for c in F])
            if not any(a.shape == f.shape and np.array_equal(a, f) for f in fields):
                fields.append(a)

    def snap():
        return dict(rho=sim.rho.numpy(), mx=sim.mx.numpy(), my=sim.my.numpy(), mz=sim.mz.numpy(),
                    xi=sim.xi.numpy(), dfront=sim.dfront.numpy())

    note()
    s0 = snap()
    meta = dict(scenario=scenario, res=res, shape=list(sim.shape), dx=sim.dx, L=list(sim.L), rays=list(rays),
                fuv=list(fuv), ion_every=sim.ion_every, fuv_every=sim.fuv_every,
                stars=[list(map(float, s)) for s in sim.stars], kinds=list(sim.kinds),
                jets=[list(map(float, j)) for j in sim.jets], jkinds=list(sim.jkinds),
                P={k: v for k, v in sim.P.items() if isinstance(v, (int, float, str, bool, type(None), list))},
                sshape=list(sim.sshape), dxs=sim.dxs, cn2=sim.cn2, ci2=sim.ci2, steps=[])
    out = {"rho_ic": s0["rho"], "torus": sim.torus0}
    for k, v in s0.items():
        out[f"s0_{k}"] = v
    for n in range(nsteps):
        sim.step(1)
        note()
        for k, v in snap().items():
            out[f"s{n + 1}_{k}"] = v
        d = sim.drv
        meta["steps"].append(dict(t=sim.t, it=sim.it, tp=sim.tp, ip=sim.ip, dt=sim.dt, phase=sim.phase,
                                  clock=None if d is None else d["clock"], mach=sim.mach))
        print(f"    step {n}: phase {sim.phase} tp={sim.tp:.5g} t={sim.t:.5g} dt={sim.dt:.5g} "
              f"clock={None if d is None else round(d['clock'], 5)} fields={len(fields)}", flush=True)
    out["fields"] = np.stack(fields)
    out["meta"] = np.array(json.dumps(meta))
    return out


# ----------------------------------------------------------------------------- bake.py's loop
def _json_safe(v):
    if isinstance(v, dict):
        return {k: _json_safe(x) for k, x in v.items()}
    if isinstance(v, (list, tuple)):
        return [_json_safe(x) for x in v]
    if isinstance(v, (np.floating, np.integer)):
        return v.item()
    return v


def ref_state(sim):
    """everything Sim.from_reference reads from a reference Sim: arrays apart, the rest as JSON"""
    meta = sim.get_state_meta()
    meta["sm0"] = None          # the triggered-formation reference field: unused with the trigger off
    d = meta.pop("drv")
    arrays = {"rho": sim.rho.numpy(), "mx": sim.mx.numpy(), "my": sim.my.numpy(), "mz": sim.mz.numpy(),
              "xi": sim.xi.numpy(), "dfront": sim.dfront.numpy(), "g0": sim.g0.numpy()}
    if sim.torus0 is not None:
        arrays["torus0"] = np.asarray(sim.torus0, np.float32)
    if d is not None:
        arrays["drv_A"] = np.stack([c.numpy() for c in d["A"]])
        arrays["drv_B"] = np.stack([c.numpy() for c in d["B"]])
    attrs = dict(scenario=sim.scenario, res=sim.res, shape=list(sim.shape), dx=sim.dx, fast=sim.fast,
                 ic_mode=sim.ic_mode, phase=sim.phase, rfront_shape=list(sim.rfront.shape),
                 att_shape=list(sim.att.shape), ion_every=sim.ion_every, fuv_every=sim.fuv_every,
                 sshape=list(sim.sshape), dxs=sim.dxs, stars=[list(map(float, x)) for x in sim.stars],
                 kinds=list(sim.kinds), jets=[list(map(float, j)) for j in sim.jets], jkinds=list(sim.jkinds),
                 P=dict(sim.P), events=[list(e) for e in sim.events], version=sim.version,
                 rf_version=sim.rf_version, fuv_version=sim.fuv_version,
                 fuv_nstars=getattr(sim, "fuv_nstars", -1), fuv_phase=getattr(sim, "fuv_phase", None),
                 dt_cap=sim.dt_cap,
                 noise=None if sim.noise is None else dict(seed=sim.noise.seed, calls=sim.noise.calls, K=sim.noise.K),
                 drv_clock=None if d is None else d["clock"], meta=meta)
    return arrays, _json_safe(attrs)


BAKE_CASES = {
    # stirring phase (matched forcing spectrum), jets, a later proto-star birth with a jet
    "bipolar": dict(overrides=dict(pre_t=0.49, pre_corr=0.02, pre_amp=7.0, seed=21, jet_r=0.35, jet_angle=35.0,
                                   clumps=0),
                    t_end=0.12, frames=4, birth=([0.55, 0.45, 0.5], 2.0e-4, 0.03, [0.0, 0.6, 0.8], "proto"),
                    events=[[0.02, "wind", 0.6], [0.05, "q_main", 1.5], [0.08, "jet", 2.0]]),
    # straight into the main phase, six stars with winds, the preset's triggered formation on at
    # construction (bake.py turns it off), a later birth without a jet
    "bubbles": dict(overrides=dict(seed=5, min_sep=0.2), t_end=0.16, frames=5,
                    birth=([0.3, 0.6, 0.4], 5.0e-5, 0.05, [0.0, 0.0, 1.0], "none"),
                    events=[[0.03, "wind", 0.8], [0.09, "q_main", 0.7]]),
    # the cloud wall lit from above: main stars kept wherever they are (above the gas, possibly
    # outside the box), embedded stars, globules on the wall's face
    "cliff": dict(overrides=dict(seed=9), t_end=0.1, frames=4,
                  birth=([0.5, 0.2, 0.5], 1.0e-4, 0.04, [0.0, 1.0, 0.0], "jet"),
                  events=[[0.02, "wind", 0.6], [0.06, "q_main", 1.3]]),
}


def bake_case(S, scen="bipolar", res=8):
    """bake.py:59-114 run by the reference on a small preset scene: Sim(..., fast=False) in the
    default matched mode (forcing fields from the matched spectrum); the stirring steps if the
    preset has a stirring phase; replace_stars with the preview's list plus a later birth; the live
    events replayed into P at their times (q_main as a factor of the preset's); at each frame time
    update_render_fields(force=True) and the frame expressions of bake.py:95-102; dt_cap landing
    the steps on the frame times.  Saves the reference Sim as constructed (what
    Sim.from_reference reads) and every frame."""
    c = BAKE_CASES[scen]
    P = S.make_params(scen, c["overrides"])
    t_end, frames = c["t_end"], c["frames"]
    sim = S.Sim(scen, res=res, params=P, ic_mode="matched", rays=(8, 16), fuv_grid=(6, 8, 16), fast=False,
                device="cpu", verbose=False)
    arrays, attrs = ref_state(sim)
    print(f"  {scen} {sim.shape} phase {sim.phase}, {len(sim.stars)} stars, noise calls {sim.noise.calls}", flush=True)
    sim.P["trigger"] = 0.0                                                    # bake.py:61-63
    while sim.phase == "pre":                                                 # bake.py:67-68
        sim.step(1)
    pre_steps = sim.ip
    stars = [list(map(float, x)) for x in sim.stars]
    L = sim.L
    pos, q_abs, t_on, axis, jkind = c["birth"]
    stars.append([pos[0] * L[0], pos[1] * L[1], pos[2] * L[2], q_abs, t_on])  # a later birth, absolute Q
    kinds = list(sim.kinds) + ["abs"]
    jets = [list(map(float, j)) for j in sim.jets] + [list(axis)]
    jkinds = list(sim.jkinds) + [jkind]
    sim.replace_stars(stars, kinds, jets, jkinds)                             # bake.py:69
    events = [[t, name, float(P["q_main"]) * v if name == "q_main" else v] for t, name, v in c["events"]]
    out = {f"s_{k}": v for k, v in arrays.items()}
    dt_frame = t_end / max(frames - 1, 1)
    next_frame, frame, ev_i, times = 0.0, 0, 0, []
    while True:                                                               # bake.py:87-114
        while ev_i < len(events) and events[ev_i][0] <= sim.t + 1e-12:
            _, name, val = events[ev_i]
            sim.P[name] = val
            sim._wkey = None
            ev_i += 1
        if sim.t >= next_frame - 1e-9:
            sim.update_render_fields(force=True)
            out[f"f{frame}_g0"] = np.minimum(sim.g0.numpy(), 6e4).astype(np.float16)
            out[f"f{frame}_rho"] = sim.rho.numpy().astype(np.float16)
            out[f"f{frame}_xi"] = np.round(np.clip(sim.xi.numpy(), 0, 1) * 255).astype(np.uint8)
            out[f"f{frame}_df"] = np.clip(sim.dfront.numpy(), -4, 4).astype(np.float16)
            out[f"f{frame}_sh"] = np.minimum(sim.shock.numpy(), 6e4).astype(np.float16)
            times.append(sim.t)
            print(f"    frame {frame} t={sim.t:.5f} step {sim.it}", flush=True)
            frame += 1
            next_frame += dt_frame
            if frame >= frames:
                break
        sim.dt_cap = next_frame - sim.t + 1e-7
        sim.step(1)
    attrs["bake"] = dict(t_end=t_end, frames=frames, stars=stars, kinds=kinds, jets=jets, jkinds=jkinds, events=events,
                         times=times, steps=sim.it, pre_steps=pre_steps, mach=sim.mach)
    out["meta"] = np.array(json.dumps(_json_safe(attrs)))
    print(f"  bake: {pre_steps} stirring steps, {sim.it} main steps, {frame} frames", flush=True)
    return out


# ----------------------------------------------------------------------------- renderer pack
def render_cases(ref, rng):
    """render.py:176-205 pack_volume_lm (RGBA16F voxel: emission rgb + dust, shock proxy inline,
    box-edge fade) and render.py:281-298 smooth_axis ([1 4 1]/6 along each axis, three passes)"""
    sys.path.insert(0, ref)
    import types
    import render as R
    shape = (10, 9, 8)
    dx = 0.125
    L = tuple(n * dx for n in shape)
    rho = np.exp(rng.normal(0.0, 1.5, shape)).astype(np.float32) + np.float32(0.01)
    rho.flat[:2] = [3e3, 0.05]
    mom = (rng.normal(0.0, 2.0, (3,) + shape) * rho).astype(np.float32)
    xi = rng.uniform(-0.2, 1.2, shape).astype(np.float32)
    df = rng.uniform(-0.2, 0.1, shape).astype(np.float16)
    df[rng.random(shape) < 0.15] = np.float16(1e3)
    g0 = np.exp(rng.normal(0.0, 3.0, shape)).astype(np.float16)
    g0.flat[:2] = [np.float16(65504.0), np.float16(0.0)]
    out = {"p_rho": rho, "p_mom": mom, "p_xi": xi, "p_df": df, "p_g0": g0, "p_dx": np.float64(dx)}
    fake = types.SimpleNamespace(L=L, dx=dx)
    cases = (("jwst", dict(R.make_look("bipolar"), shock=0.002, edge_fade=0.3), 1),
             ("sho", dict(R.make_look("bubbles"), palette="sho", edge_fade=0.0), 0),
             ("nat", dict(R.make_look("cliff"), palette="natural", gs=12.0, edge_fade=0.08), 1))
    for tag, look, shock_on in cases:
        pp = R.Renderer.pack_params(look, fake)
        o = np.zeros(shape + (4,), np.float16)
        R.pack_volume_lm.run(shape, [rho, mom[0], mom[1], mom[2], xi, df, g0, pp, shock_on, o])
        a, b = o.copy(), np.zeros_like(o)
        for ax in range(3):                                   # render.py:725-728
            src, dst = (a, b) if ax != 1 else (b, a)
            R.smooth_axis.run(shape, [src, dst, ax])
        out[f"p_{tag}_params"] = np.array(
            list(pp.c_ha) + list(pp.c_o3) + list(pp.c_s2) + list(pp.c_dg) + list(pp.c_sh) +
            [pp.gs, pp.ambient, pp.edge] + list(pp.inv_L) + [pp.dx, shock_on], np.float32)
        out[f"p_{tag}_packed"] = o
        out[f"p_{tag}_smooth"] = b
        print(f"  pack {tag}: max {float(np.abs(o.astype(np.float32)).max()):.4g}", flush=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("NEBULA_REFERENCE"),
                    help="the reference checkout (default: $NEBULA_REFERENCE)")
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    if not a.ref:
        ap.error("give the reference checkout with --ref or NEBULA_REFERENCE")
    N, S = import_reference(a.ref)
    rng = np.random.default_rng(20261203)
    if a.only in (None, "kernels"):
        print("kernels:", flush=True)
        np.savez_compressed(os.path.join(HERE, "kernels.npz"), **kernel_cases(N, S, rng))
    if a.only in (None, "render"):
        print("render:", flush=True)
        np.savez_compressed(os.path.join(HERE, "render.npz"), **render_cases(a.ref, np.random.default_rng(77)))
    if a.only in (None, "stir"):
        print("stir:", flush=True)
        np.savez_compressed(os.path.join(HERE, "stir.npz"), **stir_cases(N, S, np.random.default_rng(515)))
    if a.only in (None, "bipolar_pre"):
        print("sim bipolar_pre:", flush=True)
        c = dict(scenario="bipolar", res=8, overrides=dict(pre_t=0.49, pre_corr=0.02, pre_amp=7.0, drive_main=0.5,
                                                            seed=13, jet_r=0.35, jet_angle=35.0, clumps=0),
                 nsteps=14, rays=(8, 16), fuv=(6, 8, 16), ic_mode="nebula3d")   # 6-cell forcing grid
        np.savez_compressed(os.path.join(HERE, "sim_bipolar_pre.npz"), **sim_pre_case(S, **c))
    for scen in BAKE_CASES:
        if a.only in (None, "bake", f"bake_{scen}"):
            print(f"bake {scen}:", flush=True)
            np.savez_compressed(os.path.join(HERE, f"bake_{scen}.npz"), **bake_case(S, scen))
    if a.only in (None, "timeline"):
        print("timeline:", flush=True)
        np.savez_compressed(os.path.join(HERE, "timeline.npz"), **timeline_cases(a.ref, np.random.default_rng(99)))
    cases = {
        # bubbles: 6 stars, wind, HLL + minmod, fast-mode budgets (dr = dx, ionize every 3 steps)
        "bubbles": dict(scenario="bubbles", res=8, overrides=dict(pre_t=0.0, trigger=0.0, seed=5, min_sep=0.2),
                        nsteps=6, fast=True, rays=(8, 16), fuv=(6, 8, 16)),
        # bipolar: jets (cone widened to reach cell centres at this resolution), wind, q ramp, MC limiter,
        # bake-mode budgets (dr = dx/2, ionize every 2 steps), and one dt_cap step
        "bipolar": dict(scenario="bipolar", res=8, overrides=dict(pre_t=0.0, seed=7, jet_r=0.35, jet_angle=35.0,
                                                                  limiter="mc", clumps=0),
                        nsteps=3, fast=False, rays=(8, 16), fuv=(6, 8, 16), dt_cap_at=1),
        # cliff: Rusanov solver, embedded stars that switch on later, van Leer is ignored by Rusanov
        "cliff": dict(scenario="cliff", res=8, overrides=dict(pre_t=0.0, seed=11, solver="rusanov", n_embedded=2,
                                                              globules=10),
                      nsteps=3, fast=True, rays=(8, 16), fuv=(6, 8, 16), ion_every=2),
    }
    for name, c in cases.items():
        if a.only not in (None, name):
            continue
        print(f"sim {name}:", flush=True)
        np.savez_compressed(os.path.join(HERE, f"sim_{name}.npz"), **sim_case(S, **c))
    print("done")


if __name__ == "__main__":
    main()

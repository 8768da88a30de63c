"""CPU oracle of the simulation step: TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, as
the reference to check against; the product (nebulaviewer_gb300) never imports it.

* `Kernels(dtype)`: ctypes access to oracle/ref_cpu.cpp, a line-by-line C++ restatement
  of the reference's Warp kernels (nebula3d.py / sim.py; each function cites its lines),
  in float32 (the parity oracle) or float64 (the FP64 re-run of the same scheme).
* `OracleSim`: a restatement of the reference `Sim` driver (sim.py:880-1152: star weights,
  ionize, fuv_field, _compute_dt, _hydro, _main_step, step, update_render_fields) over
  those kernels, on host numpy arrays in the reference's layout.

Pinned against tests/golden/ (fixtures made by running the reference's own kernel source
and its own `Sim` driver on small inputs): hydro bit for bit, rays / FUV to float32
rounding of the transcendental functions.
"""
import ctypes as C
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build as _build  # noqa: E402

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build(verbose=False)
        L = C.CDLL(path)
        P = C.c_void_p
        for sfx, T in (("f32", C.c_float), ("f64", C.c_double)):
            getattr(L, f"oracle_hydro_stage_{sfx}").argtypes = [C.c_int] * 3 + [P] * 13 + [P, C.c_int, T, P] + \
                [T] * 11 + [C.c_int, C.c_int]
            getattr(L, f"oracle_max_speed_{sfx}").argtypes = [C.c_int] * 3 + [P] * 5 + [T, T]
            getattr(L, f"oracle_max_speed_{sfx}").restype = T
            getattr(L, f"oracle_cast_rays_{sfx}").argtypes = [C.c_int] * 3 + [P, P, T, T, C.c_int, T, T, P,
                                                                            C.c_int, C.c_int, P]
            getattr(L, f"oracle_apply_front_{sfx}").argtypes = [C.c_int] * 3 + [P, C.c_int, C.c_int, P, T, T, P, P]
            getattr(L, f"oracle_smooth_xi_{sfx}").argtypes = [C.c_int] * 3 + [P, P]
            getattr(L, f"oracle_cast_fuv_{sfx}").argtypes = [C.c_int] * 3 + [P, P, P, T, T, C.c_int, T, T, P,
                                                                           C.c_int, C.c_int, C.c_int, P]
            getattr(L, f"oracle_apply_fuv_{sfx}").argtypes = [C.c_int] * 3 + [P, C.c_int, C.c_int, C.c_int, P, T, T,
                                                                            T, P]
            getattr(L, f"oracle_plane_front_{sfx}").argtypes = [C.c_int] * 3 + [P, T, T, T, P]
            getattr(L, f"oracle_apply_plane_{sfx}").argtypes = [C.c_int] * 3 + [P, T, T, P, P]
            getattr(L, f"oracle_plane_fuv_{sfx}").argtypes = [C.c_int] * 3 + [P, P, T, T, T, P]
            getattr(L, f"oracle_drive_{sfx}").argtypes = [C.c_int] * 3 + [P] * 4 + [C.c_int] * 3 + [P, P] + [T] * 5
            getattr(L, f"oracle_add_torus_{sfx}").argtypes = [C.c_long] + [P] * 5
        L.oracle_to_half.argtypes = [P, P, C.c_long]
        L.oracle_render_pack.argtypes = [C.c_int] * 3 + [P] * 8 + [C.c_int, P]
        L.oracle_render_smooth.argtypes = [C.c_int] * 3 + [P, P, C.c_int]
        L.oracle_threads.restype = C.c_int
        _LIB = L
    return _LIB


def threads():
    return lib().oracle_threads()


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Kernels:
    """The reference kernels in dtype (np.float32 = oracle, np.float64 = FP64 re-run)."""

    def __init__(self, dtype=np.float32):
        self.dt = np.dtype(dtype)
        self.sfx = "f32" if self.dt == np.float32 else "f64"
        self.L = lib()

    def _a(self, a):
        a = np.ascontiguousarray(a, dtype=self.dt)
        return a

    def _fn(self, name):
        return getattr(self.L, f"oracle_{name}_{self.sfx}")

    # nebula3d.py:76-151 / sim.py:423-498
    def hydro_stage(self, U, xi, U0, out, stars, nstars, wind, jets, jet_cos, jet_r, pulse, dt, dx, a, b, floor_,
                    cn2, ci2, vmax, solver, lim):
        nx, ny, nz = U[0].shape
        ins = [self._a(x) for x in U] + [self._a(xi)]
        u0 = [self._a(x) for x in U0]
        for o in out:
            assert o.dtype == self.dt and o.flags.c_contiguous
        st = self._a(np.asarray(stars).reshape(-1, 4))
        jt = self._a(np.asarray(jets).reshape(-1, 4))
        self._fn("hydro_stage")(nx, ny, nz, *[_p(x) for x in ins], *[_p(x) for x in u0], *[_p(o) for o in out],
                                _p(st), int(nstars), wind, _p(jt), jet_cos, jet_r, pulse, dt, dx, a, b, floor_, cn2,
                                ci2, vmax, int(solver), int(lim))
        # keep inputs alive until the call returns
        return out

    def max_speed(self, rho, mx, my, mz, xi, cn2, ci2):
        nx, ny, nz = rho.shape
        a = [self._a(x) for x in (rho, mx, my, mz, xi)]
        return float(self._fn("max_speed")(nx, ny, nz, *[_p(x) for x in a], cn2, ci2))

    def cast_rays(self, rho, star, Q, dr, nsteps, dx, rcap, bmax, nu, nphi):
        nx, ny, nz = rho.shape
        r = self._a(rho)
        s = self._a(np.asarray(star, np.float64).astype(self.dt))
        bm = self._a(np.asarray(bmax, np.float64).astype(self.dt))
        out = np.zeros((nu, nphi), self.dt)
        self._fn("cast_rays")(nx, ny, nz, _p(r), _p(s), Q, dr, int(nsteps), dx, rcap, _p(bm), int(nu), int(nphi),
                              _p(out))
        return out

    def apply_front(self, rfront, star, dx, width, xi, dfront):
        nx, ny, nz = xi.shape
        rf = self._a(rfront)
        s = self._a(np.asarray(star, np.float64).astype(self.dt))
        assert xi.dtype == self.dt and dfront.dtype == self.dt
        self._fn("apply_front")(nx, ny, nz, _p(rf), rf.shape[0], rf.shape[1], _p(s), dx, width, _p(xi), _p(dfront))

    def smooth_xi(self, src):
        nx, ny, nz = src.shape
        s = self._a(src)
        out = np.zeros_like(s)
        self._fn("smooth_xi")(nx, ny, nz, _p(s), _p(out))
        return out

    def cast_fuv(self, rho, xi, star, kappa, dr, nsteps, dx, binr, bmax, nr, nu, nphi):
        nx, ny, nz = rho.shape
        r, x = self._a(rho), self._a(xi)
        s = self._a(np.asarray(star, np.float64).astype(self.dt))
        bm = self._a(np.asarray(bmax, np.float64).astype(self.dt))
        out = np.zeros((nr, nu, nphi), self.dt)
        self._fn("cast_fuv")(nx, ny, nz, _p(r), _p(x), _p(s), kappa, dr, int(nsteps), dx, binr, _p(bm), int(nr),
                             int(nu), int(nphi), _p(out))
        return out

    def apply_fuv(self, att, star, lum, dx, binr, g0):
        nx, ny, nz = g0.shape
        a = self._a(att)
        s = self._a(np.asarray(star, np.float64).astype(self.dt))
        assert g0.dtype == self.dt
        self._fn("apply_fuv")(nx, ny, nz, _p(a), a.shape[0], a.shape[1], a.shape[2], _p(s), lum, dx, binr, _p(g0))


    # the -x plane-parallel source (no reference counterpart)
    def plane_front(self, rho, F, dx, rcap):
        nx, ny, nz = rho.shape
        r = self._a(rho)
        out = np.zeros((ny, nz), self.dt)
        self._fn("plane_front")(nx, ny, nz, _p(r), F, dx, rcap, _p(out))
        return out

    def apply_plane(self, xf, dx, width, xi, dfront):
        nx, ny, nz = xi.shape
        x = self._a(xf)
        assert xi.dtype == self.dt and dfront.dtype == self.dt
        self._fn("apply_plane")(nx, ny, nz, _p(x), dx, width, _p(xi), _p(dfront))

    def plane_fuv(self, rho, xi, kappa, lum, dx):
        nx, ny, nz = rho.shape
        r, x = self._a(rho), self._a(xi)
        out = np.zeros(rho.shape, self.dt)
        self._fn("plane_fuv")(nx, ny, nz, _p(r), _p(x), kappa, lum, dx, _p(out))
        return out


    # nebula3d.py:165-179 drive (momenta updated in place); fa / fb: [3][sx][sy][sz]
    def drive(self, rho, mx, my, mz, fa, fb, blend, amp, dt, dx, dxs):
        nx, ny, nz = rho.shape
        for m in (mx, my, mz):
            assert m.dtype == self.dt and m.flags.c_contiguous
        r, a, b = self._a(rho), self._a(fa), self._a(fb)
        sx, sy, sz = a.shape[1:]
        self._fn("drive")(nx, ny, nz, _p(r), _p(mx), _p(my), _p(mz), sx, sy, sz, _p(a), _p(b), blend, amp, dt, dx,
                          dxs)

    # sim.py:352-363 add_torus (fields updated in place)
    def add_torus(self, torus, rho, mx, my, mz):
        for m in (rho, mx, my, mz):
            assert m.dtype == self.dt and m.flags.c_contiguous
        t = self._a(torus)
        self._fn("add_torus")(rho.size, _p(t), _p(rho), _p(mx), _p(my), _p(mz))


def render_pack(rho, mom, xi, df16, g016, params, shock_on, smooth=True):
    """render.py:176-205 pack_volume_lm (+ render.py:281-298 smooth_axis x, y, z when `smooth`):
    float16 (nx, ny, nz, 4) voxels.  params: the 22 PackParams floats (c_ha, c_o3, c_s2, c_dg,
    c_sh, gs, ambient, edge, inv_L, dx)."""
    L = lib()
    f = lambda a: np.ascontiguousarray(a, np.float32)  # noqa: E731
    h = lambda a: np.ascontiguousarray(np.asarray(a, np.float16)).view(np.uint16)  # noqa: E731
    r, x, m = f(rho), f(xi), [f(v) for v in mom]
    d, g, pp = h(df16), h(g016), f(np.asarray(params, np.float32)[:22])
    nx, ny, nz = r.shape
    out = np.zeros((nx, ny, nz, 4), np.uint16)
    L.oracle_render_pack(nx, ny, nz, _p(r), _p(m[0]), _p(m[1]), _p(m[2]), _p(x), _p(d), _p(g), _p(pp), int(shock_on),
                         _p(out))
    if smooth:
        tmp = np.zeros_like(out)
        for ax in range(3):                                         # render.py:725-728
            src, dst = (out, tmp) if ax != 1 else (tmp, out)
            L.oracle_render_smooth(nx, ny, nz, _p(src), _p(dst), ax)
        out = tmp
    return out.view(np.float16)


def to_half(x):
    """sim.py:511-514 to_half (round to nearest even) restated in C."""
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros(x.shape, np.uint16)
    lib().oracle_to_half(_p(x), _p(out), x.size)
    return out.view(np.float16)


# ----------------------------------------------------------------------------- the Sim driver
class OracleSim:
    """sim.py Sim's driver restated over the oracle kernels (host numpy state): the stirring
    phase (sim.py:1030-1059), its end (sim.py:806-818) and the main phase (sim.py:1099-1114).

    Inputs mirror what reset() leaves behind (sim.py:591-795): the grid, the fields, the
    star / jet lists with their kinds, the parameter dict P and the ray budgets; with
    P['pre_t'] > 0 also the torus that joins at the end of the stirring phase, the forcing
    fields in order of use ([3][sx][sy][sz] arrays) and the forcing grid ((sx, sy, sz), dxs)."""

    def __init__(self, shape, dx, rho, stars, kinds, jets, jkinds, P, rays=None, fuv_grid=None, ion_every=None,
                 fast=True, mom=None, dtype=np.float32, start_main=True, cn2=None, ci2=None, vmax=None,
                 torus=None, stir_fields=None, stir_grid=None):
        self.K = Kernels(dtype)
        self.T = np.dtype(dtype)
        self.shape = tuple(int(v) for v in shape)
        nx, ny, nz = self.shape
        self.dx = float(dx)
        self.L = (nx * self.dx, ny * self.dx, nz * self.dx)
        self.P = dict(P)
        self.rho = np.array(rho, dtype=self.T)
        z = lambda: np.zeros(self.shape, self.T)  # noqa: E731
        if mom is None:
            self.mx, self.my, self.mz = z(), z(), z()
        else:
            self.mx, self.my, self.mz = (np.array(m, dtype=self.T) for m in mom)
        self.xi = z()
        self.stage = np.zeros((4,) + self.shape, self.T)
        half = self.T == np.float32 and not self.P.get("fp32_fields")
        self.hdt = np.float16 if half else self.T
        self.dfront = np.full(self.shape, 1e3, self.hdt)
        self.g0 = np.zeros(self.shape, self.hdt)
        self.stars = [tuple(float(v) for v in s) for s in stars]
        self.kinds = list(kinds)
        self.jets = [tuple(float(v) for v in j[:3]) for j in jets]
        self.jkinds = list(jkinds)
        self.cn2 = cn2 if cn2 is not None else (1.0 / self.P["ci_over_cn"]) ** 2      # sim.py:740
        self.ci2 = ci2 if ci2 is not None else 1.0                                     # sim.py:741
        self.vmax = vmax if vmax is not None else 6.0                                  # sim.py:1020
        Lx, Ly, Lz = self.L
        self.diag = math.sqrt(Lx ** 2 + Ly ** 2 + Lz ** 2) + 0.6                       # sim.py:742
        self.fast = fast
        self.dr = (1.0 if fast else 0.5) * self.dx                                     # sim.py:743
        self.nsteps = int(self.diag / self.dr) + 1
        self.cap = max(len(self.stars), self.P["max_stars"])
        nu = rays[0] if rays else (512 if nz <= 256 else 1024)                          # sim.py:753-754
        nphi = rays[1] if rays else 2 * nu
        self.rays = (nu, nphi)
        self.fuv = tuple(fuv_grid) if fuv_grid else \
            ((128, 128, 256) if nz <= 192 else ((160, 160, 320) if nz <= 256 else (256, 256, 512)))
        self.ion_every = ion_every or (max(self.P["ion_every"], 3) if fast else self.P["ion_every"])
        self.fuv_every = (8 if nz <= 160 else 16) if fast else 8
        self.bmax = (Lx, Ly, Lz)
        self.t, self.it, self.dt = 0.0, 0, 0.0
        self.tp, self.ip, self.mach = 0.0, 0, None
        self.version, self.rf_version, self.fuv_version = 0, -1, -10 ** 9
        self.dt_cap = None
        self.star_arr = np.zeros((self.cap, 4), np.float32)
        self.jet_arr = np.zeros((self.cap, 4), np.float32)
        pre = float(self.P.get("pre_t", 0.0) or 0.0) > 0.0
        self.torus = None
        if torus is not None:
            if pre:
                self.torus = np.array(torus, dtype=self.T)
            else:
                self.rho += np.asarray(torus, dtype=self.T)
        self._src = None if stir_fields is None else [np.asarray(f, dtype=self.T) for f in stir_fields]
        if stir_grid is not None:
            self.sshape, self.dxs = tuple(stir_grid[0]), float(stir_grid[1])
        self.drv = None
        self.phase = "pre" if pre else "main"
        if pre:
            self.drv = {"A": self._mkF(), "B": self._mkF(), "clock": 0.0}          # sim.py:786-788
        elif start_main:
            self._start_main()

    # sim.py:880-902
    def q_of(self, i):
        s = self.stars[i]
        return s[3] * self.P["q_main"] if self.kinds[i] == "main" else s[3]

    def ramp(self, i):
        age = self.t - self.stars[i][4]
        if self.phase != "main" or age < 0.0:
            return 0.0
        tr = float(self.P.get("q_ramp", 0.0))
        if tr <= 0.0 or age >= tr:
            return 1.0
        x = age / tr
        s = x * x * (3.0 - 2.0 * x)
        return max(s * s * s, 1e-4)

    def q_eff(self, i):
        return self.q_of(i) * self.ramp(i)

    def jet_of(self, i):
        k = self.jkinds[i]
        return self.P["jet"] if k == "jet" else (self.P["jet_proto"] if k == "proto" else 0.0)

    def _set_star_weights(self):                                   # sim.py:914-925
        qm = self.P["q_main"]
        w = [(s[0], s[1], s[2], (self.q_eff(i) / qm) if self.t >= s[4] else 0.0) for i, s in enumerate(self.stars)]
        w += [(0.0, 0.0, 0.0, 0.0)] * (self.cap - len(w))
        self.star_arr = np.array(w, dtype=np.float32)
        jw = [(a[0], a[1], a[2], self.jet_of(i)) for i, a in enumerate(self.jets)]
        jw += [(0.0, 0.0, 1.0, 0.0)] * (self.cap - len(jw))
        self.jet_arr = np.array(jw, dtype=np.float32)

    def _store(self, src, dst):                                    # sim.py:980-985
        dst[...] = to_half(src) if dst.dtype == np.float16 else src

    def ionize(self):                                              # sim.py:927-947
        df = self.stage[1]
        self.xi[...] = 0
        df[...] = 1e3
        nu, nphi = self.rays
        for i, (sx, sy, sz, _, ton) in enumerate(self.stars):
            if self.t < ton:
                continue
            rf = self.K.cast_rays(self.rho, (sx, sy, sz), self.q_eff(i), self.dr, self.nsteps, self.dx, self.diag,
                                  self.bmax, nu, nphi)
            self.rfront = rf
            self.K.apply_front(rf, (sx, sy, sz), self.dx, 1.2 * self.dx, self.xi, df)
        F = float(self.P.get("plane_flux", 0.0) or 0.0)
        if F > 0.0:
            xf = self.K.plane_front(self.rho, F, self.dx, self.diag)
            self.K.apply_plane(xf, self.dx, 1.2 * self.dx, self.xi, df)
        self.xi[...] = self.K.smooth_xi(self.xi)
        self._store(df, self.dfront)

    def fuv_field(self):                                           # sim.py:949-985
        if self.phase != "main":
            self.g0[...] = 0
            return
        acc = self.stage[2]
        acc[...] = 0
        fnr, fnu, fnp = self.fuv
        binr = self.diag / fnr
        for i, (sx, sy, sz, _, ton) in enumerate(self.stars):
            if self.t < ton:
                continue
            att = self.K.cast_fuv(self.rho, self.xi, (sx, sy, sz), self.P["kappa_fuv"], self.dr, self.nsteps,
                                  self.dx, binr, self.bmax, fnr, fnu, fnp)
            self.att = att
            self.K.apply_fuv(att, (sx, sy, sz), self.q_eff(i) / self.P["q_main"], self.dx, binr, acc)
        if float(self.P.get("plane_flux", 0.0) or 0.0) > 0.0:
            acc += self.K.plane_fuv(self.rho, self.xi, self.P["kappa_fuv"], float(self.P.get("plane_fuv", 0.0)),
                                    self.dx)
        self._store(acc, self.g0)

    def update_render_fields(self, force=False):                   # sim.py:989-1007
        if self.rf_version == self.version and not force:
            return False
        n_on = sum(1 for s in self.stars if self.t >= s[4])
        tr = float(self.P.get("q_ramp", 0.0))
        ramping = tr > 0 and any(0.0 <= self.t - s[4] < tr for s in self.stars)
        if ramping and self.version - self.fuv_version >= max(2, self.fuv_every // 4):
            force = True
        if (force or self.version - self.fuv_version >= self.fuv_every
                or n_on != getattr(self, "fuv_nstars", -1) or self.phase != getattr(self, "fuv_phase", None)):
            self.fuv_field()
            self.fuv_version, self.fuv_nstars, self.fuv_phase = self.version, n_on, self.phase
        self.rf_version = self.version
        return True

    def _compute_dt(self):                                         # sim.py:1009-1012
        smax = self.K.max_speed(self.rho, self.mx, self.my, self.mz, self.xi, self.cn2, self.ci2)
        return self.P["cfl"] * self.dx / smax

    def _hydro(self, dt, nstars, wind, pulse):                     # sim.py:1014-1028
        P = self.P
        hll = P.get("solver", "rusanov") == "hll"
        lim = {"minmod": 0, "vanleer": 1, "mc": 2}[P.get("limiter", "minmod")] if hll else 0
        jet_cos = math.cos(math.radians(P["jet_angle"]))
        U = [self.rho, self.mx, self.my, self.mz]
        U1 = [self.stage[c] for c in range(4)]
        common = dict(stars=self.star_arr, nstars=nstars, wind=wind, jets=self.jet_arr, jet_cos=jet_cos,
                      jet_r=P["jet_r"], pulse=pulse, dt=dt, dx=self.dx, floor_=P["floor"], cn2=self.cn2,
                      ci2=self.ci2, vmax=self.vmax, solver=1 if hll else 0, lim=lim)
        self.K.hydro_stage(U, self.xi, U, U1, a=0.0, b=1.0, **common)
        # stage 2 in place: every cell reads its own U^n before writing it
        self.K.hydro_stage(U1, self.xi, U, U, a=0.5, b=0.5, **common)

    def _main_step(self):                                          # sim.py:1099-1114
        P = self.P
        if self.it % self.ion_every == 0:
            self.ionize()
        self._set_star_weights()
        dt = self._compute_dt()
        if self.dt_cap is not None:
            dt = min(dt, self.dt_cap)
        pulse = max(0.0, 1.0 + P["jet_pulse"] * math.sin(2 * math.pi * self.t / P["jet_period"]))
        self._hydro(dt, len(self.stars), P["wind"], pulse)
        if P.get("drive_main", 0.0) > 0 and self.drv is not None:
            self._stir(dt, P["pre_amp"] * P["drive_main"])
        self.t += dt
        self.it += 1
        self.dt = dt

    def step(self, k=1):                                           # sim.py:1141-1152
        for _ in range(k):
            if self.phase == "pre":
                self._pre_step()
            else:
                self._main_step()
            self.version += 1

    # ---- stirring
    def _mkF(self):                                                # sim.py:801-804 (fields given in order)
        if not self._src:
            raise RuntimeError("the oracle ran out of forcing fields")
        return self._src.pop(0)

    def _stir(self, dt, amp):                                      # sim.py:1030-1042
        d = self.drv
        blend = min(d["clock"] / self.P["pre_corr"], 1.0)
        self.K.drive(self.rho, self.mx, self.my, self.mz, d["A"], d["B"], blend, amp, dt, self.dx, self.dxs)
        d["clock"] += dt
        if d["clock"] >= self.P["pre_corr"]:
            d["A"], d["B"], d["clock"] = d["B"], self._mkF(), 0.0

    def _pre_step(self):                                           # sim.py:1044-1059
        dt = self._compute_dt()
        self._hydro(dt, 0, 0.0, 0.0)
        self._stir(dt, self.P["pre_amp"])
        self.tp += dt
        self.ip += 1
        self.dt = dt
        if self.tp >= self.P["pre_t"]:
            r = self.rho.astype(np.float64)
            m2 = (self.mx * self.mx + self.my * self.my + self.mz * self.mz) / self.rho
            self.mach = math.sqrt(float(m2.astype(np.float64).sum()) / float(r.sum())) * self.P["ci_over_cn"]
            if self.P["drive_main"] <= 0:
                self.drv = None
            self._start_main()

    def _start_main(self):                                         # sim.py:806-818
        if self.torus is not None:
            self.K.add_torus(self.torus, self.rho, self.mx, self.my, self.mz)
            self.torus = None
        self.phase = "main"
        self._set_star_weights()
        self.ionize()

"""`Sim`: the drop-in for the reference's GPU-resident simulation class (sim.py:543-1222)
on the simulation-step path, backed by libnebula.so (hand-written sm_103a kernels).

Same call surface as the reference for what viewer.py / bake.py / bench.py use on this
path: step(k), ionize(), fuv_field(), update_render_fields(force), set_param(), replace_stars(),
stars_absolute(), active_stars(), get_state_meta() / set_state_meta(), tau(), time_label(),
stats(), render_scratch(); attributes rho, mx, my, mz, xi, dfront, g0, stage, shape, dx, L,
t, it, dt, phase, P, prof, profile, dt_cap, version, rf_version, stars, kinds, jets, jkinds,
events, ion_every, fuv_every.  Fields are device buffers with the wp.array surface the
callers use (.numpy(), .shape, .dtype, .ptr, .fill_, .zero_, .assign, __cuda_array_interface__).

What differs by design: the clock (t, dt, it, tp, ip) lives on the device, so step(k)
enqueues k steps without a host round trip per step (the reference blocks on a max-speed
read every step, sim.py:1012); reading `t` synchronizes.  The stirring (pre-turbulence)
phase and main-phase stirring (sim.py:1030-1059, 1110-1111) run on the device too: the
cross-fade clock and the field swaps are evaluated there, and the host pushes forcing
fields into a device ring ahead of use, synchronizing once per chunk of steps that the CFL
bound dt <= cfl dx / c_n proves cannot end the phase or exhaust the ring.  Triggered star
formation and cropped domains are outside this package's scope: a parameter set that asks
for them is rejected.
"""
import collections
import copy
import ctypes as C
import math
import time

import numpy as np
import torch

from . import _lib
from . import ics as _ics
from . import stir as _stir
from .params import LIVE, make_params, sound_speeds

DRIVE_SLOTS = 16          # forcing fields the device ring holds
REFERENCE_PRESETS = ("bipolar", "bubbles", "cliff")      # sim.py:50-59 PRESETS
DRIVE_LOOKAHEAD = 2       # fields pushed beyond B before a chunk of stirred steps


class Field:
    """A device buffer (torch tensor) with the wp.array methods the reference's callers use."""

    def __init__(self, t):
        self.t = t

    @property
    def shape(self):
        return tuple(self.t.shape)

    @property
    def dtype(self):
        return np.dtype(str(self.t.dtype).replace("torch.", ""))

    @property
    def ptr(self):
        return self.t.data_ptr()

    @property
    def __cuda_array_interface__(self):
        return self.t.__cuda_array_interface__

    def numpy(self):
        return self.t.detach().cpu().numpy()

    def torch(self):
        return self.t

    def fill_(self, v):
        self.t.fill_(v)

    def zero_(self):
        self.t.zero_()

    def assign(self, x):
        self.t.copy_(torch.as_tensor(np.asarray(x)).reshape(self.t.shape).to(self.t.dtype))

    def __getitem__(self, k):
        return Field(self.t[k])

    def __repr__(self):
        return f"Field({self.shape}, {self.dtype}, {self.t.device})"


class _Shape:
    def __init__(self, shape):
        self.shape = tuple(shape)


def _ray_budget(nz, fast, rays, fuv_grid):
    nu = rays[0] if rays else (512 if nz <= 256 else 1024)                       # sim.py:753-754
    nphi = rays[1] if rays else 2 * nu
    fg = tuple(fuv_grid) if fuv_grid else \
        ((128, 128, 256) if nz <= 192 else ((160, 160, 320) if nz <= 256 else (256, 256, 512)))   # sim.py:756
    return (int(nu), int(nphi)), tuple(int(v) for v in fg)


def instance_desc(shape, dx, P, rays, fuv, fast, cap):
    """the library's description of an instance (nb_desc, without field pointers or stream): the
    values sim.py:Sim.reset computes for the grid, the physics and the ray / FUV budgets
    (sim.py:718-759)"""
    nx, ny, nz = (int(v) for v in shape)
    cn2, ci2, vmax = sound_speeds(P)
    L = (nx * dx, ny * dx, nz * dx)
    diag = math.sqrt(L[0] ** 2 + L[1] ** 2 + L[2] ** 2) + 0.6                          # sim.py:742
    dr = (1.0 if fast else 0.5) * dx                                                  # sim.py:743
    d = _lib.NbDesc()
    d.abi_version = _lib.NB_ABI_VERSION
    d.nx, d.ny, d.nz = nx, ny, nz
    d.dx = float(dx)
    d.cn2, d.ci2, d.vmax = cn2, ci2, vmax
    d.floor_rho = float(P["floor"])
    d.cfl = float(P["cfl"])
    d.solver = _lib.SOLVERS[P.get("solver", "rusanov")]
    d.limiter = _lib.LIMITERS[P.get("limiter", "minmod")]
    d.nu, d.nphi = (int(v) for v in rays)
    d.dr = dr
    d.nsteps = int(diag / dr) + 1                                                     # sim.py:744
    d.diag = diag
    d.fnr, d.fnu, d.fnphi = (int(v) for v in fuv)
    d.fields_fp32 = 1 if P.get("fp32_fields") else 0
    d.max_stars = min(256, max(int(cap), 1))
    return d


def field_bytes(shape, P):
    """device bytes of an instance's fields: rho, mx, my, mz, xi and the 4-plane stage block in
    float32, dfront and g0 in float16 (float32 with fp32_fields) -- the reference's 40 B/cell
    (sim.py:718-735)"""
    n = int(np.prod(shape))
    return n * (9 * 4 + 2 * (4 if P.get("fp32_fields") else 2))


def footprint_bytes(shape, dx, P, rays, fuv, fast, nstars, arith=None):
    """device bytes an instance of this description holds once built with `nstars` stars: its fields
    plus the library's scratch (nb_instance_bytes), known before anything is allocated"""
    lib = _lib.load(arith)
    cap = max(int(nstars), int(P["max_stars"]))
    d = instance_desc(shape, dx, P, rays, fuv, fast, cap)
    out = C.c_longlong()
    _lib.check(lib.nb_instance_bytes(None, C.byref(d), int(nstars), C.byref(out)), None, "nb_instance_bytes", lib)
    return field_bytes(shape, P) + int(out.value)


class Sim:
    """GPU-resident simulation on the GB300 kernels.

    Sim("sheet", res=256); sim.step(4); sim.update_render_fields()
    """

    profile = False

    def __init__(self, scenario="torus", res=None, params=None, ic_mode="synthetic", rays=None, fuv_grid=None,
                 ion_every=None, device="cuda:0", verbose=True, fast=True, seed=None, arith=None):
        self.arith = _lib.arith_of(arith)
        self.device = torch.device(device)
        self.fast = fast
        self.verbose = verbose
        self.ic_mode = ic_mode
        self.rays_override = rays
        self.fuv_override = fuv_grid
        self.ion_every_override = ion_every
        self.prof = {}
        self._h = None
        self.reset(scenario, res, params, seed=seed)

    # ------------------------------------------------------------------ construction
    @classmethod
    def from_state(cls, shape, dx, rho, stars, kinds, jets, jkinds, P, mom=None, rays=None, fuv_grid=None,
                   ion_every=None, fast=True, device="cuda:0", verbose=False, start_main=True, torus=None,
                   stir_fields=None, stir_grid=None, arith=None):
        """An instance from explicit fields and star lists (what the reference's reset() leaves
        behind, sim.py:710-795), e.g. initial conditions built by the reference's own IC code.
        `torus` joins rho when the main phase starts (at once without a stirring phase);
        `stir_fields` ([3][sx][sy][sz] arrays) replaces the forcing generator, in order of use;
        `stir_grid` = ((sx, sy, sz), dxs) overrides the forcing grid.  `arith`: "exact" (bit-identical
        to the reference's kernels) or "fast" (FMA, approximate division / square root)."""
        self = cls.__new__(cls)
        self.arith = _lib.arith_of(arith)
        self.device = torch.device(device)
        self.fast = fast
        self.verbose = verbose
        self.ic_mode = "state"
        self.rays_override = rays
        self.fuv_override = fuv_grid
        self.ion_every_override = ion_every
        self.prof = {}
        self._h = None
        self.scenario = "state"
        self.res = None
        ic = dict(shape=tuple(shape), dx=float(dx), rho=rho, mom=mom, stars=stars, kinds=kinds, jets=jets,
                  jkinds=jkinds, P={}, torus=torus, stir_fields=stir_fields, stir_grid=stir_grid)
        self._setup(ic, dict(P), start_main=start_main)
        return self

    @classmethod
    def from_reference(cls, ref, params=None, arith=None, device="cuda:0", verbose=False):
        """The drop-in taking over a reference `Sim` instance (sim.py:543-1222) as it stands: one
        built by the reference's own reset() from its presets and initial conditions
        (sim.py:50-59, 591-795), in the stirring phase or the main phase.  It copies the fields
        (rho, mx, my, mz, xi, dfront, g0), the star and jet lists, the parameters P, the ray / FUV
        budgets, the cadences, the clocks, the live-event log, the render-field bookkeeping and
        the stirring state (fields A and B, the cross-fade clock, the forcing generator: the
        Generator state, or the matched spectrum's seed and call count, sim.py:270-337), so that
        stepping the drop-in continues the reference's run.

        The reference package is never imported: `ref` is read through its attributes and
        get_state_meta() alone, and every field through .numpy() (a Warp array, a NumPy array or
        anything with that method).  `params` overrides entries of P, e.g. {"trigger": 0.0} as
        bake.py sets it after construction (bake.py:61-63); triggered star formation and cropped
        domains are outside this package and are refused."""
        def host(x):
            return np.asarray(x.numpy() if hasattr(x, "numpy") else x)

        if getattr(ref, "L_full", None) is not None:              # sim.py:634: a cropped window
            raise NotImplementedError("a cropped domain (crop.py) is outside this package")
        P = dict(ref.P)
        P.update(params or {})
        meta = dict(ref.get_state_meta())
        meta["P"] = dict(P)
        d = meta.get("drv")
        if d is not None:
            meta["drv"] = {"A": [host(c) for c in d["A"]], "B": [host(c) for c in d["B"]], "clock": float(d["clock"])}
        noise = getattr(ref, "noise", None)
        if noise is not None and not hasattr(noise, "seed"):
            raise NotImplementedError("the reference's noise generator is not the matched one (a cropped domain?)")
        noise = None if noise is None else {"seed": int(noise.seed), "calls": int(noise.calls),
                                            "modes": int(getattr(noise, "K", _stir.MATCHED_MODES))}
        torus0 = getattr(ref, "torus0", None)
        self = cls.__new__(cls)
        self.arith = _lib.arith_of(arith)
        self.device = torch.device(device)
        self.fast = bool(ref.fast)
        self.verbose = verbose
        self.ic_mode = getattr(ref, "ic_mode", "matched")
        self.rays_override = tuple(int(v) for v in ref.rfront.shape)
        self.fuv_override = tuple(int(v) for v in ref.att.shape)
        self.ion_every_override = int(ref.ion_every)
        self.prof = {}
        self._h = None
        self.scenario = getattr(ref, "scenario", "reference")
        self.res = getattr(ref, "res", None)
        ic = dict(shape=tuple(int(v) for v in ref.shape), dx=float(ref.dx), rho=host(ref.rho),
                  mom=[host(ref.mx), host(ref.my), host(ref.mz)], stars=ref.stars, kinds=ref.kinds, jets=ref.jets,
                  jkinds=ref.jkinds, P={}, torus=host(torus0) if (torus0 is not None and ref.phase == "pre") else None,
                  stir_grid=(tuple(int(v) for v in ref.sshape), float(ref.dxs)), noise=noise)
        self._setup(ic, P, start_main=False)
        if torus0 is not None:
            self.torus0 = torch.as_tensor(host(torus0), dtype=torch.float32, device=self.device)
        self._xi.copy_(torch.as_tensor(host(ref.xi)).to(self._xi.dtype))
        self._dfront.copy_(torch.as_tensor(host(ref.dfront)).to(self._dfront.dtype))
        self._g0.copy_(torch.as_tensor(host(ref.g0)).to(self._g0.dtype))
        self.events = [tuple(e) for e in ref.events]
        self.set_state_meta(meta)
        # the render-field bookkeeping continues the reference's cadence (sim.py:989-1007)
        for k in ("version", "rf_version", "fuv_version"):
            setattr(self, k, int(getattr(ref, k)))
        self.fuv_nstars = getattr(ref, "fuv_nstars", -1)
        self.fuv_phase = getattr(ref, "fuv_phase", None)
        self.dt_cap = getattr(ref, "dt_cap", None)
        self._sync()
        return self

    def reset(self, scenario=None, res=None, params=None, seed=None):
        if scenario is not None:
            self.scenario = scenario
        if self.scenario in REFERENCE_PRESETS:
            raise ValueError(f"{self.scenario!r} is one of the reference's preset scenes, whose initial conditions the "
                             f"reference's own reset() builds (sim.py:591-795): build the reference Sim and hand it "
                             f"over with Sim.from_reference(ref_sim); synthetic scenarios: {sorted(_ics.SCENARIOS)}")
        if self.scenario not in _ics.SCENARIOS:
            raise ValueError(f"unknown scenario {self.scenario!r}; synthetic scenarios: {sorted(_ics.SCENARIOS)}")
        gen = _ics.SCENARIOS[self.scenario]
        kw = {"device": self.device}
        if res is not None:
            kw["res"] = int(res)
        if seed is not None:
            kw["seed"] = int(seed)
        ic = gen(**kw)
        self.res = kw.get("res")
        self._setup(ic, dict(params or {}))

    def _setup(self, ic, overrides, start_main=True):
        t_setup = time.perf_counter()
        self.close()
        self._clock_fresh = False
        P = make_params(overrides, base=ic["P"])
        if float(P.get("trigger", 0.0) or 0.0) > 0.0:
            raise NotImplementedError("triggered star formation (trigger > 0) is outside this package's simulation step")
        if P.get("crop"):
            raise NotImplementedError("cropped domains are outside this package's simulation step")
        self.P = P
        self.shape = tuple(int(v) for v in ic["shape"])
        nx, ny, nz = self.shape
        if nz % 4:
            raise ValueError("nz must be a multiple of 4 (16-byte rows for the TMA tiles)")
        self.dx = float(ic["dx"])
        self.L = (nx * self.dx, ny * self.dx, nz * self.dx)
        if min(self.shape) < 1 or not self.dx > 0.0:
            raise ValueError(f"a grid needs positive sizes and dx, not {self.shape}, dx = {self.dx}")
        dev = self.device
        f32 = dict(device=dev, dtype=torch.float32)

        def field(x, what):                      # the kernels index every field by the grid's shape
            t = x if torch.is_tensor(x) else torch.as_tensor(np.asarray(x, np.float32))
            if tuple(t.shape) != self.shape:
                raise ValueError(f"{what} has shape {tuple(t.shape)}; the grid is {self.shape}")
            return t.to(**f32).contiguous()

        self._rho = field(ic["rho"], "rho").clone()
        pre = float(P.get("pre_t", 0.0) or 0.0) > 0.0
        torus = ic.get("torus")
        self.torus = None
        if torus is not None:                                                       # sim.py:669-671, 737
            torus = field(torus, "torus")
            if pre:
                self.torus = torus
            else:
                self._rho += torus
        self.torus0 = self.torus
        if ic.get("mom") is None:
            m = [torch.zeros(self.shape, **f32) for _ in range(3)]
        else:
            if len(ic["mom"]) != 3:
                raise ValueError("mom holds the three momentum fields (mx, my, mz)")
            m = [field(v, name).clone() for v, name in zip(ic["mom"], ("mx", "my", "mz"))]
        self._mx, self._my, self._mz = m
        self._xi = torch.zeros(self.shape, **f32)
        self._stage = torch.zeros((4,) + self.shape, **f32)
        hdt = torch.float32 if P.get("fp32_fields") else torch.float16
        self._dfront = torch.full(self.shape, 1e3, device=dev, dtype=hdt)
        self._g0 = torch.zeros(self.shape, device=dev, dtype=hdt)
        self.stars = [tuple(float(v) for v in s) for s in ic["stars"]]
        self.kinds = list(ic["kinds"])
        self.jets = [tuple(float(v) for v in j[:3]) for j in ic["jets"]]
        self.jkinds = list(ic["jkinds"])
        self.cn2, self.ci2, self.vmax = sound_speeds(P)
        Lx, Ly, Lz = self.L
        self.diag = math.sqrt(Lx ** 2 + Ly ** 2 + Lz ** 2) + 0.6                    # sim.py:742
        self.dr = (1.0 if self.fast else 0.5) * self.dx                             # sim.py:743
        self.nsteps = int(self.diag / self.dr) + 1                                  # sim.py:744
        self.cap = max(len(self.stars), int(P["max_stars"]))                        # sim.py:745
        rays, fuv = _ray_budget(nz, self.fast, self.rays_override, self.fuv_override)
        self.rfront = _Shape(rays)
        self.att = _Shape(fuv)
        self.ion_every = self.ion_every_override or (max(P["ion_every"], 3) if self.fast else P["ion_every"])
        self.fuv_every = (8 if nz <= 160 else 16) if self.fast else 8               # sim.py:759
        self._stream = torch.cuda.current_stream(dev) if dev.type == "cuda" else None
        lib = _lib.load(self.arith)
        d = instance_desc(self.shape, self.dx, P, rays, fuv, self.fast, self.cap)
        st = self._stage
        n = nx * ny * nz
        d.f = _lib.NbFields(self._rho.data_ptr(), self._mx.data_ptr(), self._my.data_ptr(), self._mz.data_ptr(),
                            self._xi.data_ptr(), st.data_ptr(), self._dfront.data_ptr(), self._g0.data_ptr())
        d.stream = self._stream.cuda_stream if self._stream is not None else None
        h = C.c_void_p()
        _lib.check(lib.nb_create(C.byref(d), C.byref(h)), None, "nb_create", lib)
        self._h = h
        self._lib = lib
        self._n = n
        # the uncropped domain's values of the crop attributes the viewer reads (sim.py:647)
        self.crop_origin, self.L_full = (0.0, 0.0, 0.0), None
        self._live_key = None
        self._stars_key = None
        self._dt_cap = None
        self._it = 0
        self.version = 0
        self.rf_version = -1
        self.fuv_version = -10 ** 9
        self.generation = getattr(self, "generation", 0) + 1
        self.events = []
        self.births = []
        self.n_born = 0
        self.last_birth = -1e9
        self.mach = None
        self.sm0 = None
        self.P_reset = dict(P)
        self.q_main0 = P["q_main"]
        # stirring (sim.py:760-768, 786-790): the forcing grid, the Generator, the ring
        self.rng = np.random.default_rng(P["seed"])
        # the reference's "matched" mode draws forcing fields from a per-call seeded spectrum
        # (sim.py:648, 802) instead of the Generator: {"seed", "calls", "modes"}, or None
        nz_ = ic.get("noise")
        self.noise = None if nz_ is None else {"seed": int(nz_["seed"]), "calls": int(nz_["calls"]),
                                               "modes": int(nz_.get("modes", _stir.MATCHED_MODES))}
        src = ic.get("stir_fields")
        self._stir_src = None if src is None else collections.deque(np.asarray(f, np.float32) for f in src)
        grid = ic.get("stir_grid")
        if grid is None:
            grid = _stir.forcing_grid(self.L, self.dx, self.shape, physical=self.ic_mode != "nebula3d")
        self.sshape, self.dxs = tuple(int(v) for v in grid[0]), float(grid[1])
        self._drv_on = False
        self._forcing = []              # (field, Generator state before it) per field drawn since the ring reset
        self._pushed = 0                # of which pushed into the device ring
        self.phase = "pre" if pre else "main"
        self._push(force=True)
        if pre:
            self._drive_new(0.0)
        elif start_main:
            self._start_main()
        self._sync()
        self.setup_s = time.perf_counter() - t_setup
        self.log(f"{self.scenario} grid {nx}x{ny}x{nz} ({n / 1e6:.1f}M cells) rays {rays[0]}x{rays[1]} "
                 f"fuv {fuv} solver {P.get('solver')} setup {self.setup_s:.2f}s, {len(self.stars)} stars")

    def close(self):
        if getattr(self, "_h", None):
            self._sync()
            self._lib.nb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ helpers
    def log(self, *a):
        if self.verbose:
            print("[sim]", *a, flush=True)

    def _sync(self):
        if self._stream is not None:
            self._stream.synchronize()

    def _tick(self, key, t0):
        self.prof[key] = self.prof.get(key, 0.0) + (time.perf_counter() - t0)

    def _chk(self, rc, what):
        _lib.check(rc, self._h, what, self._lib)

    # sim.py:914-925 keys the star-weight upload on _wkey, and bake.py:91 resets it after editing P.
    # Here P and the star lists are compared at every push; resetting _wkey forces the next push.
    @property
    def _wkey(self):
        return (self._live_key, self._stars_key)

    @_wkey.setter
    def _wkey(self, value):
        if value is None:
            self._live_key = None
            self._stars_key = None

    def _push(self, force=False):
        """upload live parameters / the star table when they changed (P may be edited directly,
        as bake.py does, sim.py:88-93 there)"""
        P = self.P
        cap = self._dt_cap if self._dt_cap is not None else -1.0
        live = (float(P["q_main"]), float(P["wind"]), float(P["jet"]), float(P["jet_proto"]), float(P["jet_pulse"]),
                float(P["jet_period"]), float(P["kappa_fuv"]), float(P.get("q_ramp", 0.0)), float(P["jet_angle"]),
                float(P["jet_r"]), float(cap), 1 if self.phase == "main" else 0,
                float(P.get("plane_flux", 0.0) or 0.0), float(P.get("plane_fuv", 0.0) or 0.0),
                float(P.get("pre_amp", 0.0) or 0.0), float(P.get("drive_main", 0.0) or 0.0))
        if force or live != self._live_key:
            L = _lib.NbLive(*live)
            self._chk(self._lib.nb_set_live(self._h, C.byref(L)), "nb_set_live")
            self._live_key = live
        skey = (tuple(self.stars), tuple(self.kinds), tuple(self.jets), tuple(self.jkinds))
        if force or skey != self._stars_key:
            n = len(self.stars)
            arr = (_lib.NbStar * max(n, 1))()
            for i, s in enumerate(self.stars):
                a = self.jets[i] if i < len(self.jets) else (0.0, 0.0, 1.0)
                jk = self.jkinds[i] if i < len(self.jkinds) else "none"
                arr[i] = _lib.NbStar(s[0], s[1], s[2], s[3], s[4], a[0], a[1], a[2], _lib.STAR_KINDS[self.kinds[i]],
                                     _lib.JET_KINDS[jk])
            self._chk(self._lib.nb_set_stars(self._h, arr, n), "nb_set_stars")
            self._stars_key = skey

    # ------------------------------------------------------------------ fields
    rho = property(lambda self: Field(self._rho))
    mx = property(lambda self: Field(self._mx))
    my = property(lambda self: Field(self._my))
    mz = property(lambda self: Field(self._mz))
    xi = property(lambda self: Field(self._xi))
    stage = property(lambda self: Field(self._stage))
    dfront = property(lambda self: Field(self._dfront))
    g0 = property(lambda self: Field(self._g0))
    r1 = property(lambda self: Field(self._stage[0]))
    mx1 = property(lambda self: Field(self._stage[1]))
    my1 = property(lambda self: Field(self._stage[2]))
    mz1 = property(lambda self: Field(self._stage[3]))
    xi_tmp = property(lambda self: Field(self._stage[0]))

    def render_scratch(self):
        """two RGBA16F grids (half4 views of the stage block), free between steps (sim.py:821-825)"""
        b = self._stage.view(torch.float16).reshape(-1)
        n = self._n
        return (Field(b[:4 * n].view(self.shape + (4,))), Field(b[4 * n:8 * n].view(self.shape + (4,))))

    # ------------------------------------------------------------------ clock (device resident)
    def _clock(self):
        """the device clock; right after a synchronized step(k) it is read from the pinned copy made
        at its end (no round trip), otherwise from the device (synchronizes)"""
        c = _lib.NbClock()
        if getattr(self, "_clock_fresh", False):
            self._chk(self._lib.nb_peek_clock(self._h, C.byref(c)), "nb_peek_clock")
        else:
            self._chk(self._lib.nb_get_clock(self._h, C.byref(c)), "nb_get_clock")
        return c

    def _set_clock(self, t=None, dt=None, it=None, tp=None, ip=None):
        c = self._clock()
        c.t = c.t if t is None else float(t)
        c.dt = c.dt if dt is None else float(dt)
        c.it = c.it if it is None else int(it)
        c.tp = c.tp if tp is None else float(tp)
        c.ip = c.ip if ip is None else int(ip)
        self._chk(self._lib.nb_set_clock(self._h, C.byref(c)), "nb_set_clock")
        self._it = int(c.it)
        self._clock_fresh = True                     # nb_set_clock synchronized and refreshed the copy

    t = property(lambda self: self._clock().t, lambda self, v: self._set_clock(t=v))
    dt = property(lambda self: self._clock().dt, lambda self, v: self._set_clock(dt=v))
    it = property(lambda self: self._it, lambda self, v: self._set_clock(it=v))
    tp = property(lambda self: self._clock().tp, lambda self, v: self._set_clock(tp=v))
    ip = property(lambda self: int(self._clock().ip), lambda self, v: self._set_clock(ip=v))

    @property
    def dt_cap(self):
        return self._dt_cap

    @dt_cap.setter
    def dt_cap(self, v):
        self._dt_cap = None if v is None else float(v)

    # ------------------------------------------------------------------ physics pieces (host views)
    def q_of(self, i):
        s = self.stars[i]
        return s[3] * self.P["q_main"] if self.kinds[i] == "main" else s[3]

    def ramp(self, i, t=None):
        t = self.t if t is None else t
        age = t - self.stars[i][4]
        if self.phase != "main" or age < 0.0:
            return 0.0
        tr = float(self.P.get("q_ramp", 0.0))
        if tr <= 0.0 or age >= tr:
            return 1.0
        x = age / tr
        s = x * x * (3.0 - 2.0 * x)
        return max(s * s * s, 1e-4)

    def q_eff(self, i, t=None):
        return self.q_of(i) * self.ramp(i, t)

    def jet_of(self, i):
        k = self.jkinds[i]
        return self.P["jet"] if k == "jet" else (self.P["jet_proto"] if k == "proto" else 0.0)

    def active_stars(self):
        if self.phase != "main":
            return []
        t = self.t
        return [(s[0], s[1], s[2], self.q_eff(i, t) / self.P["q_main"], t - s[4]) for i, s in enumerate(self.stars)
                if t >= s[4]]

    # ------------------------------------------------------------------ the step
    def ionize(self):
        """sim.py:927-947: rays of every active star, front apply, smoothing, fp16 dfront"""
        t0 = time.perf_counter()
        self._push()
        self._chk(self._lib.nb_ionize(self._h), "nb_ionize")
        if self.profile:
            self._sync()
            self._tick("ionize", t0)

    def fuv_field(self):
        """sim.py:949-985: G0 of every active star into g0"""
        self._push()
        self._chk(self._lib.nb_fuv(self._h), "nb_fuv")

    fuv_every = 8

    def update_render_fields(self, force=False):
        """sim.py:989-1007: recompute G0 when the simulation advanced, on the reference's cadence"""
        if self.rf_version == self.version and not force:
            return False
        t0 = time.perf_counter()
        t = self.t
        n_on = sum(1 for s in self.stars if t >= s[4])
        tr = float(self.P.get("q_ramp", 0.0))
        ramping = tr > 0 and any(0.0 <= t - s[4] < tr for s in self.stars)
        if ramping and self.version - self.fuv_version >= max(2, self.fuv_every // 4):
            force = True
        if (force or self.version - self.fuv_version >= self.fuv_every
                or n_on != getattr(self, "fuv_nstars", -1) or self.phase != getattr(self, "fuv_phase", None)):
            self.fuv_field()
            self.fuv_version, self.fuv_nstars, self.fuv_phase = self.version, n_on, self.phase
        self.rf_version = self.version
        if self.profile:
            self._sync()
            self._tick("render_fields", t0)
        return True

    def step(self, k=1, sync=True):
        """advance k hydro steps, stirring-phase or main-phase (sim.py:1141-1152).  Returns wall
        seconds.  With sync=False the steps are only enqueued on the stream (the stirring phase
        and stirred main-phase steps still synchronize once per chunk)."""
        t0 = time.perf_counter()
        self._clock_fresh = False
        self._push()
        left = int(k)
        while left > 0:
            n = self._pre_chunk(left) if self.phase == "pre" else self._main_chunk(left)
            left -= n
            self.version += n
        if sync:
            self._chk(self._lib.nb_mirror_clock(self._h), "nb_mirror_clock")
            self._sync()
            self._clock_fresh = True                 # the stream passed the clock's copy to host memory
            self._clock()                            # host read; raises if a hydro stage's TMA wait gave up
            if self._drv_on:
                self._drive_info()                 # raises if a stirred step found no forcing field
        self._tick("step", t0)
        self.prof["n_steps"] = self.prof.get("n_steps", 0) + k
        return time.perf_counter() - t0

    def _stirring(self):
        return self._drv_on and float(self.P.get("drive_main", 0.0) or 0.0) > 0.0

    def _main_chunk(self, left):
        """main-phase steps (sim.py:1099-1114); stirred steps in chunks the pushed fields cover"""
        if not self._stirring():
            self._chk(self._lib.nb_step(self._h, int(left), int(self.ion_every)), "nb_step")
            self._it += left
            return left
        info = self._drive_ready()
        n = min(left, self._drive_steps())
        self._chk(self._lib.nb_step(self._h, int(n), int(self.ion_every)), "nb_step")
        self._it += n
        self._drive_ahead(info)
        return n

    def _pre_chunk(self, left):
        """stirring-phase steps (sim.py:1044-1059): as many as provably cannot reach pre_t but
        the last (and whose field swaps the pushed fields cover), then the end-of-phase test"""
        c = self._clock()
        gap = float(self.P["pre_t"]) - c.tp
        n_end = max(1, math.ceil(gap / self._dt_bound())) if gap > 0.0 else 1
        info = self._drive_ready()
        n = min(left, n_end, self._drive_steps())
        self._chk(self._lib.nb_pre_step(self._h, int(n)), "nb_pre_step")
        self._drive_ahead(info)
        if n == n_end and self._clock().tp >= float(self.P["pre_t"]):
            self._end_pre()
        return n

    # ---- stirring helpers
    def _dt_bound(self):
        """an upper bound of the CFL dt (sim.py:1012): the max speed is at least the smallest
        sound speed sqrt(cn2 + xi (ci2 - cn2)), xi in [0, 1], as the kernels round it"""
        c = min(float(np.sqrt(np.float32(self.cn2))), float(np.sqrt(np.float32(self.ci2))))
        return float(self.P["cfl"]) * self.dx / c * (1.0 + 1e-6)

    def _drive_steps(self):
        """steps a chunk may take with DRIVE_LOOKAHEAD fields pushed beyond B: n steps make at
        most 1 + (n - 1) // m field swaps (the first may come at once, each next one needs at
        least m = ceil(pre_corr / dt_max) steps)"""
        m = max(1, math.ceil(float(self.P["pre_corr"]) / self._dt_bound()))
        return (DRIVE_LOOKAHEAD - 1) * m + 1

    def _drive_ready(self):
        """the device's swap count (synchronizes) and the fields a chunk may need pushed"""
        info = self._drive_info()
        self._drive_fill(int(info.swaps) + 2 + DRIVE_LOOKAHEAD)
        return info

    def _drive_ahead(self, info):
        """draw the next fields on the host while the GPU runs the chunk just launched"""
        self._drive_make(int(info.swaps) + 2 + 2 * DRIVE_LOOKAHEAD)

    def _drive_info(self):
        info = _lib.NbDriveInfo()
        self._chk(self._lib.nb_drive_state(self._h, C.byref(info)), "nb_drive_state")
        if info.status & 2:
            raise _lib.NebulaError("a stirred step found no forcing field B in the ring")
        return info

    def _mkF(self):
        """sim.py:801-804: the next forcing field, [3][sx][sy][sz] float32"""
        if self._stir_src is not None:
            if not self._stir_src:
                raise _lib.NebulaError("the given forcing fields are used up")
            return np.ascontiguousarray(self._stir_src.popleft(), np.float32)
        kmax = float(self.P["pre_kmax"])
        if self.noise is not None:
            c = self.noise["calls"]
            self.noise["calls"] = c + 3                      # one call per component (sim.py:330)
            return np.ascontiguousarray(np.stack(_stir.matched_solenoidal(self.sshape, self.noise["seed"], c, 1.0, kmax,
                                                                          self.noise["modes"])), np.float32)
        return np.ascontiguousarray(np.stack(_stir.solenoidal(self.sshape, self.rng, 1.0, kmax)), np.float32)

    def _gen_state(self):
        """the forcing generator's state: the Generator's, or the matched spectrum's call count"""
        if self.noise is not None:
            return ("calls", self.noise["calls"])
        return copy.deepcopy(self.rng.bit_generator.state)

    def _gen_restore(self, st):
        if self.noise is not None:
            self.noise["calls"] = int(st[1])
        else:
            self.rng.bit_generator.state = st

    def _drive_make(self, upto):
        """draw forcing fields on the host until `upto` exist since the ring reset (a given, finite
        list of fields goes as far as it goes: a step that then finds no field B raises)"""
        while len(self._forcing) < upto:
            if self._stir_src is not None and not self._stir_src:
                break
            st = self._gen_state()
            self._forcing.append((self._mkF(), st))

    def _push_forcing(self, buf):
        """copy n forcing fields ([n][3][sx][sy][sz] float32, host) into the device ring: the library
        reads n whole fields of the forcing grid from the buffer, so its shape is checked here"""
        want = (3,) + tuple(self.sshape)
        if buf.dtype != np.float32 or buf.ndim != 5 or tuple(buf.shape[1:]) != want or not buf.flags.c_contiguous:
            raise ValueError(f"forcing fields must be float32 [n]{list(want)}, not {buf.dtype} {list(buf.shape)}")
        self._chk(self._lib.nb_drive_push(self._h, C.c_void_p(buf.ctypes.data), len(buf)), "nb_drive_push")

    def _drive_fill(self, upto):
        """push forcing fields until `upto` fields were pushed since the ring reset"""
        self._drive_make(upto)
        new = [f for f, _ in self._forcing[self._pushed:upto]]
        if new:
            self._push_forcing(np.ascontiguousarray(np.stack(new), np.float32))
            self._pushed += len(new)

    def _drive_new(self, clock, fields=None):
        """a fresh cross-fade (sim.py:788, 1160-1161): reset the ring, push A and B"""
        self._drive_rewind()
        d = _lib.NbDriveDesc(self.sshape[0], self.sshape[1], self.sshape[2], DRIVE_SLOTS, self.dxs,
                             float(self.P["pre_corr"]), float(clock))
        self._chk(self._lib.nb_drive_config(self._h, C.byref(d)), "nb_drive_config")
        self._forcing = []
        self._pushed = 0
        if fields is not None:
            buf = np.ascontiguousarray(np.stack([np.asarray(f, np.float32) for f in fields]))
            self._push_forcing(buf)
            self._forcing = [(f, None) for f in buf]
            self._pushed = len(buf)
        else:
            self._drive_fill(2)
        self._drv_on = True
        self._chk(self._lib.nb_drive_enable(self._h, 1), "nb_drive_enable")

    def _drive_rewind(self):
        """return the fields pushed ahead of use to the source: the Generator goes back to the
        state after the last field the reference would have drawn (A and B of now)"""
        if not self._forcing:
            return
        info = self._drive_info() if self._drv_on else None
        used = len(self._forcing) if info is None else min(len(self._forcing), int(info.swaps) + 2)
        extra = self._forcing[used:]
        if extra:
            if self._stir_src is not None:
                self._stir_src.extendleft(f for f, _ in reversed(extra))
            elif extra[0][1] is not None:
                self._gen_restore(extra[0][1])
        self._forcing = self._forcing[:used]
        self._pushed = min(self._pushed, used)

    def _drive_drop(self):
        """drv = None (sim.py:1057-1058)"""
        self._drive_rewind()
        self._drv_on = False
        self._forcing = []
        self._pushed = 0
        self._chk(self._lib.nb_drive_enable(self._h, 0), "nb_drive_enable")

    @property
    def drv(self):
        """the reference's drv dict {'A', 'B', 'clock'} (host copies), or None"""
        if not self._drv_on:
            return None
        info = self._drive_info()
        a = self._forcing[int(info.swaps)][0]
        b = self._forcing[int(info.swaps) + 1][0]
        return {"A": list(a), "B": list(b), "clock": float(info.clock)}

    def _end_pre(self):
        """sim.py:1051-1059: Mach number of the turbulence, end of the stirring phase"""
        s = (C.c_double * 2)()
        self._chk(self._lib.nb_mach_sums(self._h, s), "nb_mach_sums")
        a, b = float(s[0]), float(s[1])
        self.mach = math.sqrt(a / b) * float(self.P["ci_over_cn"])
        self.log(f"pre-turbulence done: {self.ip} steps t={self.tp:.3f} mass-weighted Mach ~{self.mach:.1f}")
        if float(self.P.get("drive_main", 0.0) or 0.0) <= 0:
            self._drive_drop()
        self._start_main()

    def _start_main(self):
        """sim.py:806-818: the torus joins (through the scratch block), the main phase starts, first ionization"""
        if self.torus is not None:
            self._stage[0].copy_(self.torus)
            self._chk(self._lib.nb_add_torus(self._h, C.c_void_p(self._stage[0].data_ptr())), "nb_add_torus")
            self.torus = None
        self.phase = "main"
        self._push()
        self.ionize()

    def set_param(self, name, value):
        """sim.py:1154-1166: live parameters take effect on the next step and are logged"""
        old = self.P.get(name)
        if isinstance(old, int) and not isinstance(old, bool):
            value = int(round(value))
        self.P[name] = value
        if name == "drive_main" and value > 0 and not self._drv_on and self.phase == "main":
            self._drive_new(0.0)
        if name in LIVE:
            self.events.append((float(self.t if self.phase == "main" else 0.0), name, value))
        return value

    def replace_stars(self, stars, kinds, jets, jkinds):
        """sim.py:1120-1133: an explicit star list (bake.py replays the preview's)"""
        self.stars = [tuple(float(v) for v in s) for s in stars]
        self.kinds = list(kinds)
        self.jets = [tuple(float(v) for v in j[:3]) for j in jets]
        self.jkinds = list(jkinds)
        if len(self.stars) > self.cap:
            self.cap = len(self.stars)
            if self.cap > 256:
                raise _lib.NebulaError("more than 256 stars")
            self.close()
            raise _lib.NebulaError("the star table grew past max_stars; rebuild the Sim with a larger max_stars")
        if self.phase == "main":
            self.ionize()

    def stars_absolute(self):
        st = [(s[0], s[1], s[2], self.q_of(i), s[4]) for i, s in enumerate(self.stars)]
        jt = [(j[0], j[1], j[2], self.jet_of(i)) for i, j in enumerate(self.jets)]
        return st, jt

    # ------------------------------------------------------------------ timeline (snapshots)
    def tau(self):
        return self.t if self.phase == "main" else self.tp - self.P["pre_t"]

    def get_state_meta(self):
        """sim.py:1173-1183: everything but the big fields needed to resume from this moment.
        The Generator state is the one after the fields in use (A and B), as the reference's."""
        c = self._clock()
        drv, gen = None, self._gen_state()
        if self._drv_on:
            info = self._drive_info()
            sw = int(info.swaps)
            drv = {"A": list(self._forcing[sw][0]), "B": list(self._forcing[sw + 1][0]), "clock": float(info.clock)}
            if sw + 2 < len(self._forcing) and self._forcing[sw + 2][1] is not None:
                gen = copy.deepcopy(self._forcing[sw + 2][1])
        matched = self.noise is not None
        rng = copy.deepcopy(self.rng.bit_generator.state) if matched else gen
        return dict(t=c.t, it=int(c.it), tp=c.tp, ip=int(c.ip), dt=c.dt, phase=self.phase, mach=self.mach,
                    stars=list(self.stars), kinds=list(self.kinds), jets=list(self.jets), jkinds=list(self.jkinds),
                    births=list(self.births), n_born=self.n_born, last_birth=self.last_birth, P=dict(self.P),
                    n_events=len(self.events), sm0=self.sm0, drv=drv, rng=rng,
                    noise_calls=int(gen[1]) if matched else 0)

    def set_state_meta(self, m):
        """sim.py:1185-1211: after the fields were restored"""
        for k in ("phase", "mach", "n_born", "last_birth", "sm0"):
            setattr(self, k, m[k])
        self.stars, self.kinds = list(m["stars"]), list(m["kinds"])
        self.jets, self.jkinds = list(m["jets"]), list(m["jkinds"])
        self.births = list(m["births"])
        self.P = dict(m["P"])
        self.events = self.events[:m["n_events"]]
        self._set_clock(t=m["t"], dt=m["dt"], it=m["it"], tp=m.get("tp", 0.0), ip=m.get("ip", 0))
        d = m.get("drv")
        if d is None:
            if self._drv_on:
                self._drive_drop()
        else:
            self._drive_new(d["clock"], fields=[np.stack(d["A"]), np.stack(d["B"])])
        if m.get("rng") is not None:
            self.rng.bit_generator.state = copy.deepcopy(m["rng"])
        if self.noise is not None:
            self.noise["calls"] = int(m.get("noise_calls", 0))                       # sim.py:1198-1199
        self.torus = self.torus0 if self.phase == "pre" else None
        self._chk(self._lib.nb_invalidate(self._h), "nb_invalidate")
        self._push(force=True)
        self.version += 1
        self.rf_version = self.version
        self.fuv_version = self.version
        self.fuv_nstars = sum(1 for s in self.stars if m["t"] >= s[4])
        self.fuv_phase = self.phase

    # ------------------------------------------------------------------ snapshots and frames
    def snapshot_pack(self, buf):
        """the 13 B/cell snapshot (timeline.py:19-89) into a device uint8 buffer of 13 * cells"""
        if buf.numel() * buf.element_size() < 13 * self._n or not buf.is_cuda:
            raise ValueError("snapshot buffer must be a device buffer of 13 bytes per cell")
        self._chk(self._lib.nb_snapshot_pack(self._h, C.c_void_p(buf.data_ptr())), "nb_snapshot_pack")

    def snapshot_unpack(self, buf):
        """restore the fields from a 13 B/cell snapshot (timeline.py k_unpack)"""
        if buf.numel() * buf.element_size() < 13 * self._n or not buf.is_cuda:
            raise ValueError("snapshot buffer must be a device buffer of 13 bytes per cell")
        self._chk(self._lib.nb_snapshot_unpack(self._h, C.c_void_p(buf.data_ptr())), "nb_snapshot_unpack")
        self.version += 1

    @property
    def shock(self):
        """compression heating proxy max(0, -div v) rho, computed now into a new fp32 grid
        (nebula3d.py:182-191; sim.py:827-833)"""
        out = torch.empty(self.shape, dtype=torch.float32, device=self.device)
        self._chk(self._lib.nb_shock(self._h, C.c_void_p(out.data_ptr())), "nb_shock")
        return Field(out)

    def frame(self, pinned=None):
        """one bake frame (bake.py:95-102): quantized on the device, read back in one copy;
        returns dict(g0, rho, xi, df, sh) of numpy arrays in the reference's dtypes"""
        n = self._n
        dev = torch.empty(9 * n, dtype=torch.uint8, device=self.device)
        self._chk(self._lib.nb_frame_pack(self._h, C.c_void_p(dev.data_ptr())), "nb_frame_pack")
        host = pinned if pinned is not None else torch.empty(9 * n, dtype=torch.uint8).pin_memory()
        host.copy_(dev, non_blocking=True)
        self._sync()
        b = host.numpy()
        sh = self.shape
        f16 = lambda off: b[off:off + 2 * n].view(np.float16).reshape(sh)  # noqa: E731
        return dict(g0=f16(0), rho=f16(2 * n), xi=b[4 * n:5 * n].reshape(sh), df=f16(5 * n), sh=f16(7 * n))

    PACK_FIELDS = ("c_ha", "c_o3", "c_s2", "c_dg", "c_sh", "gs", "ambient", "edge", "inv_L", "dx")

    def render_pack(self, pp, shock_on=None, smooth=True):
        """render.py:176-205 pack_volume_lm (+ render.py:281-298 smooth_axis x, y, z): the RGBA16F
        voxel grid (emission r, g, b; dust) of the current fields, packed into the render scratch
        (the stage block, free between steps) as Renderer.pack does; returns it as a
        (nx, ny, nz, 4) float16 Field.  `pp`: the reference's PackParams (render.py:77-88,
        Renderer.pack_params) or a mapping with the same keys; shock_on defaults to any(c_sh)."""
        get = (lambda k: pp[k]) if isinstance(pp, dict) else (lambda k: getattr(pp, k))
        vals = {k: get(k) for k in self.PACK_FIELDS}
        P = _lib.NbPackParams()
        for k in ("c_ha", "c_o3", "c_s2", "c_dg", "c_sh", "inv_L"):
            getattr(P, k)[:] = [float(v) for v in vals[k]]
        for k in ("gs", "ambient", "edge", "dx"):
            setattr(P, k, float(vals[k]))
        if shock_on is None:
            shock_on = any(float(v) != 0.0 for v in vals["c_sh"])                # render.py:734
        packed, packed2 = self.render_scratch()
        out, tmp = (packed2, packed) if smooth else (packed, packed2)          # render.py:725-730
        self._chk(self._lib.nb_render_pack(self._h, C.byref(P), 1 if shock_on else 0, 1 if smooth else 0,
                                           C.c_void_p(out.ptr), C.c_void_p(tmp.ptr)), "nb_render_pack")
        return out

    def write_frame(self, root, frame):
        """np.save the frame files f####_{g0,rho,xi,df,sh}.npy as bake.py:95-102 does"""
        import os
        fr = self.frame()
        p = os.path.join(root, "frames", f"f{frame:04d}")
        os.makedirs(os.path.dirname(p), exist_ok=True)
        for k in ("g0", "rho", "xi", "df", "sh"):
            np.save(f"{p}_{k}.npy", fr[k])
        return fr

    def time_label(self):
        if self.phase == "pre":
            return f"pre-turb {self.tp:.3f}/{self.P['pre_t']:.2f}"
        return f"t={self.t:.4f}"

    def stats(self):
        xi = self._xi
        r = self._rho
        return dict(ion=float(xi.double().mean()), rho_max=float(r.max()), rho_min=float(r.min()))

    def conservation(self):
        """FP64 totals (mass, x/y/z momentum) of the current state, times the cell volume."""
        out = (C.c_double * 4)()
        self._chk(self._lib.nb_reduce_fp64(self._h, out), "nb_reduce_fp64")
        v = self.dx ** 3
        return tuple(float(x) * v for x in out)

    def footprint(self):
        """device bytes this instance holds: its fields and the library's scratch for it"""
        out = C.c_longlong()
        self._chk(self._lib.nb_instance_bytes(self._h, None, 0, C.byref(out)), "nb_instance_bytes")
        fields = sum(t.numel() * t.element_size() for t in (self._rho, self._mx, self._my, self._mz, self._xi,
                                                            self._stage, self._dfront, self._g0))
        return fields + int(out.value)

    def invalidate(self):
        """call after writing rho / m / xi directly: the next step recomputes the CFL max speed"""
        self._chk(self._lib.nb_invalidate(self._h), "nb_invalidate")

"""A launch-shape autotuner for one simulation instance.

Knobs (nb_set_tuning): the tile depth along i of the hydro march (`chunk_i`: the tile shape of
the persistent 2.5-D sweep), the tile sweep order (`tile_order`), the lanes per ray of the
ionizing and FUV ray kernels (`ray_group`, `fuv_group`), and the layouts of the ray-front and FUV
attenuation tables (`front_pairs`, `fuv_pairs`: neighbour pairs or single entries; the same bits
either way).  Each knob is tuned in turn
(coordinate descent) on the instance's own state: the state and clock are saved, every
candidate runs a few steps (or FUV passes) timed by the library's per-kernel CUDA events, the
state is restored, and the fastest candidate is kept.  The hydro result never depends on these
knobs; the ray sums only through rounding.  Results are cached per problem shape.
"""
import ctypes as C

from . import _lib

CANDIDATES = {
    "chunk_i": (16, 20, 24, 32, 64),
    "tile_order": (0, 1),
    "ray_group": (1, 2, 4, 8),
    "fuv_group": (8, 16, 32),
    "front_pairs": (0, 1),
    "fuv_pairs": (0, 1),
}
# which kernel kinds a knob moves (names of _lib.PROF_KINDS)
AFFECTS = {"chunk_i": ("stage1", "stage2"), "tile_order": ("stage1", "stage2"), "ray_group": ("cast_rays",),
           "fuv_group": ("cast_fuv",), "front_pairs": ("cast_rays", "apply_front"),
           "fuv_pairs": ("cast_fuv", "apply_fuv")}

_CACHE = {}


def _key(sim):
    return (tuple(sim.shape), len(sim.stars), tuple(sim.rfront.shape), tuple(sim.att.shape), sim.P.get("solver"),
            sim.arith)


def get(sim, knob):
    v = C.c_int()
    _lib.check(sim._lib.nb_get_tuning(sim._h, _lib.TUNE[knob], C.byref(v)), sim._h, "nb_get_tuning")
    return int(v.value)


def put(sim, knob, value):
    _lib.check(sim._lib.nb_set_tuning(sim._h, _lib.TUNE[knob], int(value)), sim._h, "nb_set_tuning")


def _measure(sim, knob, steps):
    lib = sim._lib
    ms = (C.c_double * 16)()
    n = (C.c_longlong * 16)()
    lib.nb_profile(sim._h, 1)
    lib.nb_profile_read(sim._h, ms, n)
    if knob in ("fuv_group", "fuv_pairs"):
        for _ in range(steps):
            sim.fuv_field()
    elif knob in ("ray_group", "front_pairs"):
        for _ in range(steps):
            sim.ionize()
    else:
        sim.step(steps, sync=False)
    lib.nb_profile_read(sim._h, ms, n)
    lib.nb_profile(sim._h, 0)
    idx = [_lib.PROF_KINDS.index(k) for k in AFFECTS[knob]]
    return sum(ms[i] for i in idx) / steps


def autotune(sim, knobs=None, steps=4, use_cache=True):
    """pick the fastest launch shapes for `sim` (its state and clock are left unchanged);
    returns {knob: (value, ms per step or pass of the kernels it moves)}"""
    key = _key(sim)
    if use_cache and key in _CACHE:
        for k, (v, _) in _CACHE[key].items():
            put(sim, k, v)
        return dict(_CACHE[key])
    sim._sync()
    saved = {k: getattr(sim, "_" + k).clone() for k in ("rho", "mx", "my", "mz", "xi", "dfront", "g0")}
    meta = sim.get_state_meta()                    # clocks, stirring state, forcing Generator
    book = {k: getattr(sim, k) for k in ("_it", "version", "rf_version", "fuv_version", "fuv_nstars", "fuv_phase")
            if hasattr(sim, k)}

    def restore():
        for k, t in saved.items():
            getattr(sim, "_" + k).copy_(t)
        sim.set_state_meta(meta)
        for k, v in book.items():
            setattr(sim, k, v)

    knobs = list(knobs or CANDIDATES)
    orig = {k: get(sim, k) for k in knobs}
    out = {}
    ok = False
    try:
        for knob in knobs:
            best = None
            for v in CANDIDATES[knob]:
                put(sim, knob, v)
                restore()
                _measure(sim, knob, 1)                 # warm the launch path
                restore()
                t = _measure(sim, knob, steps)
                if best is None or t < best[1]:
                    best = (v, t)
            put(sim, knob, best[0])
            out[knob] = best
        ok = True
    finally:                                           # a failed candidate leaves no trace
        sim._lib.nb_profile(sim._h, 0)
        if not ok:
            for k, v in orig.items():
                put(sim, k, v)
        restore()
        sim._sync()
    _CACHE[key] = dict(out)
    return out

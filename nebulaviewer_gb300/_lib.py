"""ctypes binding of libnebula.so / libnebula_fast.so (include/nebula.h).

The libraries are built in-tree by `nebulaviewer_gb300.build.build()`; loading one that is
missing raises immediately: there is no CPU or PyTorch fallback for the simulation step.
Two builds of the same ABI: "exact" (every float operation the reference's: bit-identical
results) and "fast" (FMA contraction, approximate division / square root, flush-to-zero:
within the path's tolerance of the exact build).  DEFAULT_ARITH is what a Sim uses unless
told otherwise (environment variable NEBULA_ARITH overrides it).
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATHS = {"exact": os.path.join(HERE, "libnebula.so"), "fast": os.path.join(HERE, "libnebula_fast.so")}
LIB_PATH = LIB_PATHS["exact"]
DEFAULT_ARITH = os.environ.get("NEBULA_ARITH", "fast")

NB_ABI_VERSION = 2
NB_OK = 0
NB_DEV_TMA_TIMEOUT = 1      # nb_device_status bit: a hydro stage's bounded TMA wait gave up
NB_DEV_DRIVE_EMPTY = 2      # nb_device_status bit: a stirred step found no forcing field B
ERRORS = {-1: "NB_ERR_ARG", -2: "NB_ERR_CUDA", -3: "NB_ERR_STATE", -4: "NB_ERR_LIMIT", -5: "NB_ERR_TIMEOUT",
          -6: "NB_ERR_NOMEM"}
SOLVERS = {"rusanov": 0, "hll": 1}
LIMITERS = {"minmod": 0, "vanleer": 1, "mc": 2}
STAR_KINDS = {"main": 0, "abs": 1}
JET_KINDS = {"jet": 0, "proto": 1, "none": 2}


class NbFields(C.Structure):
    _fields_ = [("rho", C.c_void_p), ("mx", C.c_void_p), ("my", C.c_void_p), ("mz", C.c_void_p),
                ("xi", C.c_void_p), ("stage", C.c_void_p), ("dfront", C.c_void_p), ("g0", C.c_void_p)]


class NbDesc(C.Structure):
    _fields_ = [("abi_version", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("dx", C.c_double), ("cn2", C.c_double), ("ci2", C.c_double), ("floor_rho", C.c_double),
                ("vmax", C.c_double), ("cfl", C.c_double), ("solver", C.c_int), ("limiter", C.c_int),
                ("nu", C.c_int), ("nphi", C.c_int), ("dr", C.c_double), ("nsteps", C.c_int), ("diag", C.c_double),
                ("fnr", C.c_int), ("fnu", C.c_int), ("fnphi", C.c_int), ("fields_fp32", C.c_int),
                ("max_stars", C.c_int), ("f", NbFields), ("stream", C.c_void_p)]


class NbLive(C.Structure):
    _fields_ = [("q_main", C.c_double), ("wind", C.c_double), ("jet", C.c_double), ("jet_proto", C.c_double),
                ("jet_pulse", C.c_double), ("jet_period", C.c_double), ("kappa_fuv", C.c_double),
                ("q_ramp", C.c_double), ("jet_angle_deg", C.c_double), ("jet_r", C.c_double),
                ("dt_cap", C.c_double), ("phase_main", C.c_int), ("plane_flux", C.c_double),
                ("plane_fuv", C.c_double), ("pre_amp", C.c_double), ("drive_main", C.c_double)]


class NbStar(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double), ("qf", C.c_double), ("t_on", C.c_double),
                ("ax", C.c_double), ("ay", C.c_double), ("az", C.c_double), ("kind", C.c_int), ("jkind", C.c_int)]


class NbClock(C.Structure):
    _fields_ = [("t", C.c_double), ("dt", C.c_double), ("it", C.c_int64), ("tp", C.c_double), ("ip", C.c_int64)]


class NbDriveDesc(C.Structure):
    _fields_ = [("sx", C.c_int), ("sy", C.c_int), ("sz", C.c_int), ("slots", C.c_int), ("dxs", C.c_double),
                ("pre_corr", C.c_double), ("clock", C.c_double)]


class NbDriveInfo(C.Structure):
    _fields_ = [("clock", C.c_double), ("swaps", C.c_int64), ("pushed", C.c_int64), ("status", C.c_int),
                ("pad", C.c_int)]


class NbPackParams(C.Structure):
    _fields_ = [("c_ha", C.c_float * 3), ("c_o3", C.c_float * 3), ("c_s2", C.c_float * 3), ("c_dg", C.c_float * 3),
                ("c_sh", C.c_float * 3), ("gs", C.c_float), ("ambient", C.c_float), ("edge", C.c_float),
                ("inv_L", C.c_float * 3), ("dx", C.c_float)]


# name -> (restype, argtypes): every symbol include/nebula.h declares
_P = C.c_void_p
_F4 = C.c_void_p * 4
SIGNATURES = {
    "nb_create": (C.c_int, [C.POINTER(NbDesc), C.POINTER(_P)]),
    "nb_destroy": (None, [_P]),
    "nb_instance_bytes": (C.c_int, [_P, C.POINTER(NbDesc), C.c_int, C.POINTER(C.c_longlong)]),
    "nb_last_error": (C.c_char_p, [_P]),
    "nb_device_status": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "nb_set_live": (C.c_int, [_P, C.POINTER(NbLive)]),
    "nb_set_stars": (C.c_int, [_P, C.POINTER(NbStar), C.c_int]),
    "nb_set_clock": (C.c_int, [_P, C.POINTER(NbClock)]),
    "nb_get_clock": (C.c_int, [_P, C.POINTER(NbClock)]),
    "nb_peek_clock": (C.c_int, [_P, C.POINTER(NbClock)]),
    "nb_mirror_clock": (C.c_int, [_P]),
    "nb_step": (C.c_int, [_P, C.c_int, C.c_int]),
    "nb_ionize": (C.c_int, [_P]),
    "nb_fuv": (C.c_int, [_P]),
    "nb_invalidate": (C.c_int, [_P]),
    "nb_drive_config": (C.c_int, [_P, C.POINTER(NbDriveDesc)]),
    "nb_drive_push": (C.c_int, [_P, _P, C.c_int]),
    "nb_drive_enable": (C.c_int, [_P, C.c_int]),
    "nb_drive_state": (C.c_int, [_P, C.POINTER(NbDriveInfo)]),
    "nb_pre_step": (C.c_int, [_P, C.c_int]),
    "nb_drive_step": (C.c_int, [_P, _P, _P, C.c_float, C.c_float, C.c_float]),
    "nb_add_torus": (C.c_int, [_P, _P]),
    "nb_mach_sums": (C.c_int, [_P, C.c_double * 2]),
    "nb_hydro_stage": (C.c_int, [_P, _F4, _F4, _F4, C.c_float, C.c_float, C.c_float, C.c_float]),
    "nb_max_speed": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "nb_cast_rays": (C.c_int, [_P, C.c_double * 3, C.c_double, _P]),
    "nb_cast_fuv": (C.c_int, [_P, C.c_double * 3, _P]),
    "nb_reduce_fp64": (C.c_int, [_P, C.c_double * 4]),
    "nb_profile": (C.c_int, [_P, C.c_int]),
    "nb_profile_read": (C.c_int, [_P, C.c_double * 16, C.c_longlong * 16]),
    "nb_counters": (C.c_int, [_P, C.POINTER(C.c_longlong)]),
    "nb_set_tuning": (C.c_int, [_P, C.c_int, C.c_int]),
    "nb_get_tuning": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int)]),
    "nb_snapshot_pack": (C.c_int, [_P, _P]),
    "nb_snapshot_unpack": (C.c_int, [_P, _P]),
    "nb_frame_pack": (C.c_int, [_P, _P]),
    "nb_shock": (C.c_int, [_P, _P]),
    "nb_render_pack": (C.c_int, [_P, C.POINTER(NbPackParams), C.c_int, C.c_int, _P, _P]),
    "nb_batch_create": (C.c_int, [C.POINTER(_P), C.POINTER(C.c_int), C.c_int, C.POINTER(_P)]),
    "nb_batch_step": (C.c_int, [_P, C.c_int]),
    "nb_batch_set_option": (C.c_int, [_P, C.c_int, C.c_int]),
    "nb_batch_counters": (C.c_int, [_P, C.POINTER(C.c_longlong)]),
    "nb_batch_destroy": (None, [_P]),
    "nb_batch_set_active": (C.c_int, [_P, C.POINTER(C.c_int), C.c_int]),
    "nb_batch_last_error": (C.c_char_p, [_P]),
    "nb_reduce_fp64_static": (C.c_int, [_P, _P, _P, _P, C.c_longlong, _P, _P]),
    "nb_static_last_error": (C.c_char_p, []),
}
TUNE = {"chunk_i": 0, "ray_group": 1, "fuv_group": 2, "tile_order": 3, "front_cull": 4, "fuv_cut": 5,
        "wait_limit": 6, "stall_test": 7, "front_pairs": 8, "fuv_pairs": 9}
PROF_KINDS = ["ctrl", "stage1", "stage2", "cast_rays", "apply_front", "smooth", "cast_fuv", "apply_fuv", "max_speed",
              "snapshot", "drive", "render"]

_libs = {}


class NebulaError(RuntimeError):
    pass


def arith_of(arith):
    a = DEFAULT_ARITH if arith is None else arith
    if a not in LIB_PATHS:
        raise ValueError(f"arith must be one of {sorted(LIB_PATHS)}, not {a!r}")
    return a


def load(arith=None, path=None):
    """Load libnebula.so ("exact") or libnebula_fast.so ("fast") once; `path` loads another build
    of the same ABI.  Raises if the file is missing: build it first."""
    key = path or arith_of(arith)
    if key in _libs:
        return _libs[key]
    p = path or LIB_PATHS[key]
    if not os.path.exists(p):
        raise NebulaError(f"{p} is missing: run nebulaviewer_gb300.build.build() (nvcc, sm_103a) first")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _libs[key] = lib
    return lib


def check(rc, handle=None, what="", lib=None):
    """raise NebulaError with the library's message for a non-zero status (`lib`: the library
    that returned it; for a handle, either build reads the handle's own message)"""
    if rc != NB_OK:
        lib = lib or load()
        msg = lib.nb_last_error(handle).decode(errors="replace")
        raise NebulaError(f"{what}: {ERRORS.get(rc, rc)}: {msg}")
    return rc


def f4(ptrs):
    return _F4(*[C.c_void_p(int(p)) for p in ptrs])

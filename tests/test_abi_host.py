"""CPU tests: the C-ABI library loads and exports every symbol include/nebula.h declares;
host-side logic (parameters, ray budgets, initial conditions, ctypes layouts)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def header_symbols():
    src = open(os.path.join(ROOT, "include", "nebula.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(nb_\w+)\s*\(", src, re.M)))


@pytest.mark.parametrize("arith", ("exact", "fast"))
def test_library_exports_every_declared_symbol(lib_built, arith):
    """both builds (exact and fast code generation) export every symbol the header declares"""
    from nebulaviewer_gb300 import _lib
    lib = _lib.load(arith)
    names = header_symbols()
    assert len(names) >= 17
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_lib.SIGNATURES), "ctypes signatures must cover the header exactly"


def test_struct_layouts_match_header(tmp_path):
    """every ctypes mirror has the size and field offsets the C compiler gives the header's struct"""
    import shutil
    import subprocess
    from nebulaviewer_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = {"nb_desc": _lib.NbDesc, "nb_fields": _lib.NbFields, "nb_live": _lib.NbLive, "nb_star": _lib.NbStar,
               "nb_clock": _lib.NbClock, "nb_drive_desc": _lib.NbDriveDesc, "nb_drive_info": _lib.NbDriveInfo}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "nebula.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    inc = os.path.join(ROOT, "include")
    subprocess.run([cc, "-std=c11", "-I", inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in mirrors.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_null_handle_errors_without_gpu(lib_built):
    from nebulaviewer_gb300 import _lib
    lib = _lib.load()
    assert lib.nb_step(None, 1, 1) == -1
    assert b"null" in lib.nb_last_error(None)
    d = _lib.NbDesc()
    d.abi_version = 999
    h = C.c_void_p()
    assert lib.nb_create(C.byref(d), C.byref(h)) == -1
    assert b"abi" in lib.nb_last_error(None)
    d.abi_version = _lib.NB_ABI_VERSION
    d.nx, d.ny, d.nz = 8, 8, 6           # nz not a multiple of 4
    assert lib.nb_create(C.byref(d), C.byref(h)) == -1
    # ray indices are 32-bit: rays per star times max_stars must stay below 2^32 (checked before
    # anything touches the device)
    d.nz = 8
    d.dx, d.dr, d.nsteps = 0.125, 0.125, 16
    d.fnr, d.fnu, d.fnphi = 16, 8, 16
    d.nu, d.nphi, d.max_stars = 4096, 8192, 128                      # 2^32 ray groups
    assert lib.nb_create(C.byref(d), C.byref(h)) == -4
    assert b"2^32" in lib.nb_last_error(None)
    d.nu, d.nphi, d.fnu, d.fnphi = 8, 16, 4096, 8192                 # the FUV rays likewise
    assert lib.nb_create(C.byref(d), C.byref(h)) == -4


def test_params_defaults_and_sound_speeds():
    from nebulaviewer_gb300.params import make_params, sound_speeds
    P = make_params()
    assert P["cfl"] == 0.3 and P["floor"] == 2e-3 and P["solver"] == "hll" and P["q_ramp"] == 0.02
    assert sound_speeds(P) == ((1 / 12.0) ** 2, 1.0, 6.0)
    assert sound_speeds(dict(P, cn2=1.0, ci2=144.0, vmax=72.0)) == (1.0, 144.0, 72.0)


def test_ray_budget_matches_reference_rule():
    from nebulaviewer_gb300.sim import _ray_budget
    assert _ray_budget(256, True, None, None) == ((512, 1024), (160, 160, 320))
    assert _ray_budget(128, True, None, None) == ((512, 1024), (128, 128, 256))
    assert _ray_budget(512, True, None, None) == ((1024, 2048), (256, 256, 512))
    assert _ray_budget(64, False, (8, 16), (4, 8, 16)) == ((8, 16), (4, 8, 16))


def test_synthetic_ics_are_seeded_and_shaped():
    from nebulaviewer_gb300 import ics
    a = ics.torus(res=8)
    b = ics.torus(res=8)
    assert a["rho"].shape == (16, 16, 16)
    assert np.array_equal(a["rho"].numpy(), b["rho"].numpy())
    assert abs(a["stars"][0][0] - 1.0) < 1e-12 and abs(a["P"]["q_main"] - 0.25 ** 3 / 3) < 1e-15
    s = ics.sheet(res=32)
    assert s["rho"].shape == (32, 32, 32) and len(s["stars"]) == 6
    v = np.stack([m.numpy() / s["rho"].numpy() for m in s["mom"]])
    assert 2.0 < np.sqrt((v ** 2).sum(0).mean()) < 8.0          # rms Mach ~5 at cs_n = 1
    c = ics.cliffwall(res=32, nclumps=4)
    r = c["rho"].numpy()
    assert r[:4].max() < 3.0 and r[-4:].min() > 150.0


def test_sheet_and_torus_follow_their_stated_distributions():
    """the turbulent sheet: slab profile 1 + 49 exp(-(y/0.1)^2) (n = 50 at the mid-plane) times a
    log-normal of sigma 0.5, a divergence-free velocity of rms Mach 5 at cs_n = 1, six stars in the
    slab with photon rates inside one decade; the torus: background n = 1 and Q = n^2 R^3 / 3 of a
    Stromgren radius 0.25"""
    from nebulaviewer_gb300 import ics
    n = 64
    s = ics.sheet(res=n)
    rho = s["rho"].numpy().astype(np.float64)
    dx = s["dx"]
    y = (np.arange(n) + 0.5) * dx
    prof = np.exp(-((y - 0.5) / 0.1) ** 2)[None, :, None]
    ln = np.log(rho / (1.0 + 49.0 * prof))
    assert 0.45 < ln.std() < 0.55 and abs(ln.mean() + 0.125) < 0.05       # exp(sigma g - sigma^2 / 2)
    v = np.stack([m.numpy() / s["rho"].numpy() for m in s["mom"]]).astype(np.float64)
    assert 4.5 < np.sqrt((v ** 2).sum(0).mean()) < 5.5
    div = sum(np.gradient(v[a], dx, axis=a) for a in range(3))
    grad = np.sqrt(sum(np.gradient(v[c], dx, axis=a) ** 2 for c in range(3) for a in range(3)))
    assert np.abs(div).mean() < 0.05 * grad.mean()
    assert len(s["stars"]) == 6
    for x, sy, z, qf, ton in s["stars"]:
        assert abs(sy - 0.5) <= 0.03 and 0.2 <= x <= 0.8 and 0.2 <= z <= 0.8 and 1.0 <= qf <= 10.0 and ton == 0.0
    t = ics.torus(res=32)
    assert 0.9 < float(np.median(t["rho"].numpy())) < 1.1
    assert abs(t["P"]["q_main"] - 5.208e-3) < 1e-6


def test_product_path_does_not_import_the_oracle():
    """the package must never route through the CPU oracle"""
    pkg = os.path.join(ROOT, "nebulaviewer_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                src = open(os.path.join(dirpath, f)).read()
                assert not re.search(r"^\s*(import|from)\s+oracle\b", src, re.M), f
                assert "liboracle" not in src and "ref_cpu" not in src, f


def _state_kwargs(shape, rho_shape=None, mom_shape=None, torus_shape=None):
    rho = np.ones(rho_shape or shape, np.float32)
    mom = None if mom_shape is None else [np.zeros(mom_shape, np.float32)] * 3
    torus = None if torus_shape is None else np.zeros(torus_shape, np.float32)
    return dict(shape=shape, dx=0.01, rho=rho, stars=[(0.1, 0.1, 0.1, 1.0)], kinds=["main"], jets=[(0.0, 0.0, 1.0)],
                jkinds=[None], P={}, mom=mom, torus=torus, device="cpu")


@pytest.mark.parametrize("bad", ("rho", "mom", "torus", "dims"))
def test_fields_of_another_shape_are_refused_before_the_library(bad):
    """every field the kernels index by the grid shape must have that shape (no library call yet)"""
    from nebulaviewer_gb300.sim import Sim
    g = (8, 8, 8)
    kw = {"rho": _state_kwargs(g, rho_shape=(8, 8, 4)), "mom": _state_kwargs(g, mom_shape=(8, 8 * 8)),
          "torus": _state_kwargs(g, torus_shape=(4, 8, 8)), "dims": _state_kwargs((0, 8, 8))}[bad]
    with pytest.raises(ValueError):
        Sim.from_state(**kw)


def test_forcing_fields_of_another_shape_are_refused():
    """the library copies whole forcing fields of the forcing grid from the host buffer"""
    from nebulaviewer_gb300.sim import Sim
    s = Sim.__new__(Sim)
    s.sshape = (4, 5, 6)
    s._h = None
    for buf in (np.zeros((2, 3, 4, 5, 5), np.float32), np.zeros((2, 3, 4, 5, 6), np.float64),
                np.zeros((3, 4, 5, 6), np.float32)):
        with pytest.raises(ValueError):
            s._push_forcing(buf)

"""bench.py's clock sampler on a stand-in nvidia-smi (a script printing one CSV line every 20 ms):
started ahead of the timed region it keeps only the samples that arrived inside the region, reads
the throttle reasons, and its child process does not outlive the region.  No GPU."""
import importlib.util
import math
import os
import stat
import sys
import time

import pytest

from conftest import ROOT

FAKE = """#!{py}
import sys, time
i = 0
while True:
    reason = "Active" if i % 2 else "Not Active"
    print(f"0, {{1900 + i}}, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, {{reason}}", flush=True)
    i += 1
    time.sleep(0.02)
"""


@pytest.fixture
def bench(tmp_path, monkeypatch):
    exe = tmp_path / "nvidia-smi"
    exe.write_text(FAKE.format(py=sys.executable))
    exe.chmod(exe.stat().st_mode | stat.S_IEXEC)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_samples_come_from_the_timed_region_only(bench):
    pytest.importorskip("torch")
    clk = bench.ClockSampler(0).start()
    time.sleep(0.5)                               # the warm-up: samples here are not the region's
    with clk:
        time.sleep(0.3)
    s = clk.summary()
    assert s is not None and 5 <= s["samples"] <= 25, s
    assert s["sm_max_mhz"] == 2070.0
    clock = lambda ln: float(ln.split(",")[1])  # noqa: E731  (the fake's clock rises line by line)
    before = [clock(ln) for t, ln in clk.arrived if t < clk.window[0]]
    assert before and min(clock(ln) for ln in clk.lines) > max(before)   # the warm-up's lines were left out
    assert s["reasons"] == ["sw_power_cap"]
    assert clk.p.poll() is not None               # the sampler process ended with the region


def test_no_sampler_no_clocks(bench, monkeypatch):
    pytest.importorskip("torch")
    monkeypatch.setenv("PATH", "/nonexistent")
    with bench.ClockSampler(0) as clk:
        pass
    assert clk.summary() is None


def _box_range(o, d, bmax):
    """nebula3d.py:229-244, one ray at a time"""
    t0, t1 = 0.0, 1e9
    for a in range(3):
        if abs(d[a]) < 1e-9:
            if o[a] < 0.0 or o[a] > bmax[a]:
                t1 = -1.0
        else:
            ta, tb = (0.0 - o[a]) / d[a], (bmax[a] - o[a]) / d[a]
            t0, t1 = max(t0, min(ta, tb)), min(t1, max(ta, tb))
    return t0, t1


def _ray_dir(iu, ip, nu, nphi):
    u = -1.0 + (iu + 0.5) * 2.0 / nu
    s = math.sqrt(max(1.0 - u * u, 0.0))
    phi = (ip + 0.5) * 2.0 * math.pi / nphi
    return (s * math.cos(phi), s * math.sin(phi), u)


def test_ray_march_samples_counts_the_reference_loops(bench):
    """the bench's sample count against the reference's loops walked one sample at a time in
    uniform gas (cast_rays: break at the front crossing; cast_fuv: break past the last bin), with
    the fronts from the oracle's cast_rays; some rays leave the box before their front"""
    import numpy as np
    import oracle as O
    shape, dx, dens = (16, 12, 20), 1.0 / 16, 2.0
    L = [n * dx for n in shape]
    diag = math.sqrt(sum(x * x for x in L)) + 0.6
    star, Q = (0.3, 0.55, 0.7), 4.0 * 0.3 ** 3 / 3.0              # front radius 0.3 at n = 2
    for dr in (dx, 0.5 * dx):
        nsteps = int(diag / dr) + 1
        nu, nphi = 8, 16
        rf = O.Kernels(np.float32).cast_rays(np.full(shape, dens, np.float32), star, Q, dr, nsteps, dx, diag,
                                             np.array(L), nu, nphi)
        assert (rf < diag).any() and (rf == np.float32(diag)).any()
        want = 0
        for iu in range(nu):
            for ip in range(nphi):
                d = _ray_dir(iu, ip, nu, nphi)
                t0, t1 = _box_range(star, d, L)
                col = 0.0
                for n in range(int(t0 / dr), min(nsteps, int(t1 / dr) + 2)):
                    r = (n + 0.5) * dr
                    inside = all(0.0 <= star[a] + d[a] * r <= L[a] for a in range(3))
                    nv = dens if inside else 0.0           # sample_n is 0 outside (nebula3d.py:197-205)
                    inc = nv * nv * r * r * dr
                    want += 1
                    if col + inc > Q:
                        break
                    col += inc
        assert bench.ray_march_samples(star, L, dr, nsteps, nu, nphi, rfront=rf, rcap=diag) == want
        fnr, fnu, fnp = 10, 6, 12
        binr = diag / fnr
        want = 0
        for iu in range(fnu):
            for ip in range(fnp):
                t0, t1 = _box_range(star, _ray_dir(iu, ip, fnu, fnp), L)
                ib = 0
                for n in range(int(t0 / dr), min(nsteps, int(t1 / dr) + 2)):
                    want += 1
                    nb = int((n + 0.5) * dr / binr)
                    ib = max(ib, nb)
                    if ib >= fnr:
                        break
        assert bench.ray_march_samples(star, L, dr, nsteps, fnu, fnp, rstop=diag) == want
        # a star near a corner, with a last radial bin inside the box: the bin cut decides
        got = bench.ray_march_samples((0.02, 0.02, 0.02), L, dr, nsteps, fnu, fnp, rstop=0.5)
        want = 0
        for iu in range(fnu):
            for ip in range(fnp):
                t0, t1 = _box_range((0.02, 0.02, 0.02), _ray_dir(iu, ip, fnu, fnp), L)
                for n in range(int(t0 / dr), min(nsteps, int(t1 / dr) + 2)):
                    want += 1
                    if (n + 0.5) * dr >= 0.5:
                        break
        assert got == want


def test_ray_rates_on_a_stand_in_instance(bench):
    """ray_rates' glue on a stand-in Sim (the attributes the real one has) and a stand-in
    nb_cast_rays that writes a fixed front: samples per launch and Gsamples/s per kernel kind"""
    import ctypes as C
    import types
    import numpy as np
    torch = pytest.importorskip("torch")
    nu, nphi, front = 8, 16, 0.2

    def cast(h, xyz, Q, ptr):
        buf = np.full(nu * nphi, front, np.float32)
        C.memmove(ptr.value, buf.ctypes.data, buf.nbytes)
        return 0

    L, dx = (1.0, 1.0, 1.0), 1.0 / 16
    diag = math.sqrt(3.0) + 0.6
    sim = types.SimpleNamespace(
        active_stars=lambda: [(0.5, 0.5, 0.5, 1.0, 0.0), (0.3, 0.6, 0.5, 0.5, 0.0)],
        rfront=types.SimpleNamespace(shape=(nu, nphi)), att=types.SimpleNamespace(shape=(10, 6, 12)),
        _rho=torch.zeros(1), _h=None, P={"q_main": 1.0}, L=L, dr=dx, nsteps=int(diag / dx) + 1, diag=diag)
    lib = types.SimpleNamespace(nb_cast_rays=cast)
    out = bench.ray_rates(sim, lib, {"cast_rays": (2.0, 4), "cast_fuv": (1.0, 1)})
    ion = sum(bench.ray_march_samples(s[:3], L, dx, sim.nsteps, nu, nphi, rfront=np.full((nu, nphi), front),
                                      rcap=diag) for s in sim.active_stars())
    fuv = sum(bench.ray_march_samples(s[:3], L, dx, sim.nsteps, 6, 12, rstop=diag) for s in sim.active_stars())
    assert out["stars"] == 2 and ion == 2 * nu * nphi * 4          # the front at 0.2 ends every ray at n = 3
    assert out["cast_rays"] == {"samples_per_launch": ion, "gsamples_per_s": ion / 0.5e-3 / 1e9}
    assert out["cast_fuv"] == {"samples_per_launch": fuv, "gsamples_per_s": fuv / 1e-3 / 1e9}

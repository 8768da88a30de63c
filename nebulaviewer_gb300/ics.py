"""Seeded synthetic initial conditions for the benchmark / parity workloads.

The reference builds its clouds on the host with NumPy/SciPy (nebula3d.py:391-576,
sim.py:113-348); that set-up runs once per reset and is not part of the step.  These
generators make the workloads this package is measured on, with fixed seeds:

  torus      box [-1,1]^3 (shifted to [0,2]^3): a torus of radius 0.4, tube radius 0.15
             at n = 100 on a background n = 1, times a log-normal (sigma 0.3); at rest;
             one central star with a Stromgren radius of 0.25 in the background.
  sheet      box [0,1]^3: a Gaussian slab of thickness 0.2 at n = 50 on n = 1, times a
             log-normal (sigma 0.5); a solenoidal k^-4 velocity field of rms Mach 5;
             stars seeded inside the sheet with rates log-uniform over one decade.
  cliffwall  box [0,1]^3: a density step n = 1 -> 200 at mid-x with seeded Gaussian clumps
             (n = 500-2000, radius 0.01-0.05) on its face; 3 stars in the low-density side.
  torus_stirred  the torus scene with a stirring phase first (as the reference's bipolar
             scenario, sim.py:51, 667-672): the log-normal background is stirred to
             supersonic turbulence for pre_t, then the torus joins and the star switches on;
             stirring continues at drive_main x pre_amp in the main phase.

Random fields are sums of seeded random plane waves (resolution independent, so a small
and a large grid of the same scenario share their large scales) evaluated with torch on
the requested device.
"""

import numpy as np
import torch


def _modes(rng, n, kmin, kmax, slope, solenoidal=False):
    """n random plane waves: wavevectors (cycles/unit) log-uniform in [kmin, kmax] with
    isotropic directions; amplitudes so that the shell spectrum goes as k^(2 - slope)
    (a 3-D power spectrum k^-slope); normalised to unit total variance."""
    lk = rng.uniform(np.log(kmin), np.log(kmax), n)
    k = np.exp(lk)
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    ph = rng.uniform(0.0, 2 * np.pi, n)
    amp = np.sqrt(k ** (3.0 - slope))
    amp /= np.sqrt(np.sum(amp ** 2) / 2.0)
    e = None
    if solenoidal:
        e = rng.standard_normal((n, 3))
        e -= np.sum(e * d, axis=1, keepdims=True) * d           # perpendicular to k: divergence free
        e /= np.linalg.norm(e, axis=1, keepdims=True)
    return 2 * np.pi * k[:, None] * d, ph, amp, e


def _eval(shape, dx, kv, ph, amp, device, comp=None):
    nx, ny, nz = shape
    x = (torch.arange(nx, device=device, dtype=torch.float64) + 0.5) * dx
    y = (torch.arange(ny, device=device, dtype=torch.float64) + 0.5) * dx
    z = (torch.arange(nz, device=device, dtype=torch.float64) + 0.5) * dx
    out = torch.zeros(shape, device=device, dtype=torch.float32)
    for m in range(len(ph)):
        a = amp[m] if comp is None else amp[m] * comp[m]
        if a == 0.0:
            continue
        arg = (kv[m, 0] * x)[:, None, None] + (kv[m, 1] * y)[None, :, None] + (kv[m, 2] * z)[None, None, :] + ph[m]
        out += (a * torch.sin(arg)).to(torch.float32)
    return out


def grf(shape, dx, seed, slope, n=96, kmin=1.0, kmax=None, device="cpu"):
    """unit-variance Gaussian-like random field (sum of n seeded plane waves)"""
    kmax = kmax or 1.0 / (8.0 * dx)
    rng = np.random.default_rng(seed)
    kv, ph, amp, _ = _modes(rng, n, kmin, max(kmax, kmin * 1.01), slope)
    return _eval(shape, dx, kv, ph, amp, device)


def solenoidal_velocity(shape, dx, seed, slope, rms, n=96, kmin=1.0, kmax=None, device="cpu"):
    kmax = kmax or 1.0 / (8.0 * dx)
    rng = np.random.default_rng(seed)
    kv, ph, amp, e = _modes(rng, n, kmin, max(kmax, kmin * 1.01), slope, solenoidal=True)
    s = rms                       # total variance of |v| is 1 before scaling
    return [s * _eval(shape, dx, kv, ph, amp, device, comp=e[:, c]) for c in range(3)]


def torus(res=32, seed=1, device="cpu", shape=None, nstars=1, stir=False):
    """the torus scene; `shape` gives a non-cubic box (dx = 2 / min(shape), torus at the centre),
    `nstars` > 1 adds seeded weaker stars near the centre; `stir` returns the torus apart
    (it joins when the stirring phase ends) with the stirring parameters in P"""
    if shape is None:
        shape = (2 * res, 2 * res, 2 * res)
        dx = 1.0 / res
    else:
        shape = tuple(int(v) for v in shape)
        dx = 2.0 / min(shape)
    c = [0.5 * s * dx for s in shape]
    ax = [(torch.arange(s, device=device, dtype=torch.float64) + 0.5) * dx - cc for s, cc in zip(shape, c)]
    X, Y, Z = ax[0][:, None, None], ax[1][None, :, None], ax[2][None, None, :]
    d = torch.sqrt((torch.sqrt(X * X + Y * Y) - 0.4) ** 2 + Z * Z)
    inside = 0.5 * (1.0 - torch.tanh((d - 0.15) / dx))
    sig = 0.3
    g = grf(shape, dx, seed, 3.8, device=device).to(torch.float64)
    ln = torch.exp(sig * g - 0.5 * sig * sig)
    rho = ((1.0 + 99.0 * inside) * ln).to(torch.float32)
    torus_part = None
    if stir:
        torus_part = (99.0 * inside * ln).to(torch.float32)
        rho = ln.to(torch.float32)
    Q = 0.25 ** 3 / 3.0                       # n^2 R^3 / 3 with n = 1, R = 0.25 (no 4 pi in cast_rays)
    P = dict(q_main=Q, wind=0.0, jet=0.0, q_ramp=0.0, kappa_fuv=10.0, cn2=1.0, ci2=144.0, vmax=72.0,
             solver="hll", limiter="minmod", cfl=0.3, floor=2e-3, seed=seed, ion_every=2)
    stars = [(c[0], c[1], c[2], 1.0, 0.0)]
    rng = np.random.default_rng(seed + 3000)
    for _ in range(nstars - 1):
        off = rng.uniform(-0.3, 0.3, 3)
        stars.append((c[0] + off[0], c[1] + off[1], c[2] + off[2], float(rng.uniform(0.1, 0.5)), 0.0))
    if stir:
        # sound speed 1: stirring to supersonic turbulence in pre_t = 0.05, forcing renewed every 0.02
        P.update(pre_t=0.05, pre_amp=60.0, pre_corr=0.02, pre_kmax=4.0, drive_main=0.25)
    return dict(shape=shape, dx=dx, rho=rho, mom=None, stars=stars, kinds=["main"] * nstars,
                jets=[(0.0, 0.0, 1.0)] * nstars, jkinds=["none"] * nstars, P=P, torus=torus_part)


def torus_stirred(res=32, seed=1, device="cpu", shape=None, nstars=1):
    return torus(res=res, seed=seed, device=device, shape=shape, nstars=nstars, stir=True)


def sheet(res=256, seed=2, nstars=6, device="cpu", shape=None):
    shape = shape or (res, res, res)
    dx = 1.0 / res
    ny = shape[1]
    y = (torch.arange(ny, device=device, dtype=torch.float64) + 0.5) * dx
    y0 = 0.5 * ny * dx
    prof = torch.exp(-((y - y0) / 0.1) ** 2)[None, :, None]
    sig = 0.5
    g = grf(shape, dx, seed, 4.0, device=device).to(torch.float64)
    rho = ((1.0 + 49.0 * prof) * torch.exp(sig * g - 0.5 * sig * sig)).to(torch.float32)
    v = solenoidal_velocity(shape, dx, seed + 1000, 4.0, 5.0, device=device)
    mom = [(rho * vc).contiguous() for vc in v]
    rng = np.random.default_rng(seed + 2000)
    L = [s * dx for s in shape]
    q_main = 2e-3
    stars = []
    for _ in range(nstars):
        p = (rng.uniform(0.2, 0.8) * L[0], y0 + rng.uniform(-0.03, 0.03), rng.uniform(0.2, 0.8) * L[2])
        qf = float(np.exp(rng.uniform(0.0, np.log(10.0))))          # log-uniform over one decade
        stars.append((float(p[0]), float(p[1]), float(p[2]), qf, 0.0))
    P = dict(q_main=q_main, wind=0.5, jet=0.0, q_ramp=0.0, kappa_fuv=10.0, cn2=1.0, ci2=144.0, vmax=72.0,
             solver="hll", limiter="minmod", cfl=0.3, floor=2e-3, seed=seed, ion_every=2)
    return dict(shape=tuple(shape), dx=dx, rho=rho, mom=mom, stars=stars, kinds=["main"] * nstars,
                jets=[(0.0, 0.0, 1.0)] * nstars, jkinds=["none"] * nstars, P=P)


def cliffwall(res=1024, seed=5, nclumps=40, device="cpu", shape=None):
    shape = shape or (res, res, res)
    dx = 1.0 / res
    nx, ny, nz = shape
    rho = torch.empty(shape, device=device, dtype=torch.float32)
    x = (torch.arange(nx, device=device, dtype=torch.float64) + 0.5) * dx
    x0 = 0.5 * nx * dx
    wall = (0.5 * (1.0 + torch.tanh((x - x0) / dx))).to(torch.float32)
    rho[:] = (1.0 + 199.0 * wall)[:, None, None]
    rng = np.random.default_rng(seed)
    y = (torch.arange(ny, device=device, dtype=torch.float64) + 0.5) * dx
    z = (torch.arange(nz, device=device, dtype=torch.float64) + 0.5) * dx
    for _ in range(nclumps):
        c = (x0 + rng.uniform(-0.02, 0.02), rng.uniform(0.05, 0.95) * ny * dx, rng.uniform(0.05, 0.95) * nz * dx)
        r = rng.uniform(0.01, 0.05)
        amp = rng.uniform(500.0, 2000.0)
        h = int(4 * r / dx) + 1
        sl = []
        for ci, n in zip(c, shape):
            q = int(ci / dx)
            sl.append(slice(max(q - h, 0), min(q + h + 1, n)))
        X = x[sl[0]][:, None, None]
        Y = y[sl[1]][None, :, None]
        Z = z[sl[2]][None, None, :]
        rr = (X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2
        rho[sl[0], sl[1], sl[2]] += (amp * torch.exp(-rr / (2 * r * r))).to(torch.float32)
    L = [s * dx for s in shape]
    stars = [(0.25 * L[0], 0.5 * L[1], 0.5 * L[2], 1.0, 0.0),
             (0.15 * L[0], 0.3 * L[1], 0.65 * L[2], 0.5, 0.0),
             (0.3 * L[0], 0.7 * L[1], 0.35 * L[2], 0.4, 0.0)]
    # plane-parallel source from -x: the flux ionizes the n = 1 side (column 0.5 x 1^2) and about
    # 0.02 into the n = 200 wall (200^2 x 0.02 = 800)
    P = dict(q_main=5e-3, wind=0.0, jet=0.0, q_ramp=0.0, kappa_fuv=10.0, cn2=1.0, ci2=144.0, vmax=72.0,
             solver="hll", limiter="minmod", cfl=0.3, floor=2e-3, seed=seed, ion_every=2,
             plane_flux=0.5 * nx * dx + 200.0 ** 2 * 0.02, plane_fuv=5.0)
    return dict(shape=tuple(shape), dx=dx, rho=rho, mom=None, stars=stars, kinds=["main"] * 3,
                jets=[(0.0, 0.0, 1.0)] * 3, jkinds=["none"] * 3, P=P)


SCENARIOS = {"torus": torus, "torus_stirred": torus_stirred, "sheet": sheet, "cliffwall": cliffwall}


def batch_scenes(n=32, seed=7, device="cpu", lo=64, hi=192):
    """The batched workload: n instances, cubes with edges drawn uniformly from [lo, hi]
    (multiples of 8) plus cropped slabs such as 96 x 160 x 288 (every fourth instance), each
    the torus or the sheet with its own seed and 1-8 stars."""
    rng = np.random.default_rng(seed)
    out = []
    slabs = [(96, 160, 288), (160, 96, 224), (128, 192, 96)]
    for m in range(n):
        if m % 4 == 3:
            shape = slabs[(m // 4) % len(slabs)]
        else:
            e = int(rng.integers(lo // 8, hi // 8 + 1)) * 8
            shape = (e, e, e)
        ns = int(rng.integers(1, 9))
        s = int(rng.integers(1, 1 << 30))
        if rng.random() < 0.5:
            ic = torus(seed=s, device=device, shape=shape, nstars=ns)
        else:
            ic = sheet(res=min(shape), seed=s, nstars=ns, device=device, shape=shape)
        out.append(ic)
    return out

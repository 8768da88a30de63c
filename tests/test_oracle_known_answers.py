"""CPU: the oracle against answers known from the physics, beside the golden fixtures.

The same known answers are asserted on the CUDA path in test_gpu_parity.py; here they
check the oracle itself, so a restatement slip that the fixtures' small cases miss
still shows up."""
import numpy as np
import pytest

import oracle as O

# reference units (sim.py:740-741, nebula3d.py:589-591): floor 2e-3, CFL 0.3
CN2, CI2, VMAX, FLOOR = 1.0, 144.0, 72.0, 2e-3
NO_STARS = np.zeros((1, 4), np.float32)


def _stage(K, U, xi, dt, dx, solver=1, lim=0, U0=None, a=0.0, b=1.0):
    out = [np.zeros_like(U[0]) for _ in range(4)]
    K.hydro_stage(U, xi, U if U0 is None else U0, out, NO_STARS, 0, 0.0, NO_STARS, 0.9, 0.3, 0.0, dt, dx, a, b,
                  FLOOR, CN2, CI2, VMAX, solver, lim)
    return out


@pytest.mark.parametrize("dtype", (np.float32, np.float64))
@pytest.mark.parametrize("solver,lim", ((0, 0), (1, 0), (1, 1), (1, 2)))
def test_uniform_gas_at_rest_stays_exactly_at_rest(dtype, solver, lim):
    """a uniform state at rest has equal left and right face states everywhere: both RK2
    stages return the input bits, ionized or not"""
    K = O.Kernels(dtype)
    n, dx = 12, 1.0 / 12
    for xi_val in (0.0, 0.37, 1.0):
        U = [np.full((n, n, n), 3.0, dtype)] + [np.zeros((n, n, n), dtype) for _ in range(3)]
        xi = np.full((n, n, n), xi_val, dtype)
        dt = 0.3 * dx / np.sqrt(CN2 + xi_val * (CI2 - CN2))
        U1 = _stage(K, U, xi, dt, dx, solver, lim)
        U2 = _stage(K, U1, xi, dt, dx, solver, lim, U0=U, a=0.5, b=0.5)
        for u, u1, u2 in zip(U, U1, U2):
            assert np.array_equal(u1, u) and np.array_equal(u2, u)


@pytest.mark.parametrize("solver", (0, 1))
def test_mass_telescopes_when_the_boundary_is_at_rest(solver):
    """with uniform gas at rest on every boundary face no mass crosses the box edge, so the
    face fluxes telescope: the FP64 re-run conserves total mass to rounding"""
    K = O.Kernels(np.float64)
    n, dx = 24, 1.0 / 24
    c = (np.arange(n) + 0.5) * dx - 0.5
    x, y, z = np.meshgrid(c, c, c, indexing="ij")
    r2 = x * x + y * y + z * z
    blob = np.maximum(1.0 - r2 / 0.25 ** 2, 0.0) ** 2          # zero beyond r = 0.25
    rho = 1.0 + 40.0 * blob
    U = [rho, 3.0 * x * blob * rho, -2.0 * y * blob * rho, 1.5 * z * blob * rho]
    xi = np.clip(1.0 - r2 / 0.05, 0.0, 1.0)
    edge = np.abs(np.stack([x, y, z])).max(axis=0) > 0.5 - 3 * dx
    assert blob[edge].max() == 0.0 and xi[edge].max() == 0.0   # uniform and at rest within 3 cells of the edge
    dt = 0.3 * dx / 12.0
    U1 = _stage(K, U, xi, dt, dx, solver)
    U2 = _stage(K, U1, xi, dt, dx, solver, U0=U, a=0.5, b=0.5)
    m0 = np.sum(U[0])
    assert abs(np.sum(U1[0]) - m0) / m0 < 1e-13
    assert abs(np.sum(U2[0]) - m0) / m0 < 1e-13
    assert np.abs(U2[0] - U[0]).max() > 1e-3                  # the blob did move


@pytest.mark.parametrize("dtype", (np.float32, np.float64))
def test_stromgren_radius_uniform_gas(dtype):
    """the front radius in uniform density n is (3Q/n^2)^(1/3) (the column is the integral of
    n^2 r^2 dr, sim.py / nebula3d.py:247-270 use no 4 pi) within half a ray step"""
    K = O.Kernels(dtype)
    n, dx, dens = 32, 1.0 / 32, 2.0
    Q = 4.0 * 0.2 ** 3 / 3.0                                   # R = 0.2 at n = 2
    R = (3 * Q / dens ** 2) ** (1.0 / 3.0)
    L = np.array([1.0, 1.0, 1.0])
    diag = float(np.linalg.norm(L)) + 0.6
    rho = np.full((n, n, n), dens, dtype)
    for dr in (dx, 0.5 * dx):
        ns = int(diag / dr) + 1
        rf = K.cast_rays(rho, (0.5, 0.5, 0.5), Q, dr, ns, dx, diag, L, 16, 32)
        assert np.abs(rf - R).max() < 0.5 * dr


def test_front_apply_marks_the_stromgren_sphere():
    """apply_front on a spherical front of radius R: cells well inside are ionized, cells
    well outside neutral, and dfront is the signed distance r - R"""
    K = O.Kernels(np.float32)
    n, dx, R = 32, 1.0 / 32, 0.2
    rf = np.full((16, 32), R, np.float32)
    xi = np.zeros((n, n, n), np.float32)
    df = np.full((n, n, n), 1e3, np.float32)
    K.apply_front(rf, (0.5, 0.5, 0.5), dx, 1.2 * dx, xi, df)
    c = (np.arange(n) + 0.5) * dx - 0.5
    x, y, z = np.meshgrid(c, c, c, indexing="ij")
    r = np.sqrt(x * x + y * y + z * z)
    assert np.all(xi[r < R - 0.7 * dx] == 1.0) and np.all(xi[r > R + 0.7 * dx] == 0.0)
    assert np.abs(df - (r - R)).max() < 1e-5


def test_plain_torus64_fp32_scheme_against_fp64_rerun():
    """the plain-step workload (torus 64^3, one central star of Stromgren radius 0.25, HLL +
    minmod, RK2, CFL 0.3, 100 steps) on the oracle in float32 and in float64: the float32 scheme
    stays within the path's tolerance of the FP64 re-run (rel-Linf 1e-3 after 100 steps; it is
    ~1e-6 here), the ionized masks agree except on at most 0.1% of cells, the clocks agree"""
    from nebulaviewer_gb300 import ics
    from nebulaviewer_gb300.params import make_params, sound_speeds
    ic = ics.torus(res=32)
    P = make_params(base=ic["P"])
    cn2, ci2, vmax = sound_speeds(P)
    args = (ic["shape"], ic["dx"], ic["rho"].numpy(), ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"], P)
    kw = dict(rays=(256, 512), fuv_grid=(64, 64, 128), cn2=cn2, ci2=ci2, vmax=vmax)
    o64 = O.OracleSim(*args, dtype=np.float64, **kw)
    o32 = O.OracleSim(*args, dtype=np.float32, **kw)
    o64.step(100)
    o32.step(100)
    for k in ("rho", "mx", "my", "mz", "xi"):
        a, b = getattr(o32, k).astype(np.float64), getattr(o64, k)
        assert np.abs(a - b).max() / np.abs(b).max() < 1e-5, k
    m32, m64 = o32.xi > 0.5, o64.xi > 0.5
    assert m64.any() and (m32 != m64).mean() <= 1e-3
    assert abs(o32.t - o64.t) / o64.t < 1e-6

"""Precision: the FP32 GPU path against an FP64 re-run of the same scheme (the oracle's double
instantiation), on the plain-step workload (torus 64^3, one central star, HLL + minmod, RK2,
CFL 0.3, 100 steps).  The FP32 CPU oracle (the reference scheme in float32) is run beside it so
the GPU's error is compared with the error the float32 reference scheme itself carries."""
import numpy as np
import pytest

from conftest import rel_linf

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("arith", ("exact", "fast"))
def test_fp32_error_against_fp64_rerun_torus64(arith):
    import oracle as O
    from nebulaviewer_gb300 import build, ics
    from nebulaviewer_gb300.params import make_params, sound_speeds
    from nebulaviewer_gb300.sim import Sim
    build.build(verbose=False)
    ic = ics.torus(res=32)
    P = make_params(base=ic["P"])
    cn2, ci2, vmax = sound_speeds(P)
    rays, fuv = (256, 512), (64, 64, 128)
    args = (ic["shape"], ic["dx"], ic["rho"].numpy(), ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"], P)
    kw = dict(rays=rays, fuv_grid=fuv, cn2=cn2, ci2=ci2, vmax=vmax)
    o64 = O.OracleSim(*args, dtype=np.float64, **kw)
    o32 = O.OracleSim(*args, dtype=np.float32, **kw)
    g = Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"], ic["P"],
                       rays=rays, fuv_grid=fuv, arith=arith)
    steps = 100
    o64.step(steps)
    o32.step(steps)
    g.step(steps)
    rows = []
    for k in ("rho", "mx", "my", "mz", "xi"):
        ref = getattr(o64, k)
        gv = getattr(g, k).numpy()
        cv = getattr(o32, k)
        rows.append((k, rel_linf(gv, ref), rel_l2(gv, ref), rel_linf(cv, ref), rel_l2(cv, ref)))
    print(f"\nfield  gpu32-vs-fp64 Linf  L2   | cpu32-vs-fp64 Linf  L2   (torus 64^3, 100 steps, {arith})")
    for r in rows:
        print(f"{r[0]:5s}  {r[1]:.3e}  {r[2]:.3e}  |  {r[3]:.3e}  {r[4]:.3e}")
    print(f"t: gpu {g.t!r} fp64 {o64.t!r} cpu32 {o32.t!r}")
    for k, gi, g2, ci, c2 in rows:
        # the GPU's FP32 result is as close to the FP64 re-run as the reference scheme's FP32 is
        assert g2 <= 3.0 * c2 + 1e-6, (k, g2, c2)
        assert g2 < 1e-3, (k, g2)
        assert gi < 1e-3, (k, gi)                 # the stated rel-L_inf after 100 steps
    assert abs(g.t - o64.t) / o64.t < 1e-4
    g.close()

"""Parameter dictionary `P` of the simulation (the keys the step reads), with the
reference's default values.

The reference builds P in layers (sim.py:102-110 make_params): the argparse defaults of
nebula3d.py (nebula3d.py:581-638), EXTRA_DEFAULTS (sim.py:75-76), VIEWER_DEFAULTS
(sim.py:77), a scenario preset, BOX_DEFAULTS.  Only the keys the simulation step consumes
are listed here, with the same names and values, so a P dict from the reference works
unchanged.  Three keys are additions of this package: `cn2`, `ci2`, `vmax` override the
reference's fixed (1/ci_over_cn)^2, 1 and 6 (sim.py:740-741, 1020), which lets a scenario
use sound speeds cs_n = 1, cs_i = 12 (cn2 = 1, ci2 = 144, vmax = 72) instead.
"""

# nebula3d.py:581-638 (argparse defaults used by the step)
STEP_DEFAULTS = dict(
    cfl=0.3, ci_over_cn=12.0, floor=2e-3, q_main=2.5e-3, wind=0.0, ion_every=2, kappa_fuv=25.0,
    max_stars=32, jet=0.0, jet_proto=0.0, jet_angle=10.0, jet_r=0.04, jet_pulse=0.6, jet_period=0.02,
    pre_t=0.0, pre_amp=1.5, pre_corr=0.06, pre_kmax=6.0, drive_main=0.0, trigger=0.0, seed=3, t_end=0.25,
    frames=60,
)
# sim.py:75-77 EXTRA_DEFAULTS / VIEWER_DEFAULTS (the step-relevant ones)
STEP_DEFAULTS.update(q_ramp=0.02, solver="hll", limiter="minmod", box=1.0)

# sim.py:82-83 parameters that may change while the simulation runs
LIVE = ("q_main", "wind", "jet", "jet_proto", "jet_pulse", "jet_period", "kappa_fuv", "drive_main", "pre_amp",
        "q_ramp")


def make_params(overrides=None, base=None):
    p = dict(STEP_DEFAULTS)
    if base:
        p.update(base)
    if overrides:
        p.update(overrides)
    return p


def sound_speeds(P):
    """(cn2, ci2, vmax) of sim.py:740-741, 1020, or the explicit overrides."""
    cn2 = float(P["cn2"]) if "cn2" in P else (1.0 / P["ci_over_cn"]) ** 2
    ci2 = float(P["ci2"]) if "ci2" in P else 1.0
    vmax = float(P["vmax"]) if "vmax" in P else 6.0
    return cn2, ci2, vmax

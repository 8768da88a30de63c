"""GB300 (sm_103a) implementation of NebulaViewer's simulation step.

`Sim` is the drop-in for the reference's `sim.Sim` on the step / ionize path; the kernels
live in libnebula.so (csrc/, C ABI in include/nebula.h), built in-tree by `build.build()`.
"""
from .params import LIVE, STEP_DEFAULTS, make_params  # noqa: F401


def __getattr__(name):
    if name == "Sim":
        from .sim import Sim
        return Sim
    if name == "Field":
        from .sim import Field
        return Field
    raise AttributeError(name)

"""A float32 stand-in for the `warp` runtime, used ONLY to execute the reference's
own kernel source (nebula3d.py / sim.py) on the CPU when generating golden fixtures.

Test infrastructure: nothing in the product imports this module.

`warp-lang` is not installed here and cannot be installed (no network), so the
reference cannot run as shipped.  Its kernels are ordinary Python functions under
`@wp.kernel` / `@wp.func`; this module supplies just the builtins those bodies
call, with Warp's documented scalar semantics restated in numpy float32:

* every `float` in a kernel body (literals, `float(i)` casts, arguments annotated
  `float`) is IEEE float32, evaluated op by op with no fused multiply-add;
* `vecN` arithmetic is component-wise; `vec / s` divides each component by `s`;
  `dot(a, b)` is `0 + a0*b0 + a1*b1 + ...` left to right; `length = sqrt(dot)`;
* `max(a, b) = a > b ? a : b`, `min(a, b) = a < b ? a : b`,
  `clamp(x, lo, hi) = min(max(lo, x), hi)`; `int()` truncates toward zero;
* `sqrt` is correctly rounded; `sin/cos/atan2/exp/floor` are numpy's float32
  versions (a transcendental may differ from CUDA's by an ulp or two);
* `float16(x)` rounds to nearest-even;
* a launch runs its threads one after another in row-major tid order.

What this does NOT reproduce: Warp's code generator (whether nvrtc contracts a*b+c
into an FMA on the GPU) and its own transcendental implementations.
"""
import itertools
import math
import sys
import types

import numpy as np

f32 = np.float32


# ----------------------------------------------------------------------------- vectors
class _Vec:
    __slots__ = ("v",)
    __array_ufunc__ = None          # make numpy scalars defer to our __rmul__
    N = 0

    def __init__(self, *args):
        if len(args) == 1 and isinstance(args[0], (tuple, list, np.ndarray, _Vec)):
            vals = tuple(args[0])
        elif len(args) == 1:
            vals = (args[0],) * self.N
        else:
            vals = args
        if len(vals) != self.N:
            raise ValueError(f"{type(self).__name__} needs {self.N} components, got {len(vals)}")
        self.v = tuple(f32(x) for x in vals)

    @classmethod
    def _of(cls, vals):
        o = object.__new__(cls)
        o.v = tuple(vals)
        return o

    def __getitem__(self, i):
        return self.v[i]

    def __iter__(self):
        return iter(self.v)

    def __len__(self):
        return self.N

    def __add__(self, o):
        return self._of(a + b for a, b in zip(self.v, o.v))

    def __sub__(self, o):
        return self._of(a - b for a, b in zip(self.v, o.v))

    def __neg__(self):
        return self._of(-a for a in self.v)

    def __mul__(self, s):
        if isinstance(s, _Vec):
            raise TypeError("vec * vec is not a Warp operator")
        s = f32(s)
        return self._of(a * s for a in self.v)

    def __rmul__(self, s):
        s = f32(s)
        return self._of(s * a for a in self.v)

    def __truediv__(self, s):
        s = f32(s)
        return self._of(a / s for a in self.v)

    def __repr__(self):
        return f"{type(self).__name__}{tuple(float(x) for x in self.v)}"


class vec2(_Vec):
    N = 2


class vec3(_Vec):
    N = 3


class vec4(_Vec):
    N = 4


class vec4h:
    """four float16 components (render.py's packed voxel), mutable as Warp's vectors are"""
    __array_ufunc__ = None

    def __init__(self, *args):
        vals = args if args else (0.0, 0.0, 0.0, 0.0)
        self.v = [np.float16(x) for x in vals]

    def __getitem__(self, i):
        return self.v[i]

    def __setitem__(self, i, x):
        self.v[i] = np.float16(x)

    def __iter__(self):
        return iter(self.v)

    def __len__(self):
        return 4


def cw_mul(a, b):
    return a._of(x * y for x, y in zip(a.v, b.v))


def struct(cls):
    """@wp.struct: instances convert assigned values to the annotated Warp types (float -> float32)"""
    ann = dict(getattr(cls, "__annotations__", {}))

    def __setattr__(self, name, value):
        t = ann.get(name)
        if t is float:
            value = f32(value)
        elif t is int:
            value = int(value)
        elif isinstance(t, type) and issubclass(t, _Vec) and not isinstance(value, _Vec):
            value = t(*value)
        object.__setattr__(self, name, value)

    cls.__setattr__ = __setattr__
    return cls


class Texture3D:                     # annotation only (render.py's ray marcher is not run here)
    pass


class TextureFilterMode:
    LINEAR = 1
    CLOSEST = 0


class TextureAddressMode:
    CLAMP = 0
    WRAP = 1


float32 = np.float32
float16 = np.float16
uint8 = np.uint8
int32 = np.int32
uint32 = np.uint32
pi = f32(math.pi)
LOG_WARNING = 2
config = types.SimpleNamespace(log_level=None, quiet=False, mode="release")


def _isfloat(x):
    return isinstance(x, (float, np.floating))


def _num(x):
    return f32(x) if _isfloat(x) else x


# ----------------------------------------------------------------------------- scalar builtins
def max(a, b):  # noqa: A001  (Warp builtin name)
    a, b = _num(a), _num(b)
    return a if a > b else b


def min(a, b):  # noqa: A001
    a, b = _num(a), _num(b)
    return a if a < b else b


def clamp(x, lo, hi):
    return min(max(lo, x), hi)


def abs(x):  # noqa: A001
    return f32(np.abs(f32(x))) if _isfloat(x) else (x if x >= 0 else -x)


def sqrt(x):
    return f32(np.sqrt(f32(x)))


def floor(x):
    return f32(np.floor(f32(x)))


def sin(x):
    return f32(np.sin(f32(x)))


def cos(x):
    return f32(np.cos(f32(x)))


def exp(x):
    return f32(np.exp(f32(x)))


def atan2(y, x):
    return f32(np.arctan2(f32(y), f32(x)))


def where(c, a, b):
    return _num(a) if c else _num(b)


def dot(a, b):
    r = f32(0.0)
    for x, y in zip(a.v, b.v):
        r = r + x * y
    return r


def length(a):
    return sqrt(dot(a, a))


_TID = [None]


def tid():
    return _TID[0]


def atomic_max(arr, idx, val):
    cur = arr[idx]
    if val > cur:
        arr[idx] = val
    return cur


def atomic_add(arr, idx, val):
    cur = arr[idx]
    arr[idx] = cur + f32(val)
    return cur


# ----------------------------------------------------------------------------- host arrays
def _dt(dtype):
    if dtype in (float, None, np.float32, float32):
        return np.float32
    return dtype


class array:
    """host-memory stand-in for wp.array (numpy storage; vec4 arrays are (n, 4) float32)"""

    def __init__(self, data=None, dtype=float, shape=None, device=None, _np=None, **kw):
        self.dtype = _dt(dtype)
        self.is_vec = self.dtype in (vec4, vec3, vec2)
        if _np is not None:
            self.np = _np
        elif data is None:                       # wp.array(dtype=...) as an annotation
            self.np = np.zeros(0, np.float32 if self.is_vec else self.dtype)
        else:
            base = np.float32 if self.is_vec else self.dtype
            self.np = np.array(data, dtype=base, copy=True)
        self.shape = self.np.shape[:1] if self.is_vec else self.np.shape

    # the reference's host code uses these
    def numpy(self):
        return self.np.copy()

    def fill_(self, v):
        self.np[...] = v

    def zero_(self):
        self.np[...] = 0

    def assign(self, x):
        self.np[...] = np.asarray(x).reshape(self.np.shape)

    def __getitem__(self, k):
        if isinstance(k, int):
            return array(dtype=self.dtype, _np=self.np[k])
        raise IndexError("host indexing is limited to a leading int")

    def kernel_view(self):
        if self.is_vec:
            cls = self.dtype
            return [cls._of(f32(x) for x in row) for row in self.np]
        return self.np


def _shape(s):
    return (s,) if isinstance(s, int) else tuple(s)


def _alloc(shape, dtype):
    dt = _dt(dtype)
    if dt in (vec4, vec3, vec2):
        return np.zeros(_shape(shape) + (dt.N,), np.float32)
    return np.zeros(_shape(shape), dt)


def zeros(shape, dtype=float, device=None):
    return array(dtype=dtype, _np=_alloc(shape, dtype))


def empty(shape, dtype=float, device=None):
    return zeros(shape, dtype, device)


def full(shape, value, dtype=float, device=None):
    a = zeros(shape, dtype, device)
    a.fill_(value)
    return a


def copy(dst, src):
    dst.np[...] = src.np


def array3d(dtype=float):
    return ("array3d", dtype)


def array2d(dtype=float):
    return ("array2d", dtype)


def init():
    pass


def synchronize():
    pass


# ----------------------------------------------------------------------------- kernels
_BUILT = {}          # module name -> globals dict with float32 `float` and rebuilt funcs


def _rebuild(fn, g):
    return types.FunctionType(fn.__code__, g, fn.__name__, fn.__defaults__, fn.__closure__)


def _kernel_globals(modname):
    """A copy of the module's globals in which `float` is float32 and every
    @wp.func / @wp.kernel is re-bound to this copy (host code keeps the real module)."""
    if modname in _BUILT:
        return _BUILT[modname]
    mod = sys.modules[modname]
    g = dict(mod.__dict__)
    g["float"] = np.float32
    _BUILT[modname] = g
    for name, val in list(g.items()):
        if getattr(val, "_wp_func", False):
            g[name] = _rebuild(val, g)
        elif isinstance(val, Kernel):
            g[name] = val
    # sim.py reaches nebula3d's funcs as attributes of the module `N`
    for name, val in list(g.items()):
        if isinstance(val, types.ModuleType) and hasattr(val, "hydro_stage") and val.__name__ != modname:
            g[name] = types.SimpleNamespace(**_kernel_globals(val.__name__))
    return g


class Kernel:
    def __init__(self, fn):
        self.fn = fn
        self.key = fn.__name__
        self._built = None
        self.__name__ = fn.__name__

    def _compiled(self):
        if self._built is None:
            self._built = _rebuild(self.fn, _kernel_globals(self.fn.__module__))
        return self._built

    def run(self, dim, inputs):
        f = self._compiled()
        ann = self.fn.__annotations__
        names = self.fn.__code__.co_varnames[:self.fn.__code__.co_argcount]
        args = []
        for n, a in zip(names, inputs):
            t = ann.get(n)
            if isinstance(a, array):
                args.append(a.kernel_view())
            elif t is float:
                args.append(f32(a))
            elif t is int:
                args.append(int(a))
            elif isinstance(t, type) and issubclass(t, _Vec) and not isinstance(a, _Vec):
                args.append(t(*a))
            else:
                args.append(a)
        dims = _shape(dim)
        with np.errstate(all="ignore"):
            for idx in itertools.product(*[range(d) for d in dims]):
                _TID[0] = idx if len(idx) > 1 else idx[0]
                f(*args)


def kernel(fn=None, **kw):
    if fn is None:
        return lambda f: Kernel(f)
    return Kernel(fn)


def func(fn):
    fn._wp_func = True
    return fn


def launch(kernel, dim, inputs, device=None, **kw):
    kernel.run(dim, inputs)


def install():
    """register this module as `warp` (call before importing the reference)"""
    sys.modules["warp"] = sys.modules[__name__]

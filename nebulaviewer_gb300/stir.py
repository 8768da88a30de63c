"""Host side of the turbulent stirring: the forcing grid and the solenoidal forcing fields.

The reference stirs with a cross-fade of two random divergence-free fields on a coarse grid
(nebula3d.py:763-776, sim.py:760-768, 801-804); a new field is drawn every `pre_corr` of
simulated time.  The fields are small (a few thousand to a few hundred thousand cells) and
drawn on the host from the simulation's NumPy Generator, so a Generator in the same state
yields the same field as the reference; the device kernels only sample them.
"""
import math

import numpy as np

# sim.py:761-763: 24 forcing cells per domain unit, whatever the grid resolution
PHYSICAL_DXS = 1.0 / 24.0
CELLS_PER_FORCING_CELL = 6          # sim.py:766-768 / nebula3d.py:764-766: one per 6 grid cells


def forcing_grid(L, dx, shape, physical=True):
    """(sshape, dxs) of the forcing grid: a fixed physical spacing of 1/24 domain units
    (sim.py:761-764, resolution independent) or one forcing cell per 6 grid cells
    (sim.py:766-768); two cells of margin per axis either way."""
    if physical:
        return tuple(int(math.ceil(L_ / PHYSICAL_DXS)) + 2 for L_ in L), PHYSICAL_DXS
    f = CELLS_PER_FORCING_CELL
    return tuple(n // f + 2 for n in shape), f * float(dx)


def solenoidal(shape, rng, kmin=1.0, kmax=6.0):
    """A unit-RMS divergence-free random vector field on a periodic grid of `shape`, as three
    float32 arrays (nebula3d.py:514-525).

    Fourier modes with kmin <= |k| <= kmax (k in integer cycles per grid) get complex Gaussian
    coefficients of amplitude 1/|k|, independently per component; each mode's component along k
    is then removed (the Helmholtz projection F -> F - k (k.F)/|k|^2), the field is transformed
    back and its real part kept, and the three components are scaled together to a total RMS of
    one.  The Generator is drawn in the reference's order (per component: a standard-normal array
    for the real parts, then one for the imaginary parts) and every array operation follows the
    reference's order, so equal Generator states give bit-identical fields."""
    waves = np.meshgrid(*[np.fft.fftfreq(n) * n for n in shape], indexing="ij")
    kmag = np.sqrt(sum(w * w for w in waves))
    weight = np.where((kmag >= kmin) & (kmag <= kmax), 1.0 / np.maximum(kmag, 1e-6), 0.0)
    coef = [weight * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) for _ in range(3)]
    along = sum(w * c for w, c in zip(waves, coef)) / np.maximum(kmag * kmag, 1e-12)
    coef = [c - w * along for w, c in zip(waves, coef)]
    comps = [np.fft.ifftn(c).real for c in coef]
    rms = np.sqrt(sum((v * v).mean() for v in comps))
    return [np.ascontiguousarray(v / rms, dtype=np.float32) for v in comps]


MATCHED_MODES = 32                   # sim.py:276: the matched spectrum covers |m| <= 32


def _matched_coefficients(shape, seed, call, modes):
    """Complex Gaussian coefficients on the full FFT grid of `shape` whose low modes |m| <= modes
    come from a master spectrum that depends only on (seed, call) -- so every grid size gets the
    same large-scale coefficients -- and whose other modes depend on the grid size as well
    (sim.py:282-304 for a grid without a half-spectrum axis).  Draw order: the master real
    parts then imaginary parts on a (2 modes + 1)^3 grid from a Generator seeded with
    [seed, 7919, call]; then the grid's own real and imaginary parts from one seeded with
    [seed, 104729, call, *shape]; the master values replace the grid's at the matched modes."""
    side = 2 * modes + 1
    g = np.random.default_rng([seed, 7919, call])
    master = g.standard_normal((side,) * len(shape)) + 1j * g.standard_normal((side,) * len(shape))
    g = np.random.default_rng([seed, 104729, call, *shape])
    out = g.standard_normal(shape) + 1j * g.standard_normal(shape)
    grid_ix, master_ix = [], []
    for n in shape:
        top = min(modes, (n - 1) // 2)
        m = np.arange(-top, top + 1)
        grid_ix.append(m % n)
        master_ix.append(m % side)
    out[np.ix_(*grid_ix)] = master[np.ix_(*master_ix)]
    return out


def matched_solenoidal(shape, seed, calls, kmin=1.0, kmax=6.0, modes=MATCHED_MODES):
    """The forcing field the reference draws in its default "matched" initial-condition mode
    (sim.py:327-337 MatchedNoise.solenoidal, used by sim.py:801-804): the construction of
    `solenoidal` with each component's coefficients taken from _matched_coefficients instead of
    the Generator.  `calls` is the generator's call count before this field; the field uses the
    next three (one per component).  Returns the three float32 components, bit-identical to the
    reference's for the same seed, count and shape."""
    waves = np.meshgrid(*[np.fft.fftfreq(n) * n for n in shape], indexing="ij")
    kmag = np.sqrt(sum(w * w for w in waves))
    weight = np.where((kmag >= kmin) & (kmag <= kmax), 1.0 / np.maximum(kmag, 1e-6), 0.0)
    coef = [weight * _matched_coefficients(shape, seed, calls + 1 + c, modes) for c in range(3)]
    along = sum(w * c for w, c in zip(waves, coef)) / np.maximum(kmag * kmag, 1e-12)
    coef = [c - w * along for w, c in zip(waves, coef)]
    comps = [np.fft.ifftn(c).real for c in coef]
    rms = np.sqrt(sum((v * v).mean() for v in comps))
    return [np.ascontiguousarray(v / rms, dtype=np.float32) for v in comps]

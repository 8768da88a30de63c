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

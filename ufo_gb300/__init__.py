"""ufo_gb300: GB300-native particle tracking behind UFO's Python API.

The names below mirror the reference's package exports (ufo/__init__.py:3-23)
for the tracking path: lattices and elements, ``Track``, ``StableAperture``,
``ClosedOrbit``, ``Optics``, ``chromaticity``, ``emittance`` /
``RadiationIntegrals``, ``Beam``, the physical constants, the flags and the
``DEFAULT_*_SLICES`` knobs.  The OpenCL context plumbing
(``list_devices``/``context``) becomes CUDA device selection.
"""
DEFAULT_QUADRUPOLE_SLICES = 8
DEFAULT_BEND_SLICES = 8
DEFAULT_MULTIPOLE_SLICES = 4
DEFAULT_SEXTUPOLE_SLICES = 4
DEFAULT_OCTUPOLE_SLICES = 4

from .flags import (LINEAR, FIVED, EXACT, KICK, RADIATION, DOUBLE_PRECISION,  # noqa: E402
                    ACHROMATIC, YOSHIDA, FMA)
from .elements import (Element, Marker, Drift, Multipole, Quadrupole, Sbend, Rbend,  # noqa: E402
                       Sextupole, Octupole, Wire, Aperture)
from .lattice import Lattice, Line, Beam  # noqa: E402
from .constants import *  # noqa: E402,F401,F403
from .radiation import emittance, RadiationIntegrals  # noqa: E402


def __getattr__(name):
    # the GPU drivers load the CUDA library lazily so that lattice work and the
    # CPU test-suite run without a GPU
    if name in ('Track', 'StableAperture', 'ClosedOrbit', 'Optics', 'chromaticity',
                'list_devices', 'context', 'Context'):
        from . import drivers
        return getattr(drivers, name)
    if name in ('TrackBatch', 'autotune'):
        from . import batch
        return getattr(batch, name)
    raise AttributeError(name)


__all__ = ['Lattice', 'Line', 'Track', 'StableAperture', 'ClosedOrbit', 'Optics']

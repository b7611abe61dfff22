"""Python host side of the GB300-native granular contact library.

A thin ctypes layer over the C ABI in ``include/dpg.h`` (``_build/libdpg.so``),
mirroring the reference's ``Particle`` / ``Integrator`` interface
(include/particles/base/particle.h, include/integrator/*.h of
mmccraw98/dpCUDA-v2): ``Disk`` exposes the same method names
(updateVelocities, updatePositions, checkForNeighborUpdate, calculateForces,
getPowerFire, mixVelocitiesAndForces, ...), and ``NVE``, ``Fire``, ``Adam``,
``minimizeFire`` and ``minimizeAdam`` drive it like the reference's
integrators and routines.

There is no CPU fallback: importing works anywhere, but creating a system
needs the CUDA library and a GPU, and fails loudly otherwise.
"""
from .lib import DpgError, load_library, library_path  # noqa: F401
from .disk import (Disk, NVE, DampedNVE, GradDesc, Fire, Adam, minimizeFire, minimizeAdam,  # noqa: F401
                   jamPressure, jamPhi, NEIGH_CELL, NEIGH_VERLET, NEIGH_ALL, FP64, MIXED)
from .bumpy import RigidBumpy  # noqa: F401
from .ensemble import Ensemble  # noqa: F401

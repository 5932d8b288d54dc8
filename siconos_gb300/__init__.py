"""siconos_gb300: GB300-native coloured NSGS for the 3D friction-contact
problem, behind the reference's fc3d_driver / SolverOptions C API.

``numerics`` mirrors the reference's ``siconos.numerics`` Python API for the
GPU solver, ``scene`` builds the seeded lattice workloads, ``device`` exposes
the device-resident API.  All compute runs in ``_lib/libfc3dgpu.so``
(include/fc3dgpu.h)."""
from . import numerics  # noqa: F401

__all__ = ["numerics", "scene", "device", "build"]

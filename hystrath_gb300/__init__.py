"""GB300-native dsmcFoam+ per-timestep particle path (dsmcCloud::evolve on
Cartesian hexahedral meshes): hand-written sm_103a kernels behind a C ABI."""
from . import spec  # noqa: F401

__all__ = ["spec", "dsmc", "build"]

"""GB300 (sm_103a) implementation of crashcat's per-step world update.

The compute path is the CUDA library ``libcrashcat_gpu.so`` (C ABI in
include/crashcat_gpu.h); this package holds its ctypes binding, the host-side
mirror of the reference's world/body/update API and the seeded scene
generators.
"""
from . import _lib, scenes  # noqa: F401
from .world import (  # noqa: F401
    Box, GpuWorld, RigidBodySettings, Sphere, World, WorldSettings, add_broadphase_layer, add_object_layer,
    create_body, create_world, create_world_settings, disable_collision, enable_collision, standard_settings,
    update_world)

__all__ = ["GpuWorld", "World", "WorldSettings", "RigidBodySettings", "Box", "Sphere", "create_world_settings",
           "add_broadphase_layer", "add_object_layer", "enable_collision", "disable_collision", "create_world",
           "create_body", "update_world", "standard_settings", "scenes"]

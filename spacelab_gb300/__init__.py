"""spacelab_gb300 -- SpaceLab's DEM step (all-pairs contact, friction,
cohesion and gravity forces with velocity-Verlet integration) as hand-written
CUDA for GB300 (sm_103a) behind a C ABI shaped like the reference's
Ball_group / sim_one_step.

The native library is required; there is no CPU fallback.
"""
from ._lib import Energy, Material, SpaceLabError  # noqa: F401
from .ball_group import BallGroup, EnergyRow, GpuStep  # noqa: F401

__all__ = ["BallGroup", "EnergyRow", "GpuStep", "Energy", "Material", "SpaceLabError"]

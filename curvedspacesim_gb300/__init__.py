"""GB300-native (sm_103a) implementation of curvedSpaceSim's per-timestep hot path.

The compute path is libcssg.so (CUDA kernels + the C ABI of include/cssg.h); ``api`` wraps it for Python and
``meshes`` generates the synthetic surfaces and initial conditions.
"""
from . import meshes  # noqa: F401

__all__ = ["meshes", "api", "build"]

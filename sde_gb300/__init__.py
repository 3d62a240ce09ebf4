"""sde_gb300 -- GB300 (sm_103a) implementation of SDE's imaging hot path.

libsdegpu (CUDA, built in-tree) implements weighting, gridding, the half-plane FFT with grid
correction, degridding and Hogbom CLEAN behind a C ABI (include/sde_gpu.h) that keeps the
reference's pixel-level calling surface; this package is the Python host layer over it.
"""
from ._abi import SdeError, lib  # noqa: F401

__all__ = ["lib", "SdeError"]

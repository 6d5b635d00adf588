"""meshoid_gb300: GB300 (sm_103a) drop-in for meshoid's particle-neighbourhood path.

``Meshoid`` mirrors the reference class (src/meshoid/Meshoid.py); all numerical
work runs in the CUDA kernels of ``libmeshoid_gb300.so`` through its C ABI
(include/meshoid_gb300.h).
"""
from .meshoid import Meshoid  # noqa: F401

__version__ = "0.1.0"

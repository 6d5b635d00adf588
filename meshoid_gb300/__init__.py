"""meshoid_gb300: GB300 (sm_103a) drop-in for meshoid's particle-neighbourhood path.

``Meshoid`` mirrors the reference class (src/meshoid/Meshoid.py); all numerical
work runs in the CUDA kernels of ``libmeshoid_gb300.so`` through its C ABI
(include/meshoid_gb300.h).  The package exports what the reference's
``meshoid/__init__.py`` star-imports: the class, the grid deposits, the
kernel / smoothing-length functions and the derivative weights.
"""
from .meshoid import Meshoid, set_order2_method, set_order2_refinement  # noqa: F401
from .grid_deposition import *  # noqa: F401,F403
from .kernel_density import *  # noqa: F401,F403
from .derivatives import *  # noqa: F401,F403

__version__ = "0.1.0"

"""CPU oracle for the meshoid hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline arm import
this package.  The product package ``meshoid_gb300`` never does.
"""
from .oracle import *  # noqa: F401,F403

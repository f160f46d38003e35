"""CPU oracle for the bendy2d solver step — test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
reference legs use this package, as the checker.  PARITY UNPINNED: the
reference (Rust) has no tests or golden vectors and cannot be compiled here.
"""
from .oracle import Oracle, load_scene  # noqa: F401

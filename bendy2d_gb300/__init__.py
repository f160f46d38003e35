"""bendy2d-gb300: GB300 (sm_103a) implementation of the bendy2d solver step.

The public surface mirrors the reference crate's (src/lib.rs:1-6):
``Solver``, ``Particle``, ``Link``, ``ParticleLink``, ``CircleLink``,
``Circle``, ``Polygon``, ``Bounds``.  ``Solver.update`` runs on the GPU
through the C ABI in include/bendy2d.h; there is no CPU fallback.
"""
from .api import (COLLIDE_PC, COLLIDE_PP, COLLIDE_PPOLY, MODE_FAST, MODE_REFERENCE, B2DError,
                  Batch, Bounds, Circle, CircleLink, Link, Particle, ParticleLink, Polygon,
                  Solver, line_intersection)

__all__ = ["Solver", "Particle", "Link", "ParticleLink", "CircleLink", "Circle", "Polygon",
           "Bounds", "Batch", "B2DError", "MODE_REFERENCE", "MODE_FAST", "COLLIDE_PP",
           "COLLIDE_PC", "COLLIDE_PPOLY", "line_intersection"]

"""Propagators (propagator.py:8-116).

Paraxial free space (propagator.py:43-76, the default) and direction-cosine
free space (propagator.py:79-116) are fused into the chain kernel rather than
applied as a separate pass.
"""
from __future__ import annotations

from typing import NamedTuple


def _step(ray, distance, propagator):
    """Free space over ``distance`` for every ray: one launch of the chain
    kernel with a single no-op plane at z + distance (the propagator the
    kernel inserts before it is the step)."""
    from .components import Plane
    from .ray import is_uniform
    from .run import run_to_end
    if not is_uniform(ray.z):
        raise NotImplementedError("a propagator call needs one z for all rays")
    # tensors stay tensors, so a requires_grad distance or z gets its gradient
    return run_to_end(ray, [Plane(z=ray.z + distance)], propagator=propagator)


class BasePropagator:
    """propagator.py:8-19."""

    def __call__(self, ray, distance):
        raise NotImplementedError

    def with_distance(self, distance) -> "Propagator":
        return Propagator(distance, self)


class Propagator(NamedTuple):
    """propagator.py:22-40: callable (distance, propagator) pair."""
    distance: float
    propagator: BasePropagator

    def __call__(self, ray):
        return self.propagator(ray, self.distance)


class FreeSpaceParaxial(BasePropagator):
    """x += dx*d, y += dy*d, z += d, pathlength += d (propagator.py:51-72)."""

    def __call__(self, ray, distance):
        return _step(ray, distance, self)

    @staticmethod
    def propagate(ray, distance):
        return FreeSpaceParaxial()(ray, distance)


class FreeSpaceDirCosine(BasePropagator):
    """Direction-cosine propagation (propagator.py:79-116): with
    N = sqrt(1 + dx^2 + dy^2), x += (dx/N)/N * d, y += (dy/N)/N * d,
    z += d, pathlength += d * N; slopes unchanged.  On the GPU it replaces
    the paraxial step inside the fused chain (``run_to_end(...,
    propagator=FreeSpaceDirCosine())``), forward and adjoint."""

    def __call__(self, ray, distance):
        return _step(ray, distance, self)

    @staticmethod
    def propagate(ray, distance):
        return FreeSpaceDirCosine()(ray, distance)

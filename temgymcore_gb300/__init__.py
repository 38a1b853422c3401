"""temgymcore_gb300 - GB300 (sm_103a) implementation of TemGymCore's batched
paraxial ray propagation and Gaussian-beamlet detector field.

Drop-in names follow temgym_core: ``Ray``, the components, ``run_to_end``,
``run_iter``, ``solve_model``, ``Detector.metres_to_pixels`` /
``into_image``, ``GaussianRay`` and ``make_gaussian_image``.  Every hot
operation is a hand-written CUDA kernel in ``csrc/`` reached through the
C ABI in ``include/temgym_gb300.h``; there is no CPU fallback.
"""
from typing import NamedTuple, Union

import numpy as np


class ShapeYX(NamedTuple):
    """Image shape (height, width) in pixels (__init__.py:16-31)."""
    y: int
    x: int


class ScaleYX(NamedTuple):
    """Pixel size (y, x) in metres per pixel (__init__.py:34-49)."""
    y: float
    x: float


class CoordXY(NamedTuple):
    """One (x, y) position in metres (__init__.py:52-69)."""
    x: float
    y: float

    def to_coords(self) -> "CoordsXY":
        return CoordsXY(x=np.array((self.x,)), y=np.array((self.y,)))


class CoordsXY(NamedTuple):
    """Arrays of x, y positions in metres (__init__.py:72-83)."""
    x: object
    y: object


class PixelYX(NamedTuple):
    """One pixel (row, column) (__init__.py:86-107)."""
    y: Union[int, float]
    x: Union[int, float]

    def to_pixels(self) -> "PixelsYX":
        return PixelsYX(x=np.array((self.x,)), y=np.array((self.y,)))


class PixelsYX(NamedTuple):
    """Arrays of pixel rows and columns (__init__.py:110-126)."""
    y: object
    x: object


Degrees = float
Radians = float

from .ray import Ray, GaussianRay  # noqa: E402,F401
from .components import (  # noqa: E402,F401
    Component, Plane, Lens, ScanGrid, Scanner, Descanner, DescanError, Detector, ThickLens,
    Deflector, Rotator, Biprism, Aperture, Source, PointSource, ParallelBeam, Grid,
    AberratedLensKrivanek,
)
from .aberrations import KrivanekCoeffs, W_krivanek, grad_W_krivanek  # noqa: E402,F401
from .transfer import (  # noqa: E402,F401
    transfer_rays, transfer_rays_pt_src, accumulate_matrices, accumulate_matrices_cumulative)
from .propagator import FreeSpaceParaxial, FreeSpaceDirCosine, Propagator, BasePropagator  # noqa: E402,F401
from .run import (  # noqa: E402,F401
    run_to_end, run_iter, solve_model, abcd_matrix, trace_to_image, pack_model, TracePlan,
    run_with_grads, calculate_derivatives, passthrough_transform, jacobian_transform, jacobian_and_value,
)
from .tree_utils import PathBuilder, HasParamsMixin  # noqa: E402,F401
from .scan import scan_images, scan_positions, scan_shard, probe_model  # noqa: E402,F401
from .gaussian import (  # noqa: E402,F401
    make_gaussian_image, evaluate_gaussian_input_image, FieldPlan, fibonacci_spiral, decompose_Q_inv)
from .sources import concentric_rings, random_coords  # noqa: E402,F401
from .batched import BatchedTrace  # noqa: E402,F401
from .fit import StemFit  # noqa: E402,F401

__version__ = "0.1.0"

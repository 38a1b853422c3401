"""Optical components (drop-in for temgym_core.components, components.py:12-559).

Each component is a frozen dataclass with the reference's field names and
defaults.  Calling a component on a Ray runs that single component on the
GPU (one fused launch); ``run_to_end`` fuses a whole model into one launch.
Parameters may be Python floats or 0-d torch tensors (``requires_grad``
tensors receive gradients through the adjoint kernel).
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field
from typing import Any, NamedTuple

import numpy as np
import torch

from . import _native as N
from .coordinate_transforms import metres_to_pixels_transform, pixels_to_metres_transform
from .ray import Ray
from .tree_utils import HasParamsMixin


def _f(v) -> float:
    if isinstance(v, torch.Tensor):
        return float(v.detach().item())
    return float(v)


class Component(HasParamsMixin):
    """Base component: ``__call__(ray) -> Ray`` (components.py:12-24)."""

    z: Any

    def __call__(self, ray: Ray) -> Ray:
        from .run import run_component
        return run_component(self, ray)

    # --- packing for the C ABI -------------------------------------------
    _kind: int = N.PLANE
    _pfields: tuple = ()  # parameter fields in p[] order (differentiable)

    def _params(self) -> list:
        return [_f(getattr(self, n)) for n in self._pfields]

    def _pack(self, comp: N.TgComponent) -> None:
        comp.kind = self._kind
        comp.flags = 0
        comp.z = _f(self.z)
        for i, v in enumerate(self._params()):
            comp.p[i] = v

    def new_with(self, **kw):
        """tree_utils.py:168-172."""
        return dataclasses.replace(self, **kw)


class Source(Component):
    """Source (source.py:11-79): a no-op as a model element (run_iter inserts
    free space before it like any component) that also generates its initial
    rays on the GPU."""

    def generate_array(self, num: int, random: bool = False, seed: int = 0) -> torch.Tensor:
        """(N, 5) float64 device rays [x, y, dx, dy, 1] (source.py:36-57)."""
        raise NotImplementedError

    def make_rays(self, num: int, random: bool = False, seed: int = 0) -> Ray:
        """Ray of the generated array at the source's z (source.py:59-79);
        scalar fields when only one ray is generated."""
        r = self.generate_array(num, random=random, seed=seed)
        sl = 0 if r.shape[0] == 1 else slice(None)
        return Ray(x=r[sl, 0], y=r[sl, 1], dx=r[sl, 2], dy=r[sl, 3], z=self.z, pathlength=0.0)


@dataclass(frozen=True)
class PointSource(Source):
    """source.py:82-135: rays from a point at ``offset_xy`` with slopes filling
    a cone of ``semi_conv`` (concentric rings, or uniform random)."""
    z: Any
    semi_conv: Any = 0.0
    offset_xy: Any = (0.0, 0.0)

    def generate_array(self, num: int, random: bool = False, seed: int = 0) -> torch.Tensor:
        from .sources import POINT, generate
        return generate(POINT, num, _f(self.semi_conv), self.offset_xy, random, seed)


@dataclass(frozen=True)
class ParallelBeam(Source):
    """source.py:138-188: parallel rays filling a disc of ``radius`` around
    ``offset_xy``."""
    z: Any
    radius: Any = 0.0
    offset_xy: Any = (0.0, 0.0)

    def generate_array(self, num: int, random: bool = False, seed: int = 0) -> torch.Tensor:
        from .sources import PARALLEL, generate
        return generate(PARALLEL, num, _f(self.radius), self.offset_xy, random, seed)


class DescanError(NamedTuple):
    """Linear descan error coefficients (components.py:27-115).

    The twelve reference fields describe how position / slope offsets depend
    on scan POSITION plus constant offsets.  The eight ``*_sxi / *_syi``
    fields (default 0, i.e. the reference's behaviour) extend the model with
    a dependence on scan TILT, giving the full 4x4 descan matrix.
    """
    pxo_pxi: Any = 0.0
    pxo_pyi: Any = 0.0
    pyo_pxi: Any = 0.0
    pyo_pyi: Any = 0.0
    sxo_pxi: Any = 0.0
    sxo_pyi: Any = 0.0
    syo_pxi: Any = 0.0
    syo_pyi: Any = 0.0
    offpxi: Any = 0.0
    offpyi: Any = 0.0
    offsxi: Any = 0.0
    offsyi: Any = 0.0
    pxo_sxi: Any = 0.0
    pxo_syi: Any = 0.0
    pyo_sxi: Any = 0.0
    pyo_syi: Any = 0.0
    sxo_sxi: Any = 0.0
    sxo_syi: Any = 0.0
    syo_sxi: Any = 0.0
    syo_syi: Any = 0.0

    def as_array(self) -> np.ndarray:
        return np.array([_f(v) for v in self[:12]])

    def as_matrix(self) -> np.ndarray:
        """components.py:93-115: the reference's 5x5 with the offsets in the
        last column, entry for entry - including its dx row, which holds offsyi
        where offsxi belongs (that matrix is informational: the descanner
        applies offsets() = offpxi, offpyi, offsxi, offsyi)."""
        v = [_f(a) for a in self[:12]]
        return np.array([[v[0], v[1], 0.0, 0.0, v[8]],
                         [v[2], v[3], 0.0, 0.0, v[9]],
                         [v[4], v[5], 0.0, 0.0, v[11]],
                         [v[6], v[7], 0.0, 0.0, v[11]],
                         [0.0, 0.0, 0.0, 0.0, 1.0]])

    def as_matrix4(self) -> np.ndarray:
        """4x4 matrix: rows (x, y, dx, dy) out, cols (spx, spy, stx, sty) in."""
        v = [_f(a) for a in self]
        return np.array([[v[0], v[1], v[12], v[13]], [v[2], v[3], v[14], v[15]],
                         [v[4], v[5], v[16], v[17]], [v[6], v[7], v[18], v[19]]])

    @classmethod
    def from_matrix4(cls, m, offsets=(0.0, 0.0, 0.0, 0.0)):
        m = np.asarray(m, dtype=np.float64)
        return cls(m[0, 0], m[0, 1], m[1, 0], m[1, 1], m[2, 0], m[2, 1], m[3, 0], m[3, 1],
                   *offsets, m[0, 2], m[0, 3], m[1, 2], m[1, 3], m[2, 2], m[2, 3],
                   m[3, 2], m[3, 3])

    def offsets(self):
        return [_f(v) for v in self[8:12]]


# ----------------------------------------------------------------- grids

class Grid:
    """Pixel geometry mixin (grid.py:12-280).  ``pixel_size`` and ``shape`` are
    (y, x); ``centre`` is (x, y) metres; ``rotation`` in degrees."""

    @property
    def pixels_to_metres_mat(self) -> np.ndarray:
        return pixels_to_metres_transform(self.centre, self.pixel_size, self.shape,
                                          self.flip_y, _f(self.rotation))

    @property
    def metres_to_pixels_mat(self) -> np.ndarray:
        return metres_to_pixels_transform(self.centre, self.pixel_size, self.shape,
                                          self.flip_y, _f(self.rotation))

    def _tg_grid(self) -> N.TgGrid:
        # grids are frozen dataclasses: the C struct is built once per instance
        # (tensor-valued fields are read each time: they may change in place)
        cached = self.__dict__.get("_tg_grid_cache")
        if cached is not None:
            return cached
        m = self.metres_to_pixels_mat
        g = N.TgGrid()
        g.h, g.w = int(self.shape[0]), int(self.shape[1])
        for i, v in enumerate((m[0, 0], m[0, 1], m[0, 2], m[1, 0], m[1, 1], m[1, 2])):
            g.m[i] = float(v)
        fields = (self.pixel_size, self.shape, self.rotation, self.centre)
        if not any(isinstance(f, torch.Tensor) for f in fields):
            object.__setattr__(self, "_tg_grid_cache", g)
        return g

    @property
    def coords_px(self):
        """grid.py:66-80."""
        h, w = self.shape
        return np.meshgrid(np.arange(h), np.arange(w), indexing="ij")

    @property
    def coords(self) -> np.ndarray:
        """grid.py:83-100: (H*W, 2) pixel-centre (x, y), row-major."""
        yy, xx = self.coords_px
        x, y = self.pixels_to_metres((yy.ravel(), xx.ravel()))
        return np.stack((np.asarray(x), np.asarray(y)), axis=-1).reshape(-1, 2)

    @property
    def coords_1d(self):
        """grid.py:103-118."""
        yy, xx = self.coords_px
        xc = self.pixels_to_metres((yy[0, :], xx[0, :]))[0]
        yc = self.pixels_to_metres((yy[:, 0], xx[:, 0]))[1]
        return xc, yc

    def metres_to_pixels(self, coords, cast: bool = True):
        """grid.py:120-153.  cast=True runs the bit-exact GPU binner and returns
        int32 (py, px) tensors; cast=False returns float64 fractional pixels."""
        from .run import bin_pixels
        cx, cy = coords
        if cast:
            return bin_pixels(self, cx, cy)
        m = self.metres_to_pixels_mat
        tx = torch.as_tensor(cx, dtype=torch.float64)
        ty = torch.as_tensor(cy, dtype=torch.float64)
        return ((m[0, 0] * ty + m[0, 1] * tx) + m[0, 2], (m[1, 0] * ty + m[1, 1] * tx) + m[1, 2])

    def pixels_to_metres(self, pixels):
        """grid.py:155-182: returns (x, y) metres (float64, host set-up math)."""
        py, px = pixels
        t = self.pixels_to_metres_mat
        py = np.asarray(py, dtype=np.float64)
        px = np.asarray(px, dtype=np.float64)
        my = (t[0, 0] * py + t[0, 1] * px) + t[0, 2]
        mx = (t[1, 0] * py + t[1, 1] * px) + t[1, 2]
        return mx, my

    def ray_at_grid(self, px_y, px_x, dx=0.0, dy=0.0, z=None):
        """grid.py:184-212."""
        x, y = self.pixels_to_metres((px_y, px_x))
        return Ray(x=x, y=y, dx=dx, dy=dy, z=self.z if z is None else z, pathlength=0.0)

    def ray_to_grid(self, ray: Ray, cast: bool = False):
        """grid.py:214-229."""
        return self.metres_to_pixels((ray.x, ray.y), cast=cast)

    def into_image(self, ray, acc: torch.Tensor | None = None):
        """grid.py:231-280: histogram of ray hits (out-of-bounds dropped).
        ``acc`` (int64 by default, like the reference's ``dtype=int``; int32
        accepted) is updated in place on the GPU and returned."""
        from .run import image_from
        return image_from(self, ray, acc)


@dataclass(frozen=True)
class Plane(Component):
    """No-op at z (components.py:118-134)."""
    z: Any


@dataclass(frozen=True)
class Lens(Component):
    """Thin lens (components.py:137-174): dx -= x/f, dy -= y/f,
    pathlength -= (x^2 + y^2)/(2f)."""
    z: Any
    focal_length: Any
    _kind = N.LENS
    _pfields = ("focal_length",)


@dataclass(frozen=True)
class AberratedLensKrivanek(Lens):
    """Thin lens with Krivanek aberrations (components.py:177-215): ideal
    thin-lens slopes u, then slopes u - grad W(u)/f and pathlength
    - (x^2 + y^2)/(2f) + W(u)/f.  ``coeffs``: KrivanekCoeffs (or a dict of
    its fields).  Runs in the forward chain kernels (run_to_end, 4D-STEM
    scans), the beamlet-field preparation and the trace adjoint (gradients
    with respect to the rays and the focal length); the batched sweep and the
    beamlet-field adjoint reject it."""
    coeffs: Any = None
    _kind = N.ABERLENS
    _pfields = ("focal_length",)

    def _params(self) -> list:
        from .aberrations import KrivanekCoeffs, as_coeffs
        c = KrivanekCoeffs() if self.coeffs is None else as_coeffs(self.coeffs)
        return [_f(self.focal_length)] + c.as_list()


@dataclass(frozen=True)
class ScanGrid(Component, Grid):
    """Scan grid geometry at z (components.py:218-249); a no-op on rays."""
    z: Any
    pixel_size: Any
    shape: Any
    rotation: Any = 0.0
    centre: Any = (0.0, 0.0)
    flip_y: bool = False


@dataclass(frozen=True)
class Scanner(Component):
    """Adds scan position/tilt (components.py:252-285)."""
    z: Any
    scan_pos_x: Any
    scan_pos_y: Any
    scan_tilt_x: Any = 0.0
    scan_tilt_y: Any = 0.0
    _kind = N.SCANNER
    _pfields = ("scan_pos_x", "scan_pos_y", "scan_tilt_x", "scan_tilt_y")


@dataclass(frozen=True)
class Descanner(Component):
    """Linear descan with error (components.py:288-372):
    delta = M @ (spx, spy, stx, sty) + offsets - (spx, spy, stx, sty)."""
    z: Any
    scan_pos_x: Any
    scan_pos_y: Any
    scan_tilt_x: Any = 0.0
    scan_tilt_y: Any = 0.0
    descan_error: DescanError = field(default_factory=DescanError)
    _kind = N.DESCANNER

    def _params(self) -> list:
        m = self.descan_error.as_matrix4()
        return ([_f(self.scan_pos_x), _f(self.scan_pos_y), _f(self.scan_tilt_x),
                 _f(self.scan_tilt_y)] + list(m.reshape(-1)) + self.descan_error.offsets())


@dataclass(frozen=True)
class Detector(Component, Grid):
    """Detector grid at z (components.py:375-406); a no-op on rays."""
    z: Any
    pixel_size: Any
    shape: Any
    rotation: Any = 0.0
    centre: Any = (0.0, 0.0)
    flip_y: bool = False


@dataclass(frozen=True)
class ThickLens(Component):
    """Thick lens (components.py:409-452): thin-lens update, z -> z - (z_po - z_pi)."""
    z_po: Any
    z_pi: Any
    focal_length: Any
    _kind = N.THICKLENS

    @property
    def z(self):
        return self.z_po

    def _params(self) -> list:
        return [_f(self.focal_length), _f(self.z_pi)]


@dataclass(frozen=True)
class Deflector(Component):
    """Constant deflection (components.py:455-482); pathlength += dx*x + dy*y
    with the incoming slopes."""
    z: Any
    def_x: Any
    def_y: Any
    _kind = N.DEFLECTOR
    _pfields = ("def_x", "def_y")


@dataclass(frozen=True)
class Rotator(Component):
    """Rotation of positions and slopes by ``angle`` degrees (components.py:485-523)."""
    z: Any
    angle: Any
    _kind = N.ROTATOR
    _pfields = ("angle",)


@dataclass(frozen=True)
class Biprism(Component):
    """Biprism (components.py:526-559): dx += def_x*sign(x); pathlength +=
    dx*x + dy*y.  ``offset``, ``rotation`` and ``side`` are stored but unused,
    as in the reference."""
    z: Any
    offset: Any = 0.0
    rotation: Any = 0.0
    def_x: Any = 0.0
    side: int = 1
    _kind = N.BIPRISM
    _pfields = ("def_x",)


@dataclass(frozen=True)
class Aperture(Component):
    """Circular aperture (this package's extension; the reference has none):
    rays with (x-cx)^2 + (y-cy)^2 >= radius^2 are blocked - their amplitude
    becomes 0 and histograms skip them; their coordinates still propagate."""
    z: Any
    radius: Any
    centre: Any = (0.0, 0.0)
    _kind = N.APERTURE

    def _params(self) -> list:
        return [_f(self.radius), _f(self.centre[0]), _f(self.centre[1])]


SUPPORTED = (Plane, Lens, ScanGrid, Scanner, Descanner, Detector, ThickLens, Deflector,
             Rotator, Biprism, Aperture, Source)
